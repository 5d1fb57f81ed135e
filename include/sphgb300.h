/*
 * sphgb300 -- GB300-native (sm_103a) DFSPH time step behind a C ABI.
 *
 * One context holds one fluid model (one fluid phase) with static Akinci2012
 * boundary particles, device-resident for the life of the context.  Every call
 * returns an int status (SPHGB_OK = 0); no C++ exception crosses the ABI and no
 * kernel traps.  A context is driven by one host thread and owns one CUDA
 * stream.  Arrays are plain host pointers, AoS Vector3 layout (x0,y0,z0,x1,...)
 * exactly like the reference's std::vector<Vector3r> storage.
 *
 * Reference interfaces replaced (SPlisHSPlasH 2.16.0, paths relative to the
 * project root):
 *   sphgb_step            TimeStepDFSPH::step           SPlisHSPlasH/DFSPH/TimeStepDFSPH.cpp:117-249
 *                         (neighbour search Simulation.cpp:606-619, densities TimeStep.cpp:54-169,
 *                          DFSPH factor :735-825, divergence solve :386-541, non-pressure forces
 *                          Simulation.cpp:495-509 with XSPH XSPH.cpp:46-216 and Weiler2018
 *                          Viscosity/Viscosity_Weiler2018.cpp:891-1089, CFL Simulation.cpp:395-493,
 *                          pressure solve TimeStepDFSPH.cpp:252-384)
 *   sphgb_upload_fluid    FluidModel::initModel          SPlisHSPlasH/FluidModel.cpp:285-327
 *   sphgb_upload_boundary BoundaryModel_Akinci2012::initModel + computeBoundaryVolume
 *                                                        SPlisHSPlasH/BoundaryModel_Akinci2012.cpp:48-110,
 *                                                        Simulation::updateBoundaryVolume Simulation.cpp:696-756
 *   sphgb_download /      FluidModel::getFieldBuffer     pySPlisHSPlasH/FluidModelModule.cpp:86-118,
 *   sphgb_upload_field    field registry                 FluidModel.cpp:694-710, TimeStepDFSPH.cpp:49-53,
 *                                                        Viscosity_Weiler2018.cpp:33
 *   sphgb_neighbors       Simulation::getNeighborList    SPlisHSPlasH/Simulation.h:451-473
 *   sphgb_set_params      ParameterObject set/getValue   TimeStepDFSPH.cpp:73-115, Simulation.cpp:163-277,
 *                                                        XSPH.cpp:27-42, Viscosity_Weiler2018.cpp:43-74
 */
#ifndef SPHGB300_H
#define SPHGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHGB_ABI_VERSION 1

/* status codes */
#define SPHGB_OK 0
#define SPHGB_ERR_ARGUMENT 1      /* bad pointer / size / enum */
#define SPHGB_ERR_CUDA 2          /* a CUDA runtime call failed (message in sphgb_last_error) */
#define SPHGB_ERR_CAPACITY 3      /* neighbour-list or particle capacity exceeded */
#define SPHGB_ERR_NONFINITE 4     /* NaN/Inf velocity detected during the step */
#define SPHGB_ERR_STATE 5         /* call out of order (e.g. step before upload) */
#define SPHGB_ERR_GRID 6          /* scene extent too large for the cell grid */

/* precision of the bulk arithmetic */
#define SPHGB_PRECISION_FP32 0    /* FP32 neighbour sums; FP64 reductions, dt, time and positions */
#define SPHGB_PRECISION_FP64 1    /* everything in FP64 */

typedef struct sphgb_config {
    int abi_version;                 /* must be SPHGB_ABI_VERSION */
    int device;                      /* CUDA device ordinal */
    int precision;                   /* SPHGB_PRECISION_* */
    uint32_t max_fluid_neighbors;    /* per-particle list capacity (0 = default 80; rounded up to a multiple of 4) */
    uint32_t max_boundary_neighbors; /* per-particle list capacity (0 = default 128) */
    int use_graph;                   /* 1: capture the step in a CUDA graph with device-side
                                        solver loops (conditional while nodes); 0: host-driven loops */
} sphgb_config;

typedef struct sphgb_params {
    double particle_radius;          /* Simulation "particleRadius"; support radius = 4 r */
    double density0;                 /* FluidModel "density0" */
    double gravity[3];               /* Simulation "gravitation" */
    int cfl_method;                  /* "cflMethod": 0 none, 1 CFL, 2 CFL + iteration heuristic */
    double cfl_factor;               /* "cflFactor" */
    double cfl_min_time_step;        /* "cflMinTimeStepSize" */
    double cfl_max_time_step;        /* "cflMaxTimeStepSize" */
    uint32_t min_iterations;         /* DFSPH "minIterations" */
    uint32_t max_iterations;         /* DFSPH "maxIterations" */
    double max_error;                /* DFSPH "maxError" (percent) */
    int enable_divergence_solver;    /* DFSPH "enableDivergenceSolver" */
    uint32_t max_iterations_v;       /* DFSPH "maxIterationsV" */
    double max_error_v;              /* DFSPH "maxErrorV" (percent) */
    double xsph;                     /* XSPH "xsph" */
    double xsph_boundary;            /* XSPH "xsphBoundary" */
    int viscosity_method;            /* 0 none, 6 "Weiler et al. 2018" */
    double viscosity;                /* Weiler "viscosity" */
    double viscosity_boundary;       /* Weiler "viscosityBoundary" */
    uint32_t visco_max_iter;         /* Weiler "viscoMaxIter" */
    double visco_max_error;          /* Weiler "viscoMaxError" */
} sphgb_params;

typedef struct sphgb_stats {
    uint32_t iterations;             /* DFSPH "iterations" (pressure solve) */
    uint32_t iterations_v;           /* DFSPH "iterationsV" (divergence solve) */
    uint32_t visco_iterations;       /* Weiler "viscoIterations" (Eigen CG iteration count) */
    uint32_t max_fluid_neighbors;    /* largest fluid neighbour count seen this step */
    uint32_t max_boundary_neighbors; /* largest boundary neighbour count seen this step */
    uint32_t flags;                  /* bit 0 capacity overflow, bit 1 non-finite */
    double avg_density_err;          /* last pressure-solve average density error (FP64) */
    double avg_density_err_v;        /* last divergence-solve average error (FP64) */
    double visco_error;              /* CG relative residual */
    double dt_used;                  /* step size used for the kick and the position update */
    double dt_next;                  /* CFL step size (used by the pressure solve) */
    double time;                     /* simulated time after the step */
    uint64_t kernel_launches;        /* kernels this step launched on the GPU */
    uint32_t learned_used;           /* bit 0 / bit 1: predicted warm start used by the divergence /
                                        pressure solve this step */
    uint32_t reserved;
    double ws_residual_classic[2];   /* average error of the classic warm start after the gate iterations
                                        (div, pressure; with a gate of 1: the initial residual) */
    double ws_residual_learned[2];   /* ... of the predicted warm start (0 when the network is off) */
} sphgb_stats;

/* field ids for sphgb_download / sphgb_upload_field; names are the reference's field names */
#define SPHGB_FIELD_POSITION 0        /* "position", 3 */
#define SPHGB_FIELD_VELOCITY 1        /* "velocity", 3 */
#define SPHGB_FIELD_ACCELERATION 2    /* "acceleration" (non-pressure), 3 */
#define SPHGB_FIELD_DENSITY 3         /* "density" */
#define SPHGB_FIELD_FACTOR 4          /* "factor" as stored after step(): alpha / dt_next^2 */
#define SPHGB_FIELD_DENSITY_ADV 5     /* "advected density" */
#define SPHGB_FIELD_PRESSURE_RHO2 6   /* "p / rho^2" (kappa, stored * dt^2) */
#define SPHGB_FIELD_PRESSURE_RHO2_V 7 /* "p_v / rho^2" (kappa_v, stored * dt) */
#define SPHGB_FIELD_PRESSURE_ACCEL 8  /* "pressure acceleration", 3 */
#define SPHGB_FIELD_VDIFF 9           /* Weiler "velocity difference", 3 */
#define SPHGB_FIELD_PARTICLE_ID 10    /* "id" (uint32) */
#define SPHGB_FIELD_FACTOR_RAW 11     /* alpha as computed by computeDFSPHFactor */
#define SPHGB_FIELD_NUM_FLUID_NEIGHBORS 12     /* uint32 */
#define SPHGB_FIELD_NUM_BOUNDARY_NEIGHBORS 13  /* uint32 */
#define SPHGB_FIELD_BOUNDARY_VOLUME 14         /* boundary "volume" V_b (nb entries) */
#define SPHGB_FIELD_BOUNDARY_POSITION 15       /* boundary "position" (nb x 3) */
#define SPHGB_FIELD_FEATURES 16                /* warm-start network inputs of the last step (n x 10) */
#define SPHGB_FIELD_POSITION_HI 17             /* position as stored: the high part of the FP32 double-float
                                                  position (FP64 mode: the position), 3 */
#define SPHGB_FIELD_STATE 19                   /* FluidModel "state" (ParticleState, FluidModel.cpp:62), uint32:
                                                  0 = Active for every particle the device steps */
#define SPHGB_FIELD_OBJECT_ID 20               /* FluidModel "object_id" (FluidModel.cpp:63), uint32: 0 (the
                                                  device keeps no object ids) */
#define SPHGB_FIELD_POSITION_LO 18             /* the low part of the FP32 double-float position (FP64 mode:
                                                  zero); HI + LO = "position" exactly, 3 */

#define SPHGB_DTYPE_F32 0
#define SPHGB_DTYPE_F64 1
#define SPHGB_DTYPE_U32 2

typedef struct sphgb_ctx sphgb_ctx;

/* lifetime */
int sphgb_create(const sphgb_config *cfg, sphgb_ctx **out);
int sphgb_destroy(sphgb_ctx *ctx);
const char *sphgb_last_error(const sphgb_ctx *ctx);
int sphgb_abi_version(void);

/* parameters (may be called between steps) */
int sphgb_default_params(sphgb_params *p);
int sphgb_set_params(sphgb_ctx *ctx, const sphgb_params *p);
int sphgb_get_params(const sphgb_ctx *ctx, sphgb_params *p);

/* scene set-up.  Positions/velocities AoS n x 3; ids may be NULL (0..n-1).
 * upload_boundary computes the Akinci2012 volumes on the device. */
int sphgb_upload_boundary(sphgb_ctx *ctx, const double *xb, uint32_t nb);
int sphgb_upload_boundary_f32(sphgb_ctx *ctx, const float *xb, uint32_t nb);
int sphgb_upload_fluid(sphgb_ctx *ctx, const double *x, const double *v, const uint32_t *id, uint32_t n);
int sphgb_upload_fluid_f32(sphgb_ctx *ctx, const float *x, const float *v, const uint32_t *id, uint32_t n);

/* time step size (TimeManager::get/setTimeStepSize) and time */
int sphgb_set_time_step(sphgb_ctx *ctx, double dt);
int sphgb_get_time_step(const sphgb_ctx *ctx, double *dt);
int sphgb_set_time(sphgb_ctx *ctx, double t);

/* one TimeStepDFSPH::step(); stats may be NULL (then the call does not wait for the GPU).
 * SPHGB_ERR_STATE before an upload or for a fluid model without particles; SPHGB_ERR_GRID when a
 * scene spans more than 1024 cells of 4.004 r per axis; SPHGB_ERR_CAPACITY when a neighbour list
 * overflowed (the step's results are then incomplete); SPHGB_ERR_NONFINITE for a non-finite
 * velocity. */
int sphgb_step(sphgb_ctx *ctx, sphgb_stats *stats);
/* blocks until the last step finished and fills stats */
int sphgb_sync(sphgb_ctx *ctx, sphgb_stats *stats);

/* field transfer in particle-id order (the host std::vector order); count = n (or nb for the
 * boundary fields) x components */
int sphgb_download(sphgb_ctx *ctx, int field, void *dst, int dtype);
int sphgb_upload_field(sphgb_ctx *ctx, int field, const void *src, int dtype);
/* several fields in one call (no counterpart in the reference, whose host vectors are read
 * field by field): the same fields, layouts and checks as above, dsts[k] / srcs[k] for
 * fields[k], all in one dtype; the transfers are queued back to back on the context's stream
 * and the call waits once.  Uploads compute the slot of each particle id once for all fields.
 * A fluid field whose buffer is page-locked host memory mapped into the device's address space
 * (cudaHostAlloc, cudaHostRegister) or memory of the context's device is read or written by the
 * device itself, in particle-id order, with no staging copy; other buffers are staged in device
 * memory and copied.  The transfers run on the context's stream: a device buffer written on
 * another stream must be complete before the call. */
int sphgb_download_fields(sphgb_ctx *ctx, uint32_t count, const int *fields, void *const *dsts, int dtype);
int sphgb_upload_fields(sphgb_ctx *ctx, uint32_t count, const int *fields, const void *const *srcs, int dtype);

/* neighbour lists of the last step in particle-id order, CSR: offsets[n+1], indices are particle
 * ids.  kind 0 = fluid-fluid, 1 = fluid-boundary (boundary indices in upload order).  Pass
 * indices == NULL to query offsets only. */
int sphgb_neighbors(sphgb_ctx *ctx, int kind, uint32_t *offsets, uint32_t *indices, size_t capacity);

/* ---- particle export and state files (the reference's exporters and state files,
 * Simulator/Exporter/ParticleExporter_VTK.cpp:25-266, SimulatorBase.cpp:1689-1870, run from
 * the device copy) ----
 * sphgb_export_vtk writes one legacy VTK 4.1 file (big-endian binary, unstructured grid of
 * vertex cells) of all fluid particles in particle-id order, like ParticleExporter_VTK:
 * POINTS (position), CELLS / CELL_TYPES, POINT_DATA "id", then a FIELD block with one array per
 * entry of `fields` (field ids above, names with white space replaced by '_').  The device
 * scatters and byte-swaps the data on its own stream and copies it to pinned host memory
 * asynchronously; a host thread writes the file.  wait = 0 returns at once (the next steps
 * overlap the copy and the write); sphgb_export_wait blocks until the last export is on disk
 * and returns its status.  A new export or sphgb_destroy waits for the previous one. */
int sphgb_export_vtk(sphgb_ctx *ctx, const char *path, const int *fields, uint32_t nfields, int wait);
int sphgb_export_wait(sphgb_ctx *ctx);
/* sphgb_export_bgeo writes one partio BGEO file of all fluid particles in particle-id order, as
 * ParticleExporter_Partio::writeParticlesPartio does through partio
 * (Simulator/Exporter/ParticleExporter_Partio.cpp:67-201): the attribute "position" (float x 3,
 * stored with w = 1), "id" (INT), then one attribute per entry of `fields` under its field name
 * (scalar fields FLOAT, uint fields INT, 3-vectors VECTOR; other fields SPHGB_ERR_ARGUMENT).
 * Values are stored as 32-bit floats in both precisions, as the reference casts them.  level:
 * -1 (zlib's default, partio's choice) or 1-9 writes the file as one gzip member, as the
 * reference's Partio::write(..., true) does, compressed on all host cores but one; 0 writes it plain.
 * The device packs the big-endian records on the export stream and copies them to pinned
 * memory; wait and sphgb_export_wait as for sphgb_export_vtk.  SPHGB_ERR_STATE when zlib
 * (libz.so.1) cannot be loaded for a compressed file. */
int sphgb_export_bgeo(sphgb_ctx *ctx, const char *path, const int *fields, uint32_t nfields, int level, int wait);
/* the field id of a fluid field name as the reference's FieldDescription names it ("velocity",
 * "p / rho^2", ...; FluidModel.cpp:61-67, TimeStepDFSPH.cpp:49-53), for exporters that take the
 * names of SimulatorBase's particleAttributes; -1 for an unknown name */
int sphgb_field_id(const char *name);
/* The simulation state of the context in a binary file, exactly as held on the device (the
 * double-float positions in both parts, velocities, velocity differences, both warm starts,
 * per-scene step size and time, the boundary particles, the parameters and the lanes per
 * particle in use): sphgb_load_state re-creates the scenes from it, and stepping continues bit
 * for bit as if the context had not been interrupted. */
int sphgb_save_state(sphgb_ctx *ctx, const char *path);
int sphgb_load_state(sphgb_ctx *ctx, const char *path);
/* The particle file of the reference's state (SimulatorBase::writeFluidParticlesState,
 * Simulator/SimulatorBase.cpp:2062-2127, called per fluid model by saveState :1689-1770): a
 * partio BGEO file holding the fluid model's fields that the reference marks storeData, under
 * their names, in particle-id order: "id", "state", "object_id", "position", "velocity",
 * "p / rho^2", "p_v / rho^2" and, with Weiler2018 viscosity, "velocity difference"
 * (FluidModel.cpp:61-66, TimeStepDFSPH.cpp:51-52, Viscosity_Weiler2018.cpp:33); values as 32-bit
 * floats and ints, as the reference stores them.  level as for sphgb_export_bgeo (the reference
 * writes it compressed).  The time and step size of the state are sphgb_get_time_step and the
 * last step's time; the simulator-level part of the reference's .bin state file stays the
 * simulator's.  One fluid model, one scene. */
int sphgb_save_particle_state(sphgb_ctx *ctx, const char *path, int level);
/* Reads such a file (SimulatorBase::readFluidParticlesState, :2130-2192), plain or compressed:
 * every attribute named like a field of this path -- "position", "velocity", "p / rho^2",
 * "p_v / rho^2", "velocity difference" -- is set for the particle whose "id" the record carries
 * (record order when there is no "id").  The file must hold as many points as the context has
 * fluid particles, and a "state" attribute must mark every particle Active (0).  The boundary,
 * the parameters and the step size stay as they are. */
int sphgb_load_particle_state(sphgb_ctx *ctx, const char *path);

/* counts (all scenes of a batch) */
int sphgb_num_particles(const sphgb_ctx *ctx, uint32_t *n, uint32_t *nb);

/* ---- batched scenes (no counterpart in the reference: it simulates one scene per process,
 * Simulation::getCurrent at Simulation.cpp:112-119) ----
 * Replaces the fluid and the boundary of the context with nscenes independent scenes that
 * advance together: every kernel launch of a step covers all scenes, each scene keeps its own
 * cell grid, CFL step size, solver iteration counts and convergence decisions (a scene whose
 * solver converged idles while the others iterate), and with use_graph = 1 a step of the whole
 * batch is one graph launch.  n[s] >= 1 fluid and nb[s] >= 0 boundary particles per scene;
 * x and v hold the scenes' fluid particles concatenated in scene order (sum(n) x 3), xb the
 * boundary particles (sum(nb) x 3).  Particle ids (the download order of every field) are this
 * concatenated order.  Parameters (sphgb_set_params) and the network are shared by all scenes;
 * sphgb_set_time_step / sphgb_set_time set every scene.  sphgb_step's stats for a batch: scene
 * 0's times, the maxima over the scenes of iteration counts and errors, the OR of the flags.
 * sphgb_upload_fluid / sphgb_upload_boundary switch the context back to one scene. */
int sphgb_upload_scenes(sphgb_ctx *ctx, uint32_t nscenes, const uint32_t *n, const uint32_t *nb, const double *x,
                        const double *v, const double *xb);
int sphgb_num_scenes(const sphgb_ctx *ctx, uint32_t *nscenes);
/* statistics of scenes first .. first+count-1 of the last step (waits for it) */
int sphgb_scene_stats(sphgb_ctx *ctx, uint32_t first, uint32_t count, sphgb_stats *out);

/* ---- learned warm start (no counterpart in the reference: new in this library) ----
 * A per-particle network 10 -> 64 -> 64 -> 2 (GELU), BF16 weights and activations on the
 * tensor cores with FP32 accumulation.  Its two outputs (times the output scales) are the
 * multipliers that the divergence and the pressure warm start apply to the previous step's
 * stored kappa_v and kappa, in place of the classic factor 0.5 (TimeStepDFSPH.cpp:449-453,
 * :293-296; classic clamps and masks kept, multiplier limited to [0, 4]).  Inputs: 5
 * dimensionless per-particle features (density deviation, velocity divergence x dt, neighbour
 * count, previous kappa relative to its neighbourhood, |v| dt / 2r) and the cubic-spline-
 * weighted neighbour means of the features (sphgb_download SPHGB_FIELD_FEATURES).  Trained
 * with Adam by hand-written kernels; the loss is the mean over samples of
 * sum_o mask_o (y_o - t_o)^2 (mask = per-output weight).  Host arrays: X n x 10,
 * targets/mask n x 2, row-major float. */
typedef struct sphgb_mlp sphgb_mlp;
int sphgb_mlp_create(int device, uint32_t seed, sphgb_mlp **out);
int sphgb_mlp_destroy(sphgb_mlp *m);
const char *sphgb_mlp_last_error(const sphgb_mlp *m);
int sphgb_mlp_num_params(void);
int sphgb_mlp_get_params(sphgb_mlp *m, float *out);
int sphgb_mlp_set_params(sphgb_mlp *m, const float *in);
/* network output o_k x scale_k = warm-start multiplier (k = 0 divergence, 1 pressure); default 1 */
int sphgb_mlp_set_output_scale(sphgb_mlp *m, float scale_v, float scale_p);
int sphgb_mlp_get_output_scale(const sphgb_mlp *m, float *scale_v, float *scale_p);
int sphgb_mlp_forward(sphgb_mlp *m, const float *X, uint32_t n, float *Y);
int sphgb_mlp_loss_grad(sphgb_mlp *m, const float *X, const float *Y, const float *mask, uint32_t n, float *loss,
                        float *grad);
int sphgb_mlp_train(sphgb_mlp *m, const float *X, const float *Y, const float *mask, uint32_t n, uint32_t epochs,
                    uint32_t batch, float lr, uint32_t seed, float *epoch_loss);
/* Use the network for both warm starts of this context (NULL: classic warm start only).  The
 * solvers still iterate to their tolerances; per step, scene and solver the first Jacobi
 * iterations (sphgb_set_warmstart_gate) run for both candidates and the predicted warm start
 * is kept only if its error after them is lower than the classic one's (sphgb_stats
 * learned_used; ws_residual_* hold both errors). */
int sphgb_set_warmstart_mlp(sphgb_ctx *ctx, const sphgb_mlp *m);
/* The gate of the learned warm start, per solver: both candidates (classic and predicted) run
 * this many Jacobi iterations, then the one with the lower average error continues (the
 * loser's iterations are not booked; a solver that converges during the gate still books the
 * gate's iterations).  1 compares the candidates' initial residuals.  0 (default): 1 for the
 * divergence solve and max(minIterations, 4) for the pressure solve, because a warm start's
 * particle-scale error dominates the first residuals but decays within a few sweeps, while
 * the low-frequency error that decides the iteration count does not. */
int sphgb_set_warmstart_gate(sphgb_ctx *ctx, uint32_t div_sweeps, uint32_t pressure_sweeps);
/* compute the network inputs every step even without a network (training-data collection);
 * they are read back with SPHGB_FIELD_FEATURES */
int sphgb_set_feature_output(sphgb_ctx *ctx, int on);

/* Akinci2012 boundary volumes that allocate nothing (no reference counterpart: the
 * reference computes volumes on the host in BoundaryModel_Akinci2012::computeBoundaryVolume).
 * For callers that may not allocate device memory: code running during CUDA stream capture,
 * where cudaMalloc cannot be recorded, and hosts with a fixed device-memory budget that forbid
 * allocation after start-up.  xb (nb x 3 floats, AoS) and volume (nb floats) are DEVICE
 * pointers owned by the caller; stream is a cudaStream_t (NULL = default stream).  The box
 * must contain every position (it sets the cell grid).  All scratch is one static device
 * array of about 5.8 MiB that every GPU loading this library holds until exit.  Limits:
 * nb <= SPHGB_NOALLOC_MAX_BOUNDARY (else SPHGB_ERR_CAPACITY) and at most
 * SPHGB_NOALLOC_MAX_CELLS grid cells of 1.001 x 4 r (else SPHGB_ERR_GRID).  The first call on a
 * device looks up the scratch address (cudaGetSymbolAddress) and should be made before any
 * stream capture; the address is looked up through the CUDA runtime, so it is that of the
 * device's primary context (callers on a non-primary driver-API context of the same device are
 * not supported).  Calls share the scratch: calls that overlap on the GPU (other streams,
 * other host threads) race; serialise them.  Non-finite box values or radius:
 * SPHGB_ERR_ARGUMENT.  Returns without waiting for the GPU. */
#define SPHGB_NOALLOC_MAX_BOUNDARY 65536
#define SPHGB_NOALLOC_MAX_CELLS 262144
int sphgb_boundary_volume_noalloc(const float *xb, uint32_t nb, double particle_radius,
                                  const double box_min[3], const double box_max[3], float *volume,
                                  void *stream);

/* Lanes per particle of the neighbour passes (1, 2 or 4; 32 / lanes particles per warp, kBlock /
 * lanes particles per 256-thread block): the lanes of a particle walk interleaved parts of its
 * fluid list, which is stored in the matching layout, and combine their sums with warp shuffles.
 * 0 (default): an autotuner times one trial step per candidate on the first step after an
 * upload (trials are undone) and keeps the fastest.  No reference counterpart. */
int sphgb_set_lanes_per_particle(sphgb_ctx *ctx, uint32_t lanes);
/* the lanes in use and the autotuner's trial step times in ms for 1, 2, 4 lanes (zeros when fixed) */
int sphgb_get_lanes_per_particle(const sphgb_ctx *ctx, uint32_t *lanes, float trial_ms[3]);

/* Threads per block of the two solver passes (pressure acceleration, Jacobi update) when they run
 * one lane per particle, unstaged: 128, 256 or 512 (512 for one scene only; a batch's blocks
 * never span two scenes' 256-slot tiles).  The resident threads per SM are the same at every
 * size.  0 (default): the autotuner times 128 and 512 beside 256 on the first step after an
 * upload.  Results do not depend on it but for the order of the FP64 error sums.  No reference
 * counterpart. */
int sphgb_set_solver_block_threads(sphgb_ctx *ctx, uint32_t threads);
/* the threads per block in use and the autotuner's trial step times in ms for 128, 256, 512 (zeros
 * where not timed) */
int sphgb_get_solver_block_threads(const sphgb_ctx *ctx, uint32_t *threads, float trial_ms[3]);

/* Neighbourhood staging of the two solver passes (FP32 contexts, one lane per particle): every
 * block of 256 particles copies the records of the cells around its particles into shared
 * memory once per pass and walks 16-bit local lists written by the list build in the order of
 * the fluid lists, so the results are bitwise those of the unstaged passes.  Blocks whose
 * neighbourhood exceeds 2048 particles (1536 in the Jacobi pass) read from global memory.
 * mode 0 (default): the
 * autotuner times it as a fourth candidate (and a fixed lane count of 1 uses it); 1: off;
 * 2: on.  No reference counterpart. */
int sphgb_set_neighbor_staging(sphgb_ctx *ctx, int mode);
/* whether the passes run staged, the fraction of the last step's blocks that were staged
 * (waits for the stream) and the autotuner's staged trial step time in ms (0 when not timed);
 * each pointer may be NULL */
int sphgb_get_neighbor_staging(sphgb_ctx *ctx, int *active, float *staged_fraction, float *trial_ms);

/* Dynamic boundary bodies: the forces and torques the fluid exerts on them, the device-side
 * counterpart of BoundaryModel::addForce / getForceAndTorque / clearForceAndTorque
 * (SPlisHSPlasH/BoundaryModel.h:38-49, 86-87; read and cleared by the boundary simulator each
 * step, Simulator/BoundarySimulator.cpp:8-25).  body[k] < nbodies is the body of boundary
 * particle k in upload order (a batch: all scenes' boundaries in scene order); center[3 b] is
 * body b's reference point for torques (RigidBodyObject::getPosition); dynamic[b] != 0 marks a
 * body that collects forces (RigidBodyObject::isDynamic), dynamic == NULL marks every body
 * dynamic.  Every step adds, for each dynamic body, the boundary terms of the divergence and
 * pressure solves' final pressure accelerations (TimeStepDFSPH.cpp:359, 514), of XSPH
 * (XSPH.cpp:183-203) and of Weiler2018 viscosity (Viscosity_Weiler2018.cpp:960-975): force
 * sum f and torque sum (x_b - center) x f, summed in FP64 in a fixed order (deterministic).
 * The boundary stays static (v_b = 0); moving a body is the caller's rigid-body solver, which
 * re-uploads the boundary.  Setting the bodies (nbodies == 0 removes them) zeroes the
 * accumulators; uploading a boundary of another particle count removes them.  With volume maps
 * (sphgb_set_boundary_method 2) body b is map b, body may be NULL, and the forces of the same
 * terms act at the particles' boundary points x_j (TimeStepDFSPH.cpp:1355-1364, XSPH.cpp:196-204). */
int sphgb_set_boundary_bodies(sphgb_ctx *ctx, const uint32_t *body, uint32_t nbodies, const double *center,
                              const int *dynamic);
/* Pose and velocity of boundary body `body` (of sphgb_set_boundary_bodies) for the following
 * steps: its particles, uploaded in body coordinates (the reference's getPosition0), are placed at
 * R x0 + t and move at w x (R x0) + v, as SimulatorBase::updateBoundaryParticles does every step
 * (SimulatorBase.cpp:1620-1645).  From the first call on, the boundary particles are placed and
 * sorted into the grid at the start of every step, their velocities enter every boundary term as
 * v_i - v_b (divergence source and density advection, TimeStepDFSPH.cpp:1218-1223, 1273-1278;
 * XSPH, XSPH.cpp:176-183; Weiler2018's right-hand side and force, Viscosity_Weiler2018.cpp:
 * 1130-1138, 966-975), their squared speeds the CFL maximum (Simulation.cpp:442-458), and the
 * body's torque is taken about t.  The volumes stay those computed for the uploaded shape.
 * Bodies without a call stay in their uploaded pose at rest.  rotation (row-major) / translation
 * NULL keep the current ones; velocity / omega NULL are zero.  In a batch a body's particles stay
 * in their scene; volume-map bodies move with sphgb_set_volume_map_motion. */
/* Several fluid phases in one scene, as the reference's multiphase scenes hold several FluidModels
 * of different rest density: the uploaded particles in particle-id order form nphases consecutive
 * groups of counts[k] particles with rest density density0[k] (mass V density0[k]; the particle
 * volume V is common).  Every particle's density and density error use its own rest density, the
 * pressure acceleration sums kappa_i + (density0_j / density0_i) kappa_j (TimeStepDFSPH.cpp:1312),
 * XSPH weighs neighbours by their own mass, and each solver iteration visits the phases in turn,
 * each against its own tolerance (:322-339, :476-495), so a phase sees the kappa the phases before
 * it updated in the same iteration.  Weiler2018 viscosity solves one system per phase, in phase
 * order, over same-phase fluid neighbours with mu = viscosity density0[k] and mub =
 * viscosity_boundary density0[k] (Viscosity_Weiler2018.cpp:288-289, a per-model force); the step's
 * visco_iterations is the phases' sum and visco_error their largest.  nphases <= 1 returns to one
 * phase of sphgb_params.density0.  At the step: SPHGB_ERR_STATE when the counts do not add up to
 * the fluid or for a batch; SPHGB_ERR_ARGUMENT with the learned warm start.  Up to 8 phases. */
int sphgb_set_fluid_phases(sphgb_ctx *ctx, uint32_t nphases, const uint32_t *counts, const double *density0);

/* Weiler2018 coefficients per fluid phase, as each FluidModel of the reference carries its own
 * viscosity and viscosityBoundary (Viscosity_Weiler2018.cpp:288-289): phase k's system takes mu =
 * viscosity[k] density0[k] and mub = viscosity_boundary[k] density0[k].  Phases beyond nphases
 * (and every phase after nphases = 0) take sphgb_params.viscosity / viscosity_boundary.
 * SPHGB_ERR_ARGUMENT for a negative or non-finite value or more than 8 phases. */
int sphgb_set_fluid_phase_viscosity(sphgb_ctx *ctx, uint32_t nphases, const double *viscosity,
                                    const double *viscosity_boundary);

/* XSPH coefficients per fluid phase, as each FluidModel's XSPH carries its own xsph and
 * xsphBoundary (XSPH.cpp:19-39): a particle's filter takes its phase's coefficients, over the
 * neighbours of every phase.  Phases beyond nphases take sphgb_params.xsph / xsph_boundary.
 * SPHGB_ERR_ARGUMENT for a non-finite value or more than 8 phases. */
int sphgb_set_fluid_phase_xsph(sphgb_ctx *ctx, uint32_t nphases, const double *xsph, const double *xsph_boundary);
int sphgb_set_body_motion(sphgb_ctx *ctx, uint32_t body, const double rotation[9], const double translation[3],
                          const double velocity[3], const double omega[3]);
/* the sums since the last clear, force[3 nbodies] and torque[3 nbodies] (either may be NULL;
 * zeros for static bodies); waits for the context's stream */
int sphgb_boundary_forces(sphgb_ctx *ctx, double *force, double *torque);
/* zero the sums of one body (body < 0: of every body), ordered after the steps already enqueued */
int sphgb_clear_boundary_forces(sphgb_ctx *ctx, int32_t body);

/* Bender2019 boundaries (BoundaryModel_Bender2019, the reference's default boundary handling,
 * Simulation.cpp:88): bodies given as volume maps instead of boundary particles.
 * A map is Discregrid's cubic Lagrange grid restated: res cells per axis over the body's box, the
 * 32-node cubic serendipity element per cell, two fields per node, the signed distance phi (positive
 * on the fluid side) and the boundary volume.  Every step samples each body at
 * R^T (x_i - translation) and treats x_j = x_i - max(phi + r / 2, 2 r) n with volume V_j, for
 * 0 < phi < 4 r, as one boundary particle per body in all DFSPH, XSPH sums
 * (TimeStep::computeVolumeAndBoundaryX, TimeStep.cpp:219-340); a particle found inside a body
 * is moved back by min(2 r - phi, r / 10) and stopped, as in the reference.  The Weiler2018
 * boundary viscosity samples each x_j at the four points x_j -+ t1 h / 2, x_j -+ t2 h / 2 of the
 * tangent plane, a quarter of V_j each (Viscosity_Weiler2018.cpp:205-255).  Supported: one
 * no boundary particles uploaded; in a batch every map belongs to one scene
 * (sphgb_set_volume_map_scene); moving bodies through sphgb_set_volume_map_motion; force
 * feedback with one body per map
 * (sphgb_set_boundary_bodies); other combinations fail at the step with SPHGB_ERR_STATE /
 * SPHGB_ERR_ARGUMENT.
 *
 * sphgb_add_volume_map builds a map on the GPU in FP64 from a closed triangle mesh in body
 * coordinates, as SimulatorBase::initVolumeMap does (SimulatorBase.cpp:2512-2660): box = mesh box
 * grown by 8 h + thickness (h = 4 r of the current parameters), phi = sign (d - thickness) with d
 * the pseudo-normal signed mesh distance and sign = -1 when invert (a container), volume = 0.8 x
 * the Gauss-Legendre integral (order; 0 = 30, the reference's) over the support of the clipped
 * kernel-weighted indicator.  rotation (row-major) / translation NULL = identity / 0.  body
 * receives the map's index.  sphgb_add_volume_map_values adds a map from node values (as a
 * reference "mapFile"); sphgb_get_volume_map reads one back (node count = (rx+1)(ry+1)(rz+1) +
 * 2 rx(ry+1)(rz+1) + 2 (rx+1) ry (rz+1) + 2 (rx+1)(ry+1) rz; distance / volume may be NULL).
 * sphgb_set_boundary_method: 0 Akinci2012 boundary particles (default), 2 Bender2019 maps
 * ("boundaryHandlingMethod", Simulation.cpp:88). */
int sphgb_add_volume_map(sphgb_ctx *ctx, const double *vertices, uint32_t nv, const uint32_t *faces, uint32_t nf,
                         const uint32_t resolution[3], double thickness, int invert, const double rotation[9],
                         const double translation[3], uint32_t order, uint32_t *body);
int sphgb_add_volume_map_values(sphgb_ctx *ctx, const uint32_t resolution[3], const double box_min[3],
                                const double box_max[3], const double *distance, const double *volume,
                                const double rotation[9], const double translation[3], uint32_t *body);
int sphgb_get_volume_map(sphgb_ctx *ctx, uint32_t body, uint32_t resolution[3], double box_min[3], double box_max[3],
                         double *distance, double *volume);
int sphgb_clear_volume_maps(sphgb_ctx *ctx);
int sphgb_set_boundary_method(sphgb_ctx *ctx, int method);
/* The scene of a batch (sphgb_upload_scenes) that volume map `body` belongs to (default 0): the
 * particles of each scene see only the maps of their scene, and a scene's step size only its
 * moving maps.  SPHGB_ERR_ARGUMENT at the step for a scene that is not uploaded. */
int sphgb_set_volume_map_scene(sphgb_ctx *ctx, uint32_t body, uint32_t scene);
/* Pose and velocity of the body of volume map `body` for the following steps, as the reference
 * reads them from the map's rigid body every step (BoundaryModel_Bender2019 with a dynamic or
 * animated RigidBodyObject): the map is sampled at R^T (x - t) (TimeStep.cpp:219-340), and the
 * velocity of a body point p, w x (p - t) + v (BoundaryModel::getPointVelocity,
 * BoundaryModel.h:78-84), enters every boundary term as v_i - v_p: the divergence source and the
 * density advection (TimeStepDFSPH.cpp:1218-1238, 1273-1293), XSPH (XSPH.cpp:119-128),
 * Weiler2018's right-hand side at its four samples (Viscosity_Weiler2018.cpp:1191-1243) and the
 * forces on the body (its torque taken about t); the CFL step size also bounds the body's speed
 * |w x (maxDist, 0, 0) + v| (Simulation.cpp:466-476, SimulatorBase.cpp:1670-1687), maxDist the
 * largest distance of a mesh vertex from the vertices' mean (0 for a map given by node values).
 * rotation (row-major) / translation NULL keep
 * the current ones; velocity / omega NULL are zero.  Moving the body is the caller's rigid-body
 * solver's job: call this before each step. */
int sphgb_set_volume_map_motion(sphgb_ctx *ctx, uint32_t body, const double rotation[9], const double translation[3],
                                const double velocity[3], const double omega[3]);

/* the cudaStream_t every kernel of this context is launched on (for event timing by callers) */
int sphgb_get_stream(const sphgb_ctx *ctx, void **stream);

/* Per-kernel CUDA-event timing, the device-side counterpart of the reference's
 * START_TIMING / STOP_TIMING_AVG scopes (Utilities/Timing.h:73-187).  While on,
 * steps run with host-driven loops so every launch can be bracketed by events.
 * profile_read walks kernel classes by index until it returns SPHGB_ERR_ARGUMENT. */
int sphgb_profile_enable(sphgb_ctx *ctx, int on);
int sphgb_profile_reset(sphgb_ctx *ctx);
int sphgb_profile_read(const sphgb_ctx *ctx, int index, const char **name, uint64_t *launches, double *total_ms);

#ifdef __cplusplus
}
#endif
#endif
