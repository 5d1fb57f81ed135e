/*
 * CPU oracle for the DFSPH time-step hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference algorithm (SPlisHSPlasH 2.16.0)
 * used as the checker for the CUDA path.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference legs may load it.  The product
 * path (splishsplash_gb300, libsphgb300.so) never calls into it.
 *
 * Pinning status:
 *   - Cubic spline W / gradW: pinned against values produced by the reference's
 *     own SPHKernels.{h,cpp} (compiled from the reference tree by
 *     oracle/build_ref.sh into oracle/_ref/), stored in tests/golden/.
 *   - 3x3 block-Jacobi preconditioned CG: pinned against the reference's
 *     MatrixFreeSolver.h + vendored Eigen 3.4 ConjugateGradient, run on the
 *     oracle's own Weiler2018 operator (tests/golden/).
 *   - DFSPH / Akinci2012 / XSPH / Weiler2018 per-particle sums and the solver
 *     loops: pinned against the reference's own TimeStepDFSPH step.  The
 *     reference's library sources are compiled by oracle/build_ref.sh (FP64,
 *     analytic kernel) against stand-ins for its absent external projects
 *     (oracle/shims/), and one reference step from three float32 states is
 *     stored in tests/golden/ref_step_*.npz; this oracle reproduces each to
 *     1e-10 with equal iteration counts (tests/test_reference_pin.py).
 *     Every function below cites the reference file:line it restates.
 *   - The neighbour predicate: CompactNSearch is not in the reference tree, so
 *     the documented |x_i - x_j|^2 < h^2 (self excluded) stands for it, here, on
 *     the GPU and in the reference build's stand-in alike.
 *
 * Build: two precisions from one source (ORC_REAL = double | float).  The FP64
 * build is the parity oracle; the FP32 build is the CPU baseline where the
 * reference's own FP32 AVX build cannot run (a port of the reference's FP32
 * OpenMP path, not the reference binary).
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef ORC_REAL
#define ORC_REAL double
#endif
typedef ORC_REAL orc_real;

typedef struct orc_params {
    double radius;               /* particle radius r; support radius = 4r (Simulation.cpp:283) */
    double density0;             /* rest density (FluidModel density0) */
    double gravity[3];           /* Simulation::GRAVITATION */
    int cfl_method;              /* 0 none, 1 CFL, 2 CFL + iteration heuristic (Simulation.cpp:395-413) */
    double cfl_factor, cfl_min, cfl_max;
    unsigned min_iterations, max_iterations;   /* DFSPH minIterations / maxIterations */
    double max_error;                          /* DFSPH maxError (percent) */
    int enable_divergence_solver;
    unsigned max_iterations_v;                 /* DFSPH maxIterationsV */
    double max_error_v;                        /* DFSPH maxErrorV (percent) */
    double xsph_fluid, xsph_boundary;          /* XSPH xsph / xsphBoundary */
    int viscosity_method;                      /* 0 none, 6 Weiler et al. 2018 */
    double viscosity, viscosity_boundary;      /* Weiler viscosity / viscosityBoundary */
    unsigned visco_max_iter;                   /* Weiler viscoMaxIter */
    double visco_max_error;                    /* Weiler viscoMaxError */
    int fp32_predicate;          /* evaluate |xi-xj|^2 < h^2 in float (as the FP32 device path) */
    int num_threads;             /* OpenMP threads (0 = runtime default) */
    int boundary_method;         /* Simulation "boundaryHandlingMethod": 0 Akinci2012 (boundary particles
                                    xb, Vb), 2 Bender2019 (volume maps of orc_state.vmaps) */
} orc_params;

/* Volume map of one Bender2019 boundary body: Discregrid's CubicLagrangeDiscreteGrid (the
 * cubic serendipity element of 32 nodes per cell: 8 vertices and 2 nodes at 1/3 and 2/3 of each
 * edge, shared between cells) restated, with two fields: 0 signed distance, 1 boundary volume.
 * The grid lies in body-local coordinates over [dmin, dmax] with res cells per axis; a point x
 * of the scene is looked up at R^T (x - t). */
typedef struct orc_vmap {
    double dmin[3], dmax[3];
    unsigned res[3];
    double *field[2];            /* orc_vmap_nodes(res) values each */
    double R[9], t[3];           /* rotation (row-major) and position of the body */
    double v[3], w[3];           /* its linear and angular velocity: the velocity of a point p of the
                                    body is w x (p - t) + v (BoundaryModel::getPointVelocity,
                                    BoundaryModel.h:78-84); zero for a static body */
    double max_dist;             /* largest distance of a mesh vertex from the vertices' mean
                                    (SimulatorBase.cpp:2706-2729), for the CFL bound of a moving body */
} orc_vmap;

typedef struct orc_state {
    unsigned n, nb;
    orc_real *x, *v, *a;                  /* 3n, AoS (x0,y0,z0,x1,...) like Vector3r */
    orc_real *density, *factor, *density_adv, *kappa, *kappa_v;   /* n */
    orc_real *pressure_accel, *vdiff;     /* 3n */
    orc_real *xb, *Vb;                    /* 3nb, nb (boundary particles and their volumes) */
    double dt, time;
    /* written by orc_step */
    unsigned iterations, iterations_v, visco_iterations;
    double avg_density_err, avg_density_err_v, visco_error;
    double dt_old;
    /* optional outputs (may be NULL) */
    orc_real *factor_raw;                 /* alpha right after computeDFSPHFactor */
    orc_real *density_adv_v;              /* divergence source (unclamped) */
    unsigned *num_fluid_neighbors, *num_boundary_neighbors;
    /* optional dynamic-boundary feedback (BoundaryModel::addForce, BoundaryModel.h:38-49):
     * body index of every boundary particle, the bodies' reference points (rigid-body
     * positions) and dynamic flags.  orc_step adds to body_force / body_torque (the caller
     * clears them, like clearForceAndTorque) the forces the fluid exerts on the dynamic bodies
     * during the step: the final pressure
     * accelerations of both solvers (TimeStepDFSPH.cpp:359, 514 with :1342-1343), the XSPH
     * boundary term (XSPH.cpp:183-203) and the Weiler2018 boundary term
     * (Viscosity_Weiler2018.cpp:960-975); torque about the reference point. */
    const unsigned *body;
    unsigned nbodies;
    const double *body_center;            /* 3 nbodies */
    const int *body_dynamic;              /* nbodies */
    double *body_force, *body_torque;     /* 3 nbodies */
    /* Bender2019 boundary (boundary_method 2): one volume map per body.  With body == NULL and
     * body_force given, map b is body b (centres, dynamic flags and sums as above), its force
     * applied at the particle's boundary point x_j (addForce(xj, ...) of the Bender2019 branches). */
    const orc_vmap *vmaps;
    unsigned nvmaps;
    /* velocities of the boundary particles [nb][3] (BoundaryModel_Akinci2012::getVelocity of a
     * moving body, SimulatorBase.cpp:1620-1645); NULL: static walls */
    const orc_real *vb;
    /* fluid phases (several FluidModels in one simulation): the particles in index order form
     * nphase consecutive groups of phase_count[k] particles with rest density phase_density0[k];
     * nphase <= 1: one model of density0 */
    unsigned nphase;
    const unsigned *phase_count;
    const double *phase_density0;
    /* Weiler2018 nu and nu_b per phase (each FluidModel's own, Viscosity_Weiler2018.cpp:288-289);
     * NULL: the parameters' viscosity / viscosity_boundary for every phase */
    const double *phase_viscosity, *phase_viscosity_boundary;
    /* XSPH fluid and boundary coefficients per phase (each FluidModel's own, XSPH.cpp:19-39);
     * NULL: the parameters' xsph_fluid / xsph_boundary for every phase */
    const double *phase_xsph, *phase_xsph_boundary;
} orc_state;

/* Cubic spline (SPHKernels.h:16-91). */
double orc_kernel_W(double r, double support);
void orc_kernel_gradW(const double r[3], double support, double out[3]);

/* Neighbour lists as CSR sorted ascending per particle.  For query points x (n)
 * against points y (m); self excluded when same_set != 0.  Returns 0 on success.
 * offsets must hold n+1 entries; when indices == NULL only the counts/offsets are
 * produced.  Predicate: squared distance < support^2, evaluated in float when
 * fp32 != 0 (separate multiplies and adds, no fused multiply-add). */
int orc_neighbors(unsigned n, const orc_real *x, unsigned m, const orc_real *y,
                  double support, int same_set, int fp32,
                  unsigned *offsets, unsigned *indices, unsigned capacity);

/* Akinci2012 boundary volume V_b = 1 / (W0 + sum_b' W(x_b - x_b'))
 * (BoundaryModel_Akinci2012.cpp:48-75). */
int orc_boundary_volume(unsigned nb, const orc_real *xb, double support, int fp32, orc_real *Vb);

/* One TimeStepDFSPH::step() (TimeStepDFSPH.cpp:117-249). */
int orc_step(orc_state *s, const orc_params *p);

/* ---- Bender2019 volume maps (vmap.c) ---- */
/* nodes of a grid of res cells: vertices, then the x-, y- and z-edge nodes */
size_t orc_vmap_nodes(const unsigned res[3]);
void orc_vmap_node_position(const orc_vmap *m, size_t node, double p[3]);
/* DiscreteGrid::interpolate with its gradient: 0 (value untouched) outside [dmin, dmax] */
int orc_vmap_interpolate(const orc_vmap *m, int field, const double xl[3], double *value, double grad[3]);
/* SimulatorBase::initVolumeMap (SimulatorBase.cpp:2512-2660): the domain is the mesh's box grown
 * by 8 h + thickness; field 0 = sign (d - thickness), d the signed distance to the triangle mesh
 * (positive outside, pseudo-normal sign), sign -1 when invert; field 1 = 0 where field 0 > 2 h,
 * else 0.8 x the Gauss-Legendre integral (order, GaussQuadrature.cpp:5930-5962) over [-h, h]^3 of
 * gamma(phi(x + y)) for |y| < h, gamma = 1 inside, W(phi) / W(0) within h, 0 beyond.  field[0]
 * and field[1] must hold orc_vmap_nodes(res) values; R and t are left to the caller. */
int orc_vmap_build(orc_vmap *m, const double *vert, unsigned nv, const unsigned *tri, unsigned nt,
                   double support, double thickness, int invert, unsigned order);
/* the domain orc_vmap_build uses, for sizing field arrays before the call */
void orc_vmap_domain(const double *vert, unsigned nv, double support, double thickness, double dmin[3],
                     double dmax[3]);

/* Weiler2018 operator pieces for the CG pin (Viscosity_Weiler2018.cpp:271-443,
 * 605-742).  Lists are rebuilt from state positions. */
int orc_weiler_system(const orc_state *s, const orc_params *p, double dt,
                      orc_real *b, orc_real *g, orc_real *diag9);
int orc_weiler_matvec(const orc_state *s, const orc_params *p, double dt,
                      const orc_real *vec, orc_real *result);
/* CG restatement (ConjugateGradient.h:29-90 with MatrixFreeSolver.h:201-272). */
int orc_weiler_solve(const orc_state *s, const orc_params *p, double dt,
                     orc_real *x_out, unsigned *iters, double *err);

#ifdef __cplusplus
}
#endif
#endif
