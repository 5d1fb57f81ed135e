// Internal structures shared by the host orchestration (api.cu) and the kernel
// translation units.  Not part of the public ABI (include/sphgb300.h).
//
// A context advances one or more independent scenes together.  Scene s owns the
// fluid slots [pstart_s, pstart_s + n_s) with pstart_s a multiple of the block
// size, so a thread block never spans two scenes; it owns the cells
// [cell_off_s, cell_off_s + ncell_s) of the shared cell tables and one
// StepScalars record (its own dt, CFL, iteration counters and convergence flags).
// Every kernel of a step covers all scenes in one launch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_common.cuh"
#include "vmap.cuh"

namespace sphgb {

// Scalars that live in device memory so that a captured step can be replayed
// without host updates.  All solver control (iteration counters, convergence
// flags, the CFL step size) is decided on the device.  One record per scene and
// one global record (launch counter, loop guard, OR of the scenes' loop flags).
struct StepScalars {
    double dt;          // step size of the current step (used by kick / position update)
    double dt_next;     // CFL result, used by the pressure solve and the next step
    double time;
    double dt_used;     // step size the last completed step used
    double avg_err;     // pressure solve
    double avg_err_v;   // divergence solve
    double cg_rhs2, cg_thresh, cg_res2, cg_absnew, cg_alpha, cg_beta, cg_err;
    double ws_rc[2], ws_rl[2];   // initial residuals of the classic / learned warm start (div, pressure)
    unsigned iters, iters_v, iters_cg;
    unsigned cont;      // 1 while the running solver loop continues (global record: any scene)
    unsigned cg_state;  // 0 running, 1 converged / no iteration, 2 zero right-hand side
    unsigned maxvel_bits;
    unsigned flags;     // bit 0 list overflow, bit 1 non-finite velocity, bit 2 loop guard
    unsigned max_nf, max_nb;
    unsigned prev_iters;
    unsigned loop_guard;   // body executions of the running device-side loop (global record)
    unsigned launches;     // kernels launched in the current step (global record)
    unsigned ws_used;      // bit 0: learned warm start used by the divergence solve, bit 1: pressure solve
    unsigned live;         // scenes whose running loop continues (global record, batches)
    unsigned pad1;
    unsigned long long maxvel_bits64;   // FP64 contexts: max |v + a h|^2 as the bits of a non-negative double
    unsigned phase_ok;  // fluid phases: bit k set when phase k met its tolerance in the running iteration
    // Weiler2018 with fluid phases, one CG system per phase: iterations summed over the phases,
    // the largest final residual of the phases before the running one, bit k: phase k had a zero
    // right-hand side (solution 0)
    unsigned iters_cg_tot, cg_zero;
    double cg_err_max;
};

constexpr unsigned kFlagOverflow = 1u;
constexpr unsigned kFlagNonFinite = 2u;
constexpr unsigned kFlagLoopGuard = 4u;   // a device loop ran past its iteration bound and was stopped

__device__ __forceinline__ void count_launch(unsigned *ctr)
{
    if (ctr && blockIdx.x == 0 && threadIdx.x == 0) *ctr += 1u;
}

// Per-scene layout and cell grid.
template <class T> struct SceneDev {
    T ox, oy, oz, inv_cell;      // grid origin, 1 / cell size
    int dimx, dimy, dimz;
    uint32_t cell_off;           // first cell of the scene in the shared cell tables
    uint32_t pstart;             // first fluid slot (multiple of kBlock)
    uint32_t n;                  // fluid particles
    uint32_t ustart;             // first particle of the scene in upload (particle id) order
    uint32_t key_prefix;         // scene index << Morton bits
};

template <class T> struct DevParams {
    Kernel<T> K;
    T V, mass, rho0, eps;
    T gx, gy, gz;
    T xsph, xsph_b;
    T mu, mub, vd, h2;            // Weiler: mu = nu rho0, d = 10, h^2 (support)
    double max_error, max_error_v;
    double cfl_factor, cfl_min, cfl_max, radius;
    double visc_tol;
    unsigned min_iter, max_iter, max_iter_v, visc_max_iter;
    int cfl_method, visc_on, div_on;
    int learned, feat_on;         // learned warm start on; features computed
    float ws_scale_v, ws_scale_p; // network output scales (output x scale = warm-start multiplier)
    // scenes
    uint32_t nscenes;
    SceneDev<T> s0;               // the scene when nscenes == 1 (no device lookup)
    const SceneDev<T> *scenes;    // device array [nscenes] when nscenes > 1
    const uint4 *blk;             // device array [blocks] when nscenes > 1: (scene, first slot, end slot, -)
    uint32_t np;                  // fluid slots (sum of padded scene ranges): launch size
    uint32_t nreal;               // fluid particles of all scenes
    uint32_t nb;                  // boundary particles of all scenes
    uint32_t capf, capb;
    uint32_t lpp_log2;            // lanes per particle of the neighbour passes (1, 2 or 4) = 1 << lpp_log2;
                                  // also fixes the layout of the fluid lists
    uint32_t nvmaps;              // Bender2019 boundary: volume maps (bodies); 0 = Akinci2012 particles
    const VMapDev<T> *vmaps;      // device array [nvmaps], ordered by scene
    const uint2 *vmap_range;      // batches: per scene, first map and map count (null: one scene, all maps)
    const uint4 *vmap_info;       // batches: per map, (body, scene, slot within the scene's maps, 0)
    uint32_t vmap_max;            // maps of the scene with the most (per-particle boundary points)
    int vmove;                    // some volume-map body moves: boundary terms use v_i - v_b
    // fluid phases (several fluid models of one scene): particle ids [phase_end[k-1], phase_end[k])
    // form phase k of rest density phase_rho0[k] and phase_count[k] particles; nphase <= 1: one model
    uint32_t nphase;
    uint32_t phase_end[8], phase_count[8];
    T phase_rho0[8];
    T phase_nu[8], phase_nub[8];  // Weiler per phase: nu and nu_b (mu = nu rho0 of the particle's phase)
    T phase_xs[8], phase_xsb[8];  // XSPH per phase: fluid and boundary coefficients
    int bmove;                    // boundary particles move with their bodies: placed and re-sorted every
                                  // step, with velocities (one scene)
    int staged;                   // FP32, one lane per particle: the solver passes read their block's
                                  // neighbourhood from shared memory (stage tables, local lists)
    uint32_t solver_nt;           // threads per block of the two solver passes with one lane per particle,
                                  // unstaged: 128, 256 or 512 (one scene)
};

// Neighbourhood staging of the solver passes.  For every block of kBlock slots the step's
// stage table lists the cells of the union of its particles' 27-cell neighbourhoods (ascending
// cell index) with the offset of each cell's first particle in the block's staged array; the
// local fluid lists hold, per neighbour, its index in that array.  A block whose neighbourhood
// has more than kStageCells cells, more than kStageCap particles or a bounding box of more than
// kStageBoxCells cells is not staged and reads its neighbours from global memory.
constexpr uint32_t kStageCap = 2048;        // staged particles per block (16-bit local indices)
constexpr uint32_t kStageCapJacobi = 1536;  // ... that the Jacobi pass stages (24 B each; 6 blocks per SM)
constexpr uint32_t kStageCells = 384;       // staged cells per block
constexpr uint32_t kStageBoxCells = 4096;   // cells of the block's dilated bounding box (bitmap)

// Scene descriptor by value: a kernel parameter for a single scene, a (cached) global load otherwise.
template <class T> __device__ __forceinline__ SceneDev<T> scene_get(const DevParams<T> &P, uint32_t s)
{
    if (P.nscenes > 1) return P.scenes[s];
    return P.s0;
}

template <class T> struct DevBufs {
    using v4 = v4_t<T>;
    // state, current order
    v4 *x, *v, *vdiff;
    float4 *xlo;                 // FP32 mode: low part of the double-float position
    T *kappa, *kappa_v;
    uint32_t *id;
    // state, alternate (gather target)
    v4 *x2, *v2, *vdiff2;
    float4 *xlo2;
    T *kappa2, *kappa_v2;
    uint32_t *id2;
    // per-step fields
    v4 *a, *pa;
    float4 *xa;                  // FP32 solver loops: (x_i, a_i) as one 32-byte record per particle,
                                 // written by the pressure-acceleration pass, read by the Jacobi pass
    v4 *xk;                      // x_i with the running solver's kappa_i in w (one gather per pair)
    v4 *bg;                      // per-particle boundary sums: xyz = sum_b V_b gradW_ib, w = sum_b V_b W_ib
    v4 *bx;                      // Bender2019: [nvmaps][np] boundary point x_j of each particle's map sample, w = V_j
    T *r0;                       // fluid phases: rest density of slot i
    uint32_t *ph;                // fluid phases: phase of slot i
    v4 *vbs;                     // moving boundary bodies: velocity of sorted boundary particle k
    uint32_t *binv;              // sorted slot of boundary particle u (upload order)
    v4 *bv;                      // moving volume-map bodies, per particle: xyz = sum_b V_b W_ib v_b,
                                 // w = sum_b V_b v_b . gradW_ib (fixed for the step, like bg)
    T *density, *factor, *dadv;
    uint32_t *nf, *nbn;
    uint32_t *lf, *lb;
    // neighbourhood staging (staged mode): per block (cells, particles) with cells = 0 for a block
    // that is not staged, the cell ids and offsets, and the local fluid lists (warp-interleaved,
    // the layout of lf with one lane per particle)
    uint2 *stage_hdr;
    uint32_t *stage_cell;
    uint16_t *stage_off;
    uint32_t *stage_src;         // [blocks][kStageCap] slot of every staged particle
    uint16_t *ll;
    // cell grid
    uint32_t *key, *key2, *perm, *perm2, *cellid, *cellid2;
    uint32_t *cstart, *cend;
    uint32_t *bcstart, *bcend;
    v4 *xb;                      // sorted boundary positions, w = volume
    T *bscratch;                 // nb scratch values (boundary volume set-up)
    uint32_t *bid;               // upload index of each sorted boundary particle
    uint32_t *bscene;            // scene of each sorted boundary particle
    // learned warm start
    float *feat;                 // raw features, 8 floats per particle (5 used)
    float *mlp_x;                // network inputs, 10 floats per particle
    float *mlp_y;                // network outputs, 2 floats per particle
    T *kl;                       // predicted warm start of the running solver
    v4 *pa2;                     // pressure acceleration of the predicted warm start
    const void *mlp_w;           // BF16 weights
    const float *mlp_p;          // FP32 parameters (biases)
    // CG
    v4 *cg_x, *cg_r, *cg_p, *cg_z, *cg_t;
    v4 *inv0, *inv1;             // symmetric 3x3 inverse blocks: (m00,m01,m02,m11), (m12,m22,-,-)
    // reductions
    double *partials;            // [4][blocks]
    unsigned *counters;          // [nscenes + 1]: per-scene last-block counters, then the global one
    StepScalars *sc;             // [nscenes]
    StepScalars *gsc;            // global record
    // radix sort scratch
    uint32_t *hist;
};

// Dynamic boundary bodies (force feedback of BoundaryModel::addForce): the boundary slots of
// the dynamic bodies grouped by body, a block table whose blocks never span two bodies, and
// the per-body accumulators.
struct BodyDev {
    const uint32_t *slot;        // [entries] sorted boundary slots, grouped by body, slot order within a body
    const uint4 *blk;            // [nblk] (body, first entry, end entry, first block of the body)
    const uint32_t *body_nblk;   // [nbodies] blocks of each body
    const double *center;        // [3 nbodies] reference points of the torques
    double *acc;                 // [6 nbodies] force xyz, torque xyz, accumulated until cleared
    double *partials;            // [6][nblk] block partial sums
    unsigned *counters;          // [nbodies] last-block counters, zero between launches
    uint32_t nblk;
    // volume-map bodies (Bender2019): body b is map b
    const int *dynamic;          // [nbodies] 1 if the body collects forces
    double *vpartials;           // [nbodies][6][blocks of the particle launch]
    uint32_t nbodies;
};

// ---- Bender2019 volume maps (vmap.cu) ----
// the grid box of a map: the mesh's bounding box grown by 8 support + thickness
void vmap_domain(const double *vert, uint32_t nv, double support, double thickness, double dmin[3], double dmax[3]);
// node fields (device, FP64, VMapLayout(res).nodes() each) of the map of a triangle mesh; waits for the stream
cudaError_t vmap_build_device(const double *vert, uint32_t nv, const uint32_t *tri, uint32_t nt, const uint32_t res[3],
                              double support, double thickness, int invert, uint32_t order, double *f0, double *f1,
                              const double dmin[3], const double dmax[3], cudaStream_t s);
// the per-cell coefficient layout the step reads (VMapDev::coef)
template <class T>
cudaError_t vmap_expand_device(const uint32_t res[3], const double *f0, const double *f1, T *coef, cudaStream_t s);

// ---- launchers (defined in kernels.cu / sort.cu, instantiated for float and double)
template <class T> void launch_keys(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
template <class T> void launch_gather(const DevParams<T> &P, const DevBufs<T> &B, const uint32_t *perm, cudaStream_t s);
template <class T> void launch_cell_ranges(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
template <class T> void launch_build(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
// Bender2019: each particle's boundary points and volumes, particles inside a body moved out
// (after the cell ranges, before the list build)
template <class T> void launch_vmap_boundary(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
// stage tables of the step (staged mode; after the cell ranges, before the list build)
template <class T> void launch_stage_table(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
// shared-memory limits of the staged solver passes; call once per device before their first launch
cudaError_t configure_staged_kernels();
// Pose and velocity of one boundary body (rotation row-major, position, velocity, angular velocity)
template <class T> struct BodyMotionDev {
    T R[9], t[3], v[3], w[3];
};
// Per-step placement of the boundary particles of moving bodies, upload order: rest positions x0
// (body coordinates) and volumes, each particle's body, the bodies' motions, and the placed
// positions (w = V) and velocities before they are sorted
template <class T> struct BoundaryMoveDev {
    const v4_t<T> *x0;
    const T *V0;
    const uint32_t *body;
    const uint32_t *scene;        // batches: each particle's scene (null: one scene)
    const BodyMotionDev<T> *motion;
    v4_t<T> *xtmp, *vtmp;
};
template <class T>
void launch_boundary_move(const DevParams<T> &P, const DevBufs<T> &B, const BoundaryMoveDev<T> &M, uint32_t *keys,
                          uint32_t *vals, cudaStream_t s);
template <class T>
void launch_boundary_regather(const DevParams<T> &P, const DevBufs<T> &B, const BoundaryMoveDev<T> &M,
                              const uint32_t *perm, uint32_t *cells, cudaStream_t s);
// phase: with fluid phases, the phase whose particles the pass updates (-1: all particles)
template <class T> void launch_pressure_accel(const DevParams<T> &P, const DevBufs<T> &B, bool div, int phase, cudaStream_t s,
                                              cudaGraphConditionalHandle h = 0, bool use_handle = false);
template <class T> void launch_jacobi(const DevParams<T> &P, const DevBufs<T> &B, bool div, int phase,
                                      cudaGraphConditionalHandle h, bool use_handle, cudaStream_t s);
template <class T> void launch_solver_finalize(const DevParams<T> &P, const DevBufs<T> &B, bool div, cudaStream_t s);
template <class T> void launch_xsph(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
// The Weiler2018 CG passes; phase >= 0 restricts them to that fluid phase's particles and
// same-phase neighbours (P then carries the phase's mub and rho0), -1 runs one system over all.
template <class T> void launch_visc_setup(const DevParams<T> &P, const DevBufs<T> &B,
                                          cudaGraphConditionalHandle h, bool use_handle, cudaStream_t s,
                                          int phase = -1);
// One fluid phase with viscosity: the XSPH pass and the viscosity set-up in one pass over the
// lists, with the results of launch_xsph followed by launch_visc_setup(phase -1).
template <class T> void launch_xsph_visc_setup(const DevParams<T> &P, const DevBufs<T> &B,
                                               cudaGraphConditionalHandle h, bool use_handle, cudaStream_t s);
template <class T> void launch_cg_matvec(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s,
                                         cudaGraphConditionalHandle h = 0, bool use_handle = false, int phase = -1);
template <class T> void launch_cg_update(const DevParams<T> &P, const DevBufs<T> &B,
                                         cudaGraphConditionalHandle h, bool use_handle, cudaStream_t s,
                                         int phase = -1);
template <class T> void launch_cg_p(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s, int phase = -1);
template <class T> void launch_kick(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
template <class T> void launch_press_init(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
template <class T> void launch_integrate(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
template <class T> void launch_step_begin(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
template <class T> void launch_loop_begin(const DevParams<T> &P, const DevBufs<T> &B, bool div, cudaStream_t s);
template <class T> void launch_boundary_volume(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
template <class T> void launch_features(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s);
// forces of the fluid on the dynamic bodies: phase 0 before the kick (divergence, XSPH and
// viscosity boundary terms), phase 1 after the pressure solve (pressure term)
template <class T> void launch_body_forces(const DevParams<T> &P, const DevBufs<T> &B, const BodyDev &D, int phase,
                                           cudaStream_t s);
// the same for volume-map bodies, from each particle's boundary points
template <class T> void launch_vmap_forces(const DevParams<T> &P, const DevBufs<T> &B, const BodyDev &D, int phase,
                                           cudaStream_t s);
// Learned warm start of one solver: both candidates, their first `sweeps` Jacobi iterations,
// the choice and the loop decision after them (needs 1 <= sweeps <= max_iter of that solver).
template <class T> void launch_warmstart_select(const DevParams<T> &P, const DevBufs<T> &B, bool div, unsigned sweeps,
                                                cudaGraphConditionalHandle h, bool use_handle, cudaStream_t s);
void mlp_infer_device(const float *X, uint32_t n, const void *w, const float *p, float *Y, cudaStream_t s);
// boundary set-up: keys (scene prefix | Morton code) of the boundary particles in upload order
template <class T> void launch_boundary_keys(const DevParams<T> &P, const v4_t<T> *xb_in, const uint32_t *bscene_in,
                                             uint32_t *keys, uint32_t *vals, cudaStream_t s);
template <class T> void launch_boundary_gather(const DevParams<T> &P, const DevBufs<T> &B, const v4_t<T> *xb_in,
                                               const uint32_t *bscene_in, const uint32_t *perm, uint32_t *cells,
                                               cudaStream_t s);
template <class T> void launch_scatter_field(const DevParams<T> &P, const DevBufs<T> &B, int field, void *out,
                                             int out_dtype, cudaStream_t s);
// Fluid fields moved in particle-id order by one launch: field[k] (comps[k] components) to or
// from ptr[k], a buffer in host memory the device maps or in device memory
constexpr uint32_t kFieldSetMax = 8;
constexpr uint32_t kFieldSetMaxComps = 10;   // components of the widest field (network features)
struct FieldSet {
    void *ptr[kFieldSetMax];
    int field[kFieldSetMax];
    uint32_t comps[kFieldSetMax];
    uint32_t n;
};
// the fields of F from slot inv[id], each written as contiguous ranges
template <class T> void launch_gather_fields(const DevParams<T> &P, const DevBufs<T> &B, const FieldSet &F, int odt,
                                             const uint32_t *inv, cudaStream_t s);
// the fields of F (sources in particle-id order) written to slot inv[id], in the order of F
template <class T> void launch_upload_fields(const DevParams<T> &P, const DevBufs<T> &B, const FieldSet &F, int in_dtype,
                                             const uint32_t *inv, cudaStream_t s);
template <class T> void launch_init_state(const DevParams<T> &P, const DevBufs<T> &B, const double *x,
                                          const double *v, const uint32_t *id, cudaStream_t s);
template <class T> void launch_inverse_perm(const DevParams<T> &P, const uint32_t *id, uint32_t *inv, cudaStream_t s);
void launch_lists_to_ids(const uint32_t *list, const uint32_t *cnt, uint32_t cap, const uint32_t *id,
                         const uint32_t *inv, const uint32_t *bid, int kind, uint32_t lpp_log2,
                         const uint32_t *offsets, uint32_t *out, uint32_t n, cudaStream_t s);
void launch_delay(cudaStream_t s, unsigned ns);
void launch_byteswap(void *data, size_t n, int bytes, cudaStream_t s);

// radix sort of (key, value) pairs, LSD, 8-bit digits, stable.  keys/vals are
// ping-ponged with keys2/vals2; returns true if the result ended in keys2/vals2.
// hist holds 256 x (tiles + 1) words, tiles = ceil(n / kSortTile).
bool radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2, uint32_t n,
                      int key_bits, uint32_t *hist, uint32_t num_tiles, cudaStream_t s,
                      unsigned *launch_counter = nullptr);
constexpr uint32_t kSortTile = 2048;   // items per radix-sort tile (256 threads x 8)

}  // namespace sphgb
