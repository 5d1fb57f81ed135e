// C-ABI entry points (include/sphgb300.h) and the host orchestration of one
// TimeStepDFSPH::step() (SPlisHSPlasH/DFSPH/TimeStepDFSPH.cpp:117-249) on the GPU.
//
// The step is a fixed sequence of kernel launches on one stream.  Solver loops
// (divergence, pressure, viscosity CG) decide on the device whether to continue;
// the host either reads that decision after each iteration (use_graph = 0) or
// the whole step is captured once into a CUDA graph whose loops are conditional
// WHILE nodes driven by the kernels (use_graph = 1), so a step is one graph
// launch with no host round trip.
//
// A context holds one scene (the reference's case) or a batch of independent
// scenes.  Scene s owns the fluid slots [pstart_s, pstart_s + n_s) (pstart_s a
// multiple of the block size for batches), its own cell grid inside shared cell
// tables, its own step size and solver decisions; every launch covers all scenes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sphgb300.h"
#include "bgeo.h"
#include "mlp.cuh"
#include "sph_ctx.h"

using namespace sphgb;

namespace sphgb {
void mlp_export(const sphgb_mlp *m, const float **params, const void **w, float scale[2], int *device);
}

namespace {
struct SceneHost {
    uint32_t n = 0, nb = 0;            // fluid / boundary particles
    uint32_t ustart = 0, bstart = 0;   // first fluid / boundary particle in upload order
    uint32_t pstart = 0;               // first fluid slot
    double fmin[3] = {0, 0, 0}, fmax[3] = {0, 0, 0}, bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    double org[3] = {0, 0, 0};         // cell grid
    int dim[3] = {1, 1, 1};
    uint32_t cell_off = 0;
    double dt = 0.001, time = 0.0;     // host copies, valid while no step is pending
    unsigned prev_iters = 0;           // pressure iterations of the last step (CFL method 2)
};
}  // namespace

struct sphgb_ctx {
    sphgb_config cfg{};
    sphgb_params prm{};
    cudaStream_t stream = nullptr;
    cudaStream_t body_stream = nullptr;
    std::string err;
    bool fp64 = false;
    // scenes
    std::vector<SceneHost> scn;
    uint32_t n = 0;                    // fluid particles of all scenes
    uint32_t np = 0;                   // fluid slots (launch size)
    uint32_t nb = 0;                   // boundary particles of all scenes
    std::vector<double> hb;            // boundary positions (host copy, scene order)
    bool have_fluid = false, have_boundary = false, prepared = false;
    // grid
    double cell = 0;
    int key_bits = 0, morton_bits = 0;
    size_t ncell = 0;
    // allocations: per-particle buffers (allocs) and the grid / boundary set-up (prep_allocs)
    std::vector<void *> allocs, prep_allocs;
    void *set_x[2] = {}, *set_v[2] = {}, *set_vdiff[2] = {}, *set_kappa[2] = {}, *set_kappa_v[2] = {};
    float4 *set_xlo[2] = {};
    uint32_t *set_id[2] = {};
    float4 *xa = nullptr;
    void *a = nullptr, *pa = nullptr, *xk = nullptr, *bg = nullptr, *density = nullptr, *factor = nullptr, *dadv = nullptr;
    uint32_t *nfc = nullptr, *nbc = nullptr, *lf = nullptr, *lb = nullptr;
    uint32_t *key = nullptr, *key2 = nullptr, *perm = nullptr, *perm2 = nullptr, *cell0 = nullptr, *cell1 = nullptr;
    uint32_t *cstart = nullptr, *cend = nullptr, *bcstart = nullptr, *bcend = nullptr;
    void *xb = nullptr, *bscratch = nullptr;
    uint32_t *bid = nullptr, *bscene = nullptr;
    void *d_scenes = nullptr;
    uint4 *d_blk = nullptr;
    void *cg[5] = {}, *inv[3] = {};
    double *partials = nullptr;
    unsigned *counters = nullptr;      // [scenes + 1]
    StepScalars *sc = nullptr;         // [scenes + 1]: per-scene records, then the global one
    StepScalars *hsc = nullptr;        // pinned mirror
    size_t hsc_cap = 0;
    uint32_t *hist = nullptr;
    uint32_t *inv_perm = nullptr;
    void *staging = nullptr;
    size_t staging_bytes = 0;
    int parity = 0;
    bool scalars_dirty = true;         // host dt/time changed since the last upload of scalars
    double dt = 0.001;                 // step size given to every scene on upload / set_time_step
    // graphs (one per parity)
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    bool graph_ok = false;
    bool step_pending = false;
    // learned warm start: network copy and per-particle buffers
    bool learned = false, feat_on = false;
    float *mlp_p = nullptr;
    void *mlp_w = nullptr;
    float ws_scale[2] = {kMlpDefaultScaleV, kMlpDefaultScaleP};
    uint32_t ws_gate[2] = {0, 0};      // Jacobi sweeps before the candidates are compared (div, pressure; 0: default)
    // lanes per particle of the neighbour passes: 1 << lpp_log2; chosen by the autotuner unless fixed
    uint32_t lpp_log2 = 2;
    uint32_t lpp_fixed = 0;            // 0: autotune on the first step after an upload
    bool tuned = false;
    // trial step times of lanes per particle 1, 2, 4, of staged passes, and of one lane with
    // 128- and 512-thread solver blocks
    float tune_ms[6] = {0, 0, 0, 0, 0, 0};
    uint32_t solver_nt = 256;          // threads per block of the one-lane unstaged solver passes
    uint32_t nt_fixed = 0;             // 0: the autotuner chooses 128, 256 or 512
    // Bender2019 boundary: volume maps of the bodies (own allocations, kept across uploads)
    struct VMap {
        uint32_t res[3];
        double dmin[3], dmax[3], R[9], t[3];
        double v[3] = {0, 0, 0}, w[3] = {0, 0, 0};   // the body's velocity and angular velocity
        double max_dist = 0;                         // CFL radius: mesh vertices from their mean (0 without a mesh)
        uint32_t scene = 0;                          // the scene of a batch the body belongs to
        double support;                // support radius the map was built for
        double *f0 = nullptr, *f1 = nullptr;   // node fields (FP64)
        void *coef = nullptr;                  // per-cell coefficients in the context's precision
    };
    int boundary_method = 0;           // 0 Akinci2012, 2 Bender2019
    std::vector<VMap> vmaps;
    void *d_vmaps = nullptr;           // VMapDev<T>[vmaps.size()], ordered by scene
    void *d_vmap_range = nullptr;      // batches: uint2 per scene (first map, count)
    void *d_vmap_info = nullptr;       // batches: uint4 per map (body, scene, slot, 0)
    uint32_t vmap_max = 0;             // maps of the scene with the most
    void *bx = nullptr;                // prepared set: [maps][np] boundary points
    void *bv = nullptr;                // prepared set: [np] boundary velocity sums of moving maps
    bool vmove = false;                // some map has a velocity
    bool vmaps_dirty = false;          // poses or velocities changed since the device copy
    // fluid phases (sphgb_set_fluid_phases): particles in id order, count and rest density per phase
    std::vector<uint32_t> phase_counts;
    std::vector<double> phase_rho0;
    std::vector<double> phase_nu, phase_nub;   // Weiler per phase; empty or short: the shared parameters
    std::vector<double> phase_xs, phase_xsb;   // XSPH per phase; likewise
    void *r0 = nullptr;                // prepared set: rest density per slot
    uint32_t *ph = nullptr;            // prepared set: phase per slot
    // moving boundary bodies (sphgb_set_body_motion): particles placed and re-sorted every step
    bool bmotion = false, bmot_dirty = false, bm_ready = false;
    std::vector<double> bmot;          // [nbodies][18]: R (row-major), t, v, w
    uint32_t bm_nb = 0;                // boundary count the buffers below were made for (body allocations)
    void *d_bmot = nullptr, *bm_x0 = nullptr, *bm_V0 = nullptr, *bm_xtmp = nullptr, *bm_vtmp = nullptr;
    void *vbs = nullptr;               // velocities of the sorted boundary particles
    uint32_t *bm_body = nullptr, *bm_scene = nullptr, *bm_k1 = nullptr, *bm_k2 = nullptr, *bm_v1 = nullptr, *bm_v2 = nullptr;
    uint32_t *bm_cells = nullptr, *bm_hist = nullptr;
    uint32_t *binv = nullptr;          // prepared set: sorted slot of boundary particle u
    // neighbourhood staging of the solver passes (FP32, one lane per particle)
    int stage_mode = 0;                // 0: the autotuner decides, 1: off, 2: on
    bool staged = false;               // in use
    uint2 *stage_hdr = nullptr;
    uint32_t *stage_cell = nullptr;
    uint16_t *stage_off = nullptr, *ll = nullptr;
    uint32_t *stage_src = nullptr;
    // particle export: own stream, device and pinned staging, one writer thread
    cudaStream_t export_stream = nullptr;
    cudaEvent_t export_scattered = nullptr, export_copied = nullptr, export_start = nullptr;
    void *export_dev = nullptr, *export_host = nullptr;
    size_t export_dev_bytes = 0, export_host_bytes = 0;
    std::thread export_thread;
    int export_rc = 0;
    std::string export_err;
    float *feat = nullptr, *mlp_x = nullptr, *mlp_y = nullptr;
    void *kl = nullptr, *pa2 = nullptr;
    // dynamic boundary bodies: body of each boundary particle (upload order), reference points and
    // flags on the host; accumulators (own allocations, kept across uploads) and the slot tables
    // (prepared set, rebuilt with the boundary sort)
    std::vector<uint32_t> body_of;
    std::vector<double> body_center;
    std::vector<int> body_dynamic;
    uint32_t nbodies = 0;
    std::vector<void *> body_allocs;
    BodyDev bodies{};
    // per-kernel CUDA-event timing (host-loop mode only)
    bool profile = false;
    std::vector<cudaEvent_t> ev_pool;
    struct Rec { int kid, a, b; };
    std::vector<Rec> recs;
    uint64_t prof_count[32] = {};
    double prof_ms[32] = {};

    uint32_t nscenes() const { return scn.empty() ? 1u : (uint32_t)scn.size(); }
};

namespace {

enum KernelId {
    K_STEP_BEGIN, K_KEYS, K_SORT, K_GATHER, K_CELL_RANGES, K_BUILD, K_LOOP_BEGIN, K_PRESSURE_ACCEL, K_JACOBI,
    K_SOLVER_FINALIZE, K_XSPH, K_VISC_SETUP, K_CG_MATVEC, K_CG_UPDATE, K_CG_P, K_KICK, K_PRESS_INIT, K_INTEGRATE,
    K_FEATURES, K_MLP, K_WS_SELECT, K_BODY_FORCES, K_STAGE_TABLE, K_VMAP_BOUNDARY, K_BOUNDARY_MOVE,
    K_XSPH_VISC_SETUP, K_COUNT
};
const char *kKernelNames[K_COUNT] = {
    "step_begin", "keys", "radix_sort", "gather", "cell_ranges", "build_lists_density_alpha", "loop_begin",
    "pressure_accel", "jacobi_update", "solver_finalize", "xsph_gravity", "visc_setup", "cg_matvec", "cg_update",
    "cg_p", "kick_cfl", "press_init", "integrate", "features", "mlp_infer", "warmstart_select", "body_forces",
    "stage_table", "vmap_boundary", "boundary_move", "xsph_visc_setup",
};

// Brackets the launches of one kernel class with events on the context stream
// when profiling is on.  Events are resolved after the step (no sync per launch).
struct ProfScope {
    sphgb_ctx *c;
    int kid;
    int a = -1;
    ProfScope(sphgb_ctx *c_, int kid_, cudaStream_t s) : c(c_), kid(kid_)
    {
        if (!c->profile) return;
        a = (int)c->recs.size() * 2;
        while ((int)c->ev_pool.size() < a + 2) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            c->ev_pool.push_back(e);
        }
        launch_delay(s, 20000);   // GPU stays busy while the host enqueues event, kernel, event
        cudaEventRecord(c->ev_pool[a], s);
        stream = s;
    }
    ~ProfScope()
    {
        if (!c->profile || a < 0) return;
        cudaEventRecord(c->ev_pool[a + 1], stream);
        c->recs.push_back({kid, a, a + 1});
    }
    cudaStream_t stream = nullptr;
};
#define PROF(kid, s) ProfScope prof_scope_##kid(c, kid, s)

void prof_resolve(sphgb_ctx *c)
{
    if (!c->profile || c->recs.empty()) return;
    cudaEventSynchronize(c->ev_pool[c->recs.back().b]);
    for (const auto &r : c->recs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev_pool[r.a], c->ev_pool[r.b]);
        c->prof_count[r.kid] += 1;
        c->prof_ms[r.kid] += ms;
    }
    c->recs.clear();
}

const sphgb_params kDefaults = {
    0.025, 1000.0, {0.0, -9.81, 0.0}, 1, 0.5, 1e-4, 5e-3, 2, 100, 0.01, 1, 100, 0.1, 0.0, 0.0, 0, 0.01, 0.0, 100, 0.01,
};

int fail(sphgb_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(c, SPHGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
    } while (0)

template <class P> int dalloc_into(sphgb_ctx *c, std::vector<void *> &list, P **p, size_t bytes)
{
    void *q = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return fail(c, SPHGB_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    list.push_back(q);
    *p = static_cast<P *>(q);
    return SPHGB_OK;
}
template <class P> int dalloc(sphgb_ctx *c, P **p, size_t bytes) { return dalloc_into(c, c->allocs, p, bytes); }
template <class P> int palloc(sphgb_ctx *c, P **p, size_t bytes) { return dalloc_into(c, c->prep_allocs, p, bytes); }

// free one allocation of a list (temporaries)
void dfree(std::vector<void *> &list, void *p)
{
    auto it = std::find(list.begin(), list.end(), p);
    if (it != list.end()) list.erase(it);
    cudaFree(p);
}

void invalidate_graphs(sphgb_ctx *c)
{
    for (int k = 0; k < 2; k++)
        if (c->exec[k]) { cudaGraphExecDestroy(c->exec[k]); c->exec[k] = nullptr; }
    c->graph_ok = false;
}

void free_prepared(sphgb_ctx *c)
{
    for (void *p : c->prep_allocs) cudaFree(p);
    c->prep_allocs.clear();
    c->cstart = c->cend = c->bcstart = c->bcend = nullptr;
    c->xb = c->bscratch = nullptr;
    c->bid = c->bscene = nullptr;
    c->binv = nullptr;
    c->r0 = nullptr;
    c->ph = nullptr;
    c->bm_ready = false;   // the rest shapes and volumes are read again from the new layout
    c->bodies.slot = nullptr;
    c->bodies.blk = nullptr;
    c->bodies.body_nblk = nullptr;
    c->bodies.partials = nullptr;
    c->bodies.nblk = 0;
    c->bodies.vpartials = nullptr;
    c->bx = nullptr;
    c->bv = nullptr;
    c->prepared = false;
}

void free_vmaps(sphgb_ctx *c)
{
    for (auto &m : c->vmaps)
        for (void *p : {(void *)m.f0, (void *)m.f1, m.coef})
            if (p) cudaFree(p);
    c->vmaps.clear();
    for (void **p : {&c->d_vmaps, &c->d_vmap_range, &c->d_vmap_info}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    c->vmap_max = 0;
}

// the slot tables of the bodies (part of the prepared set)
void drop_body_tables(sphgb_ctx *c)
{
    for (void *p : {(void *)c->bodies.slot, (void *)c->bodies.blk, (void *)c->bodies.body_nblk,
                    (void *)c->bodies.partials})
        if (p) dfree(c->prep_allocs, p);
    c->bodies.slot = nullptr;
    c->bodies.blk = nullptr;
    c->bodies.body_nblk = nullptr;
    c->bodies.partials = nullptr;
    c->bodies.nblk = 0;
}

void free_bodies(sphgb_ctx *c)
{
    drop_body_tables(c);
    for (void *p : c->body_allocs) cudaFree(p);
    c->body_allocs.clear();
    c->bodies = BodyDev{};
    c->body_of.clear();
    c->body_center.clear();
    c->body_dynamic.clear();
    c->nbodies = 0;
    c->bmotion = c->bmot_dirty = c->bm_ready = false;
    c->bmot.clear();
    c->bm_nb = 0;
    c->d_bmot = c->bm_x0 = c->bm_V0 = c->bm_xtmp = c->bm_vtmp = c->vbs = nullptr;
    c->bm_body = c->bm_scene = c->bm_k1 = c->bm_k2 = c->bm_v1 = c->bm_v2 = c->bm_cells = c->bm_hist = nullptr;
    invalidate_graphs(c);
}

void free_all(sphgb_ctx *c)
{
    if (c->export_stream) cudaStreamSynchronize(c->export_stream);   // an export may still read the state
    free_prepared(c);
    for (void *p : c->allocs) cudaFree(p);
    c->allocs.clear();
    invalidate_graphs(c);
}

size_t real_size(const sphgb_ctx *c) { return c->fp64 ? sizeof(double) : sizeof(float); }
size_t vec_size(const sphgb_ctx *c) { return c->fp64 ? sizeof(dquad) : sizeof(float4); }

template <class T> SceneDev<T> scene_dev(const sphgb_ctx *c, uint32_t s)
{
    SceneDev<T> S{};
    if (c->scn.empty()) {
        S.dimx = S.dimy = S.dimz = 1;
        S.inv_cell = T(1);
        return S;
    }
    const SceneHost &h = c->scn[s];
    S.ox = (T)h.org[0];
    S.oy = (T)h.org[1];
    S.oz = (T)h.org[2];
    S.inv_cell = (T)(c->cell > 0 ? 1.0 / c->cell : 1.0);
    S.dimx = h.dim[0];
    S.dimy = h.dim[1];
    S.dimz = h.dim[2];
    S.cell_off = h.cell_off;
    S.pstart = h.pstart;
    S.n = h.n;
    S.ustart = h.ustart;
    S.key_prefix = c->scn.size() > 1 ? (s << c->morton_bits) : 0u;
    return S;
}

// Weiler2018 coefficients of fluid phase k: sphgb_set_fluid_phase_viscosity's, else the shared ones
double phase_nu(const sphgb_ctx *c, uint32_t k) { return k < c->phase_nu.size() ? c->phase_nu[k] : c->prm.viscosity; }
double phase_nub(const sphgb_ctx *c, uint32_t k)
{
    return k < c->phase_nub.size() ? c->phase_nub[k] : c->prm.viscosity_boundary;
}

template <class T> DevParams<T> make_params(const sphgb_ctx *c)
{
    DevParams<T> P{};
    const sphgb_params &q = c->prm;
    const double h = 4.0 * q.particle_radius;
    P.K.h = (T)h;
    P.K.invh = (T)(1.0 / h);
    P.K.invh2 = (T)(1.0 / (h * h));
    P.K.k = (T)(8.0 / (M_PI * h * h * h));
    P.K.l = (T)(48.0 / (M_PI * h * h * h));
    P.K.w0 = P.K.k;
    P.K.h2 = (T)(h * h);
    const double d = 2.0 * q.particle_radius;
    const double V = 0.8 * d * d * d;
    P.V = (T)V;
    P.mass = (T)(V * q.density0);
    P.rho0 = (T)q.density0;
    P.eps = (T)1.0e-5;
    P.gx = (T)q.gravity[0];
    P.gy = (T)q.gravity[1];
    P.gz = (T)q.gravity[2];
    P.xsph = (T)q.xsph;
    P.xsph_b = (T)q.xsph_boundary;
    P.mu = (T)(q.viscosity * q.density0);
    P.mub = (T)(q.viscosity_boundary * q.density0);
    P.vd = (T)10.0;
    P.h2 = (T)(h * h);
    P.max_error = q.max_error;
    P.max_error_v = q.max_error_v;
    P.cfl_factor = q.cfl_factor;
    P.cfl_min = q.cfl_min_time_step;
    P.cfl_max = q.cfl_max_time_step;
    P.radius = q.particle_radius;
    P.visc_tol = q.visco_max_error;
    P.min_iter = q.min_iterations;
    P.max_iter = q.max_iterations;
    P.max_iter_v = q.max_iterations_v;
    P.visc_max_iter = q.visco_max_iter;
    P.cfl_method = q.cfl_method;
    P.visc_on = q.viscosity_method == 6 ? 1 : 0;
    P.div_on = q.enable_divergence_solver ? 1 : 0;
    P.learned = c->learned ? 1 : 0;
    P.feat_on = (c->learned || c->feat_on) ? 1 : 0;
    P.ws_scale_v = c->ws_scale[0];
    P.ws_scale_p = c->ws_scale[1];
    P.nscenes = c->nscenes();
    P.s0 = scene_dev<T>(c, 0);
    P.scenes = P.nscenes > 1 ? static_cast<const SceneDev<T> *>(c->d_scenes) : nullptr;
    P.blk = P.nscenes > 1 ? c->d_blk : nullptr;
    P.np = c->np;
    P.nreal = c->n;
    P.nb = c->nb;
    P.capf = c->cfg.max_fluid_neighbors;
    P.capb = c->cfg.max_boundary_neighbors;
    P.lpp_log2 = c->lpp_log2;
    P.solver_nt = c->solver_nt;
    P.staged = (c->staged && !c->fp64 && c->lpp_log2 == 0 && c->ll) ? 1 : 0;
    P.nvmaps = (c->boundary_method == 2 && c->bx) ? (uint32_t)c->vmaps.size() : 0u;
    P.vmaps = static_cast<const VMapDev<T> *>(c->d_vmaps);
    P.vmap_range = static_cast<const uint2 *>(c->d_vmap_range);
    P.vmap_info = static_cast<const uint4 *>(c->d_vmap_info);
    P.vmap_max = P.nvmaps ? c->vmap_max : 0u;
    P.vmove = (P.nvmaps && c->vmove && c->bv) ? 1 : 0;
    P.bmove = (c->bmotion && c->bm_ready && c->nb && c->boundary_method == 0 && c->bv) ? 1 : 0;
    P.nphase = 1;
    if (c->phase_counts.size() > 1 && c->r0) {
        P.nphase = (uint32_t)c->phase_counts.size();
        // the step-wide XSPH and boundary-viscosity switches follow the phases' own coefficients
        // (which fall back to the shared ones where a phase sets none): any non-zero one
        P.xsph = P.xsph_b = P.mub = T(0);
        uint32_t end = 0;
        for (uint32_t k = 0; k < 8; k++) {
            const bool has = k < P.nphase;
            P.phase_count[k] = has ? c->phase_counts[k] : 0u;
            end += P.phase_count[k];
            P.phase_end[k] = end;
            P.phase_rho0[k] = has ? (T)c->phase_rho0[k] : P.rho0;
            P.phase_nu[k] = (T)phase_nu(c, k);
            P.phase_nub[k] = (T)phase_nub(c, k);
            P.phase_xs[k] = (T)(k < c->phase_xs.size() ? c->phase_xs[k] : q.xsph);
            P.phase_xsb[k] = (T)(k < c->phase_xsb.size() ? c->phase_xsb[k] : q.xsph_boundary);
            if (has && P.xsph == T(0)) P.xsph = P.phase_xs[k];
            if (has && P.xsph_b == T(0)) P.xsph_b = P.phase_xsb[k];
            if (has && P.mub == T(0)) P.mub = (T)(phase_nub(c, k) * c->phase_rho0[k]);
        }
        P.staged = 0;   // the staged passes read one rest density
    }
    return P;
}

// view 0: x = state set of the previous step (sort source), x2 = gather target
// view 1: x = the gathered set (working set of this step)
template <class T> DevBufs<T> make_bufs(const sphgb_ctx *c, int view)
{
    using v4 = v4_t<T>;
    DevBufs<T> B{};
    const int cur = view == 0 ? c->parity : 1 - c->parity;
    const int alt = 1 - cur;
    B.x = (v4 *)c->set_x[cur];
    B.v = (v4 *)c->set_v[cur];
    B.vdiff = (v4 *)c->set_vdiff[cur];
    B.xlo = c->set_xlo[cur];
    B.kappa = (T *)c->set_kappa[cur];
    B.kappa_v = (T *)c->set_kappa_v[cur];
    B.id = c->set_id[cur];
    B.x2 = (v4 *)c->set_x[alt];
    B.v2 = (v4 *)c->set_v[alt];
    B.vdiff2 = (v4 *)c->set_vdiff[alt];
    B.xlo2 = c->set_xlo[alt];
    B.kappa2 = (T *)c->set_kappa[alt];
    B.kappa_v2 = (T *)c->set_kappa_v[alt];
    B.id2 = c->set_id[alt];
    B.a = (v4 *)c->a;
    B.pa = (v4 *)c->pa;
    B.xa = c->xa;
    B.xk = (v4 *)c->xk;
    B.bg = (v4 *)c->bg;
    B.density = (T *)c->density;
    B.factor = (T *)c->factor;
    B.dadv = (T *)c->dadv;
    B.nf = c->nfc;
    B.nbn = c->nbc;
    B.lf = c->lf;
    B.lb = c->lb;
    B.stage_hdr = c->stage_hdr;
    B.stage_cell = c->stage_cell;
    B.stage_off = c->stage_off;
    B.stage_src = c->stage_src;
    B.bx = (v4 *)c->bx;
    B.bv = (v4 *)c->bv;
    B.vbs = (v4 *)c->vbs;
    B.binv = c->binv;
    B.r0 = (T *)c->r0;
    B.ph = c->ph;
    B.ll = c->ll;
    B.key = c->key;
    B.key2 = c->key2;
    B.perm = c->perm;
    B.perm2 = c->perm2;
    B.cellid = view == 0 ? c->cell0 : c->cell1;
    B.cellid2 = c->cell1;
    B.cstart = c->cstart;
    B.cend = c->cend;
    B.bcstart = c->bcstart;
    B.bcend = c->bcend;
    B.xb = (v4 *)c->xb;
    B.bscratch = (T *)c->bscratch;
    B.bid = c->bid;
    B.bscene = c->bscene;
    B.feat = c->feat;
    B.mlp_x = c->mlp_x;
    B.mlp_y = c->mlp_y;
    B.kl = (T *)c->kl;
    B.pa2 = (v4 *)c->pa2;
    B.mlp_w = c->mlp_w;
    B.mlp_p = c->mlp_p;
    B.cg_x = (v4 *)c->cg[0];
    B.cg_r = (v4 *)c->cg[1];
    B.cg_p = (v4 *)c->cg[2];
    B.cg_z = (v4 *)c->cg[3];
    B.cg_t = (v4 *)c->cg[4];
    B.inv0 = (v4 *)c->inv[0];
    B.inv1 = (v4 *)c->inv[1];
    B.partials = c->partials;
    B.counters = c->counters;
    B.sc = c->sc;
    B.gsc = c->sc ? c->sc + c->nscenes() : nullptr;
    B.hist = c->hist;
    return B;
}

template <class T> int upload_scene_table(sphgb_ctx *c)
{
    if (c->scn.size() <= 1) return SPHGB_OK;
    std::vector<SceneDev<T>> t(c->scn.size());
    for (uint32_t s = 0; s < c->scn.size(); s++) t[s] = scene_dev<T>(c, s);
    CK(cudaMemcpy(c->d_scenes, t.data(), t.size() * sizeof(SceneDev<T>), cudaMemcpyHostToDevice));
    return SPHGB_OK;
}

int upload_scalars(sphgb_ctx *c)
{
    if (!c->scalars_dirty) return SPHGB_OK;
    const uint32_t S = c->nscenes();
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(c->hsc, c->sc, (S + 1) * sizeof(StepScalars), cudaMemcpyDeviceToHost));
    for (uint32_t s = 0; s < S; s++) {
        const double dt = c->scn.empty() ? c->dt : c->scn[s].dt;
        const double t = c->scn.empty() ? 0.0 : c->scn[s].time;
        c->hsc[s].dt = dt;
        c->hsc[s].dt_next = dt;
        c->hsc[s].time = t;
        c->hsc[s].prev_iters = c->scn.empty() ? 0u : c->scn[s].prev_iters;
    }
    CK(cudaMemcpy(c->sc, c->hsc, (S + 1) * sizeof(StepScalars), cudaMemcpyHostToDevice));
    c->scalars_dirty = false;
    return SPHGB_OK;
}

int bits_for(size_t v)
{
    int b = 0;
    while (((size_t)1 << b) < v) b++;
    return b;
}

// Slot tables of the dynamic bodies after the boundary sort: the sorted boundary slots whose
// particle belongs to a dynamic body, grouped by body (counting sort, slot order kept within a
// body), and the block table of the force gather (blocks of kBlock entries, never two bodies).
int build_body_tables(sphgb_ctx *c)
{
    c->bodies.nblk = 0;
    if (c->nbodies == 0 || c->nb == 0) return SPHGB_OK;
    // each dynamic body's particles in upload order; the kernel finds their sorted slots through
    // binv, so the tables hold when moving bodies are re-sorted every step
    const uint32_t B = c->nbodies;
    std::vector<uint32_t> count(B + 1, 0);
    for (uint32_t u = 0; u < c->nb; u++) {
        const uint32_t b = c->body_of[u];
        if (c->body_dynamic[b]) count[b + 1]++;
    }
    for (uint32_t b = 0; b < B; b++) count[b + 1] += count[b];
    const uint32_t entries = count[B];
    if (entries == 0) return SPHGB_OK;
    std::vector<uint32_t> slot(entries), fill(count.begin(), count.end() - 1);
    for (uint32_t u = 0; u < c->nb; u++) {
        const uint32_t b = c->body_of[u];
        if (c->body_dynamic[b]) slot[fill[b]++] = u;
    }
    std::vector<uint4> blk;
    std::vector<uint32_t> nblk(B, 0);
    for (uint32_t b = 0; b < B; b++) {
        const uint32_t first = (uint32_t)blk.size();
        for (uint32_t e = count[b]; e < count[b + 1]; e += kBlock)
            blk.push_back(make_uint4(b, e, std::min(e + (uint32_t)kBlock, count[b + 1]), first));
        nblk[b] = (uint32_t)blk.size() - first;
    }
    uint32_t *d_slot, *d_nblk;
    uint4 *d_blk;
    double *d_part;
    int rc;
    if ((rc = palloc(c, &d_slot, (size_t)entries * 4))) return rc;
    if ((rc = palloc(c, &d_blk, blk.size() * sizeof(uint4)))) return rc;
    if ((rc = palloc(c, &d_nblk, (size_t)B * 4))) return rc;
    if ((rc = palloc(c, &d_part, blk.size() * 6 * sizeof(double)))) return rc;
    CK(cudaMemcpy(d_slot, slot.data(), (size_t)entries * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_blk, blk.data(), blk.size() * sizeof(uint4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_nblk, nblk.data(), (size_t)B * 4, cudaMemcpyHostToDevice));
    c->bodies.slot = d_slot;
    c->bodies.blk = d_blk;
    c->bodies.body_nblk = d_nblk;
    c->bodies.partials = d_part;
    c->bodies.nblk = (uint32_t)blk.size();
    return SPHGB_OK;
}

template <class T> int upload_vmaps(sphgb_ctx *c);

// Build each scene's cell grid over the union of its fluid and boundary extents,
// sort the boundary particles into it and compute their Akinci2012 volumes.
template <class T> int prepare(sphgb_ctx *c)
{
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    free_prepared(c);
    invalidate_graphs(c);
    const double h = 4.0 * c->prm.particle_radius;
    // slightly larger than the support radius: keeps |dx| < h => |cell delta| <= 1 under float rounding
    c->cell = h * 1.001;
    size_t off = 0;
    int maxdim = 1;
    for (SceneHost &S : c->scn) {
        size_t nc = 1;
        for (int d = 0; d < 3; d++) {
            double lo = S.fmin[d], hi = S.fmax[d];
            if (S.nb > 0) {
                lo = std::min(lo, S.bmin[d]);
                hi = std::max(hi, S.bmax[d]);
            }
            S.org[d] = lo - c->cell;
            const double ext = hi - S.org[d];
            const double nd = std::floor(ext / c->cell) + 2;
            if (!(nd <= 1024.0)) return fail(c, SPHGB_ERR_GRID, "scene extent exceeds 1024 cells per axis");
            S.dim[d] = (int)nd;
            maxdim = std::max(maxdim, S.dim[d]);
            nc *= (size_t)S.dim[d];
        }
        S.cell_off = (uint32_t)off;
        off += nc;
        if (off >= 0xffffffffull) return fail(c, SPHGB_ERR_GRID, "more than 2^32 cells in the scenes' grids");
    }
    c->ncell = std::max<size_t>(off, 1);
    c->morton_bits = 3 * std::max(1, bits_for((size_t)maxdim));
    const int scene_bits = c->scn.size() > 1 ? bits_for(c->scn.size()) : 0;
    c->key_bits = c->morton_bits + scene_bits;
    if (c->key_bits > 32)
        return fail(c, SPHGB_ERR_GRID, "scene count and grid size need more than 32 sort-key bits");
    int rc;
    if ((rc = palloc(c, &c->cstart, c->ncell * 4))) return rc;
    if ((rc = palloc(c, &c->cend, c->ncell * 4))) return rc;
    if ((rc = palloc(c, &c->bcstart, c->ncell * 4))) return rc;
    if ((rc = palloc(c, &c->bcend, c->ncell * 4))) return rc;
    CK(cudaMemsetAsync(c->bcstart, 0xff, c->ncell * 4, c->stream));
    if ((rc = upload_scene_table<T>(c))) return rc;
    const uint32_t nb = c->nb;
    if ((rc = palloc(c, &c->xb, (size_t)std::max(nb, 1u) * vec_size(c)))) return rc;
    if ((rc = palloc(c, &c->bid, (size_t)std::max(nb, 1u) * 4))) return rc;
    if ((rc = palloc(c, &c->binv, (size_t)std::max(nb, 1u) * 4))) return rc;
    if ((rc = palloc(c, &c->bscratch, (size_t)std::max(nb, 1u) * real_size(c)))) return rc;
    if (c->scn.size() > 1 && (rc = palloc(c, &c->bscene, (size_t)std::max(nb, 1u) * 4))) return rc;
    if (nb > 0) {
        // upload-order boundary positions (and scenes), sorted by (scene, cell Morton code)
        std::vector<char> host((size_t)nb * vec_size(c));
        for (uint32_t i = 0; i < nb; i++) {
            const double *p = c->hb.data() + 3 * (size_t)i;
            if (c->fp64) {
                dquad q{p[0], p[1], p[2], 0.0};
                std::memcpy(host.data() + (size_t)i * sizeof(dquad), &q, sizeof(q));
            } else {
                float4 q = make_float4((float)p[0], (float)p[1], (float)p[2], 0.f);
                std::memcpy(host.data() + (size_t)i * sizeof(float4), &q, sizeof(q));
            }
        }
        void *xb_raw;
        uint32_t *bscene_raw = nullptr, *k1, *k2, *v1, *v2, *cells, *hist;
        if ((rc = palloc(c, &xb_raw, host.size()))) return rc;
        CK(cudaMemcpy(xb_raw, host.data(), host.size(), cudaMemcpyHostToDevice));
        if (c->scn.size() > 1) {
            std::vector<uint32_t> bs(nb);
            for (uint32_t s = 0; s < c->scn.size(); s++)
                for (uint32_t k = 0; k < c->scn[s].nb; k++) bs[c->scn[s].bstart + k] = s;
            if ((rc = palloc(c, &bscene_raw, (size_t)nb * 4))) return rc;
            CK(cudaMemcpy(bscene_raw, bs.data(), (size_t)nb * 4, cudaMemcpyHostToDevice));
        }
        const uint32_t tiles = (nb + kSortTile - 1) / kSortTile;
        if ((rc = palloc(c, &k1, (size_t)nb * 4))) return rc;
        if ((rc = palloc(c, &k2, (size_t)nb * 4))) return rc;
        if ((rc = palloc(c, &v1, (size_t)nb * 4))) return rc;
        if ((rc = palloc(c, &v2, (size_t)nb * 4))) return rc;
        if ((rc = palloc(c, &cells, (size_t)nb * 4))) return rc;
        if ((rc = palloc(c, &hist, (size_t)(tiles + 1) * 256 * 4))) return rc;
        const DevParams<T> P = make_params<T>(c);
        const DevBufs<T> B = make_bufs<T>(c, 1);
        launch_boundary_keys<T>(P, (const v4_t<T> *)xb_raw, bscene_raw, k1, v1, c->stream);
        const bool sw = radix_sort_pairs(k1, v1, k2, v2, nb, c->key_bits, hist, tiles, c->stream);
        launch_boundary_gather<T>(P, B, (const v4_t<T> *)xb_raw, bscene_raw, sw ? v2 : v1, cells, c->stream);
        launch_boundary_volume<T>(P, B, c->stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
        for (void *p : {(void *)xb_raw, (void *)bscene_raw, (void *)k1, (void *)k2, (void *)v1, (void *)v2,
                        (void *)cells, (void *)hist})
            if (p) dfree(c->prep_allocs, p);
    }
    if ((rc = build_body_tables(c))) return rc;
    if (c->phase_counts.size() > 1) {   // fluid phases: rest density and phase per slot (set by the gather)
        if ((rc = palloc(c, &c->r0, (size_t)std::max(c->np, 1u) * real_size(c)))) return rc;
        if ((rc = palloc(c, &c->ph, (size_t)std::max(c->np, 1u) * 4))) return rc;
    }
    if (c->boundary_method == 0 && c->nb) {   // boundary velocity sums of moving bodies
        if ((rc = palloc(c, &c->bv, (size_t)std::max(c->np, 1u) * vec_size(c)))) return rc;
    }
    if (c->boundary_method == 2 && !c->vmaps.empty()) {
        // the maps for the current scenes; each particle keeps one boundary point per map of its scene
        if ((rc = c->fp64 ? upload_vmaps<double>(c) : upload_vmaps<float>(c))) return rc;
        if ((rc = palloc(c, &c->bx, (size_t)std::max(c->np, 1u) * c->vmap_max * vec_size(c)))) return rc;
        if ((rc = palloc(c, &c->bv, (size_t)std::max(c->np, 1u) * vec_size(c)))) return rc;
        if (c->nbodies) {   // block partials of the volume-map body forces
            const size_t nblk = (std::max(c->np, 1u) + kBlock - 1) / kBlock;
            if ((rc = palloc(c, &c->bodies.vpartials, (size_t)c->vmap_max * 6 * nblk * sizeof(double)))) return rc;
        }
    }
    c->prepared = true;
    return SPHGB_OK;
}

// Gate of the learned warm start: both candidates run this many Jacobi iterations of the
// solver before they are compared.  Default: 1 for the divergence solve (the candidates'
// initial residuals) and max(minIterations, 4) for the pressure solve: the first sweeps damp
// the particle-scale error of a warm start, after four the errors compared reflect the
// low-frequency error that decides the iteration count.  Never more than the solver's maximum.
constexpr unsigned kDefaultPressureGate = 4;
unsigned gate_sweeps(const sphgb_ctx *c, bool div)
{
    const unsigned max_iter = div ? c->prm.max_iterations_v : c->prm.max_iterations;
    const uint32_t set = c->ws_gate[div ? 0 : 1];
    const unsigned g = set ? set : (div ? 1u : std::max(kDefaultPressureGate, c->prm.min_iterations));
    return std::min(g, max_iter);
}

template <class T> void enqueue_solver_loop_body(sphgb_ctx *c, const DevParams<T> &P, const DevBufs<T> &B, bool div,
                                                 cudaGraphConditionalHandle h, bool use_handle, cudaStream_t s)
{
    // one iteration: with fluid phases, both passes for each phase in turn (TimeStepDFSPH.cpp:322-339)
    const int nph = P.nphase > 1 ? (int)P.nphase : 1;
    for (int k = 0; k < nph; k++) {
        const int phase = P.nphase > 1 ? k : -1;
        {
            PROF(K_PRESSURE_ACCEL, s);
            launch_pressure_accel<T>(P, B, div, phase, s, h, use_handle);
        }
        {
            PROF(K_JACOBI, s);
            launch_jacobi<T>(P, B, div, phase, h, use_handle, s);
        }
    }
}

// the batch's loop decision (global record)
int read_cont(sphgb_ctx *c, unsigned *cont)
{
    StepScalars *g = c->sc + c->nscenes();
    StepScalars *hg = c->hsc + c->nscenes();
    CK(cudaMemcpyAsync(&hg->cont, &g->cont, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *cont = hg->cont;
    return SPHGB_OK;
}

// The body-force gather before the kick has terms to collect: the divergence solve's pressure,
// the XSPH boundary term or the Weiler2018 boundary term.
template <class T> bool body_phase0(const sphgb_ctx *c, const DevParams<T> &P)
{
    const bool bodies = c->bodies.nblk || (P.nvmaps && c->bodies.nbodies && c->bodies.vpartials);
    return bodies && (P.div_on || P.xsph_b != T(0) || (P.visc_on && P.mub != T(0)));
}

template <class T> BoundaryMoveDev<T> boundary_move_dev(const sphgb_ctx *c)
{
    BoundaryMoveDev<T> M;
    M.x0 = static_cast<const v4_t<T> *>(c->bm_x0);
    M.V0 = static_cast<const T *>(c->bm_V0);
    M.body = c->bm_body;
    M.scene = c->nscenes() > 1 ? c->bm_scene : nullptr;
    M.motion = static_cast<const BodyMotionDev<T> *>(c->d_bmot);
    M.xtmp = static_cast<v4_t<T> *>(c->bm_xtmp);
    M.vtmp = static_cast<v4_t<T> *>(c->bm_vtmp);
    return M;
}

// Enqueue the launches that precede the solver loops.
// Weiler2018 with fluid phases: one system per phase in phase order (the reference's viscosity is a
// per-model force, Viscosity_Weiler2018.cpp:891-936 run for each FluidModel); phase k's system
// takes mub = nu_b rho0 and rho0 of that phase in its boundary terms.  -1: one system over all.
template <class T> int visc_systems(const DevParams<T> &P) { return P.nphase > 1 ? (int)P.nphase : 1; }
// one fluid phase with viscosity: the XSPH pass runs fused into the viscosity set-up pass
template <class T> bool fused_xsph_visc(const DevParams<T> &P) { return P.visc_on && P.nphase <= 1; }
template <class T> DevParams<T> visc_system_params(const sphgb_ctx *c, const DevParams<T> &P, int k, int &phase)
{
    phase = P.nphase > 1 ? k : -1;
    if (phase < 0) return P;
    DevParams<T> Q = P;
    Q.mub = (T)(phase_nub(c, k) * c->phase_rho0[k]);
    Q.rho0 = (T)c->phase_rho0[k];
    return Q;
}

template <class T> void enqueue_prologue(sphgb_ctx *c, const DevParams<T> &P, const DevBufs<T> &B0, const DevBufs<T> &B1,
                                         cudaStream_t s)
{
    { PROF(K_STEP_BEGIN, s); launch_step_begin<T>(P, B1, s); }
    if (P.bmove) {   // moving bodies: place, sort and bin the boundary particles (after the CFL reset)
        PROF(K_BOUNDARY_MOVE, s);
        const BoundaryMoveDev<T> M = boundary_move_dev<T>(c);
        launch_boundary_move<T>(P, B1, M, c->bm_k1, c->bm_v1, s);
        const uint32_t btiles = (c->nb + kSortTile - 1) / kSortTile;
        const bool bsw = radix_sort_pairs(c->bm_k1, c->bm_v1, c->bm_k2, c->bm_v2, c->nb, c->key_bits, c->bm_hist,
                                          btiles, s, &B1.gsc->launches);
        cudaMemsetAsync(c->bcstart, 0xff, c->ncell * 4, s);
        launch_boundary_regather<T>(P, B1, M, bsw ? c->bm_v2 : c->bm_v1, c->bm_cells, s);
    }
    { PROF(K_KEYS, s); launch_keys<T>(P, B0, s); }
    const uint32_t tiles = (c->n + kSortTile - 1) / kSortTile;
    bool sw;
    {
        PROF(K_SORT, s);
        sw = radix_sort_pairs(c->key, c->perm, c->key2, c->perm2, c->n, c->key_bits, c->hist, tiles, s, &B1.gsc->launches);
    }
    { PROF(K_GATHER, s); launch_gather<T>(P, B0, sw ? c->perm2 : c->perm, s); }
    {
        PROF(K_CELL_RANGES, s);
        cudaMemsetAsync(c->cstart, 0xff, c->ncell * 4, s);
        launch_cell_ranges<T>(P, B1, s);
    }
    if (P.nvmaps) { PROF(K_VMAP_BOUNDARY, s); launch_vmap_boundary<T>(P, B1, s); }
    if (P.staged) { PROF(K_STAGE_TABLE, s); launch_stage_table<T>(P, B1, s); }
    { PROF(K_BUILD, s); launch_build<T>(P, B1, s); }
    if (P.feat_on) { PROF(K_FEATURES, s); launch_features<T>(P, B1, s); }
    if (P.learned) { PROF(K_MLP, s); mlp_infer_device(c->mlp_x, c->np, c->mlp_w, c->mlp_p, c->mlp_y, s); }
}

template <class T> int step_host_loop(sphgb_ctx *c)
{
    const DevParams<T> P = make_params<T>(c);
    const DevBufs<T> B0 = make_bufs<T>(c, 0);
    const DevBufs<T> B1 = make_bufs<T>(c, 1);
    cudaStream_t s = c->stream;
    int rc;
    unsigned cont = 0;
    enqueue_prologue<T>(c, P, B0, B1, s);
    // one solver loop: with the network, the warm-start selection is iteration 1
    auto solve = [&](bool div) -> int {
        const unsigned max_iter = div ? P.max_iter_v : P.max_iter;
        { PROF(K_LOOP_BEGIN, s); launch_loop_begin<T>(P, B1, div, s); }
        unsigned guard = 0, cont = 0;
        int r;
        if (max_iter > 0 && P.learned) {
            const unsigned g = gate_sweeps(c, div);
            guard = g - 1;
            { PROF(K_WS_SELECT, s); launch_warmstart_select<T>(P, B1, div, g, 0, false, s); }
            if ((r = read_cont(c, &cont))) return r;
            while (cont && ++guard <= max_iter) {
                enqueue_solver_loop_body<T>(c, P, B1, div, 0, false, s);
                if ((r = read_cont(c, &cont))) return r;
            }
        } else if (max_iter > 0) {
            do {
                enqueue_solver_loop_body<T>(c, P, B1, div, 0, false, s);
                if ((r = read_cont(c, &cont))) return r;
            } while (cont && ++guard <= max_iter);
        }
        { PROF(K_SOLVER_FINALIZE, s); launch_solver_finalize<T>(P, B1, div, s); }
        return SPHGB_OK;
    };
    if (P.div_on && (rc = solve(true))) return rc;
    const bool fused = fused_xsph_visc(P);
    if (!fused) { PROF(K_XSPH, s); launch_xsph<T>(P, B1, s); }
    if (P.visc_on) {
        for (int k = 0; k < visc_systems(P); k++) {
            int ph;
            const DevParams<T> Q = visc_system_params(c, P, k, ph);
            if (fused) { PROF(K_XSPH_VISC_SETUP, s); launch_xsph_visc_setup<T>(Q, B1, 0, false, s); }
            else { PROF(K_VISC_SETUP, s); launch_visc_setup<T>(Q, B1, 0, false, s, ph); }
            if ((rc = read_cont(c, &cont))) return rc;
            unsigned guard = 0;
            while (cont && guard++ <= P.visc_max_iter) {
                { PROF(K_CG_MATVEC, s); launch_cg_matvec<T>(Q, B1, s, 0, false, ph); }
                { PROF(K_CG_UPDATE, s); launch_cg_update<T>(Q, B1, 0, false, s, ph); }
                if ((rc = read_cont(c, &cont))) return rc;
                if (!cont) break;
                { PROF(K_CG_P, s); launch_cg_p<T>(Q, B1, s, ph); }
            }
        }
    }
    if (body_phase0(c, P)) {
        PROF(K_BODY_FORCES, s);
        launch_body_forces<T>(P, B1, c->bodies, 0, s);
        launch_vmap_forces<T>(P, B1, c->bodies, 0, s);
    }
    { PROF(K_KICK, s); launch_kick<T>(P, B1, s); }
    { PROF(K_PRESS_INIT, s); launch_press_init<T>(P, B1, s); }
    if ((rc = solve(false))) return rc;
    {
        PROF(K_BODY_FORCES, s);
        launch_body_forces<T>(P, B1, c->bodies, 1, s);
        launch_vmap_forces<T>(P, B1, c->bodies, 1, s);
    }
    { PROF(K_INTEGRATE, s); launch_integrate<T>(P, B1, s); }
    CK(cudaGetLastError());
    prof_resolve(c);
    return SPHGB_OK;
}

// --- graph capture with conditional WHILE nodes ----------------------------
// A loop-condition handle of the graph being captured on c->stream, reset to
// default_value at every launch of the graph (kernels before the loop may set it).
cudaError_t make_handle(sphgb_ctx *c, cudaGraphConditionalHandle *h, unsigned default_value)
{
    cudaStreamCaptureStatus st;
    cudaGraph_t g;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return e;
    return cudaGraphConditionalHandleCreate(h, g, default_value, cudaGraphCondAssignDefault);
}

// Adds a WHILE node on handle h after the current capture tail of c->stream and
// captures body(stream, h) into it on the body stream.
template <class F> cudaError_t add_while_node(sphgb_ctx *c, cudaGraphConditionalHandle h, F body)
{
    cudaStreamCaptureStatus st;
    cudaGraph_t g;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np);
    if (e != cudaSuccess) return e;
    e = cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(c->body_stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return e;
    body(c->body_stream, h);
    return cudaStreamEndCapture(c->body_stream, &bodyg);
}

// The whole step (prologue, loops, epilogue) captured for one parity.  Kernels
// that decide a loop's first condition (the viscosity set-up, the learned
// warm-start selection) are captured after the loop's handle exists.
template <class T> int build_graph(sphgb_ctx *c, int parity, cudaGraphExec_t *out)
{
    const int saved = c->parity;
    c->parity = parity;
    const DevParams<T> P = make_params<T>(c);
    const DevBufs<T> B0 = make_bufs<T>(c, 0);
    const DevBufs<T> B1 = make_bufs<T>(c, 1);
    c->parity = saved;
    cudaStream_t s = c->stream;
    const bool prof_saved = c->profile;
    c->profile = false;   // no event records inside the captured graph
    struct Restore { sphgb_ctx *c; bool v; ~Restore() { c->profile = v; } } restore{c, prof_saved};
    cudaGraph_t graph = nullptr;
    CK(cudaGraphCreate(&graph, 0));
    cudaError_t e = cudaStreamBeginCaptureToGraph(s, graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { cudaGraphDestroy(graph); return fail(c, SPHGB_ERR_CUDA, cudaGetErrorString(e)); }
    enqueue_prologue<T>(c, P, B0, B1, s);
    // one solver loop; with the network the warm-start selection (iteration 1) sets the condition
    auto solve = [&](bool div) {
        const unsigned max_iter = div ? P.max_iter_v : P.max_iter;
        launch_loop_begin<T>(P, B1, div, s);
        cudaGraphConditionalHandle h = 0;
        const bool sel = max_iter > 0 && P.learned;
        if (e == cudaSuccess) e = make_handle(c, &h, (!sel && max_iter > 0) ? 1u : 0u);
        if (e == cudaSuccess && sel) launch_warmstart_select<T>(P, B1, div, gate_sweeps(c, div), h, true, s);
        if (e == cudaSuccess)
            e = add_while_node(c, h, [&](cudaStream_t bs, cudaGraphConditionalHandle hh) {
                enqueue_solver_loop_body<T>(c, P, B1, div, hh, true, bs);
            });
        launch_solver_finalize<T>(P, B1, div, s);
    };
    if (P.div_on) solve(true);
    const bool fused = fused_xsph_visc(P);
    if (!fused) launch_xsph<T>(P, B1, s);
    for (int k = 0; P.visc_on && e == cudaSuccess && k < visc_systems(P); k++) {
        // the set-up kernel sets the CG loop's condition; one loop per system
        int ph;
        const DevParams<T> Q = visc_system_params(c, P, k, ph);
        cudaGraphConditionalHandle hcg = 0;
        e = make_handle(c, &hcg, 0u);
        if (e == cudaSuccess) {
            if (fused) launch_xsph_visc_setup<T>(Q, B1, hcg, true, s);
            else launch_visc_setup<T>(Q, B1, hcg, true, s, ph);
            e = add_while_node(c, hcg, [&](cudaStream_t bs, cudaGraphConditionalHandle hh) {
                launch_cg_matvec<T>(Q, B1, bs, hh, true, ph);
                launch_cg_update<T>(Q, B1, hh, true, bs, ph);
                launch_cg_p<T>(Q, B1, bs, ph);
            });
        }
    }
    if (body_phase0(c, P)) {
        launch_body_forces<T>(P, B1, c->bodies, 0, s);
        launch_vmap_forces<T>(P, B1, c->bodies, 0, s);
    }
    launch_kick<T>(P, B1, s);
    launch_press_init<T>(P, B1, s);
    solve(false);
    launch_body_forces<T>(P, B1, c->bodies, 1, s);
    launch_vmap_forces<T>(P, B1, c->bodies, 1, s);
    launch_integrate<T>(P, B1, s);
    cudaGraph_t done = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(s, &done);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, SPHGB_ERR_CUDA, std::string("graph build: ") + cudaGetErrorString(e));
    }
    return SPHGB_OK;
}

// Lanes per particle of the neighbour passes (and with it the fluid-list layout), chosen by
// timing one trial step per candidate (1, 2 and 4 lanes, twice each, the faster of the two
// kept) from the current state.  A step never writes the state set it starts from (it
// gathers into the other set), so a trial is undone by restoring the step scalars.
// staged solver passes: FP32 and not switched off
bool staging_possible(const sphgb_ctx *c) { return !c->fp64 && c->stage_mode != 1 && c->ll != nullptr; }

template <class T> int autotune(sphgb_ctx *c)
{
    const uint32_t S = c->nscenes();
    std::vector<StepScalars> saved(S + 1);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(saved.data(), c->sc, (S + 1) * sizeof(StepScalars), cudaMemcpyDeviceToHost));
    // the trial steps also add to the body accumulators, and leave their pressure accelerations,
    // which the next step carries over for fluid phases
    std::vector<double> saved_acc(6 * (size_t)c->nbodies);
    if (c->nbodies)
        CK(cudaMemcpy(saved_acc.data(), c->bodies.acc, saved_acc.size() * sizeof(double), cudaMemcpyDeviceToHost));
    const size_t pa_bytes = (size_t)std::max(c->np, 1u) * sizeof(v4_t<T>);
    void *saved_pa = nullptr;
    if (c->phase_counts.size() > 1) {
        CK(cudaMalloc(&saved_pa, pa_bytes));
        CK(cudaMemcpy(saved_pa, c->pa, pa_bytes, cudaMemcpyDeviceToDevice));
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const bool prof = c->profile;
    c->profile = false;
    // candidates 0..2: 1, 2, 4 lanes per particle; 3: one lane with staged solver passes; 4, 5:
    // one lane with 128- and 512-thread blocks in the solver passes (512: one scene)
    float best[6] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
    bool cand[6] = {c->stage_mode != 2, c->stage_mode != 2, c->stage_mode != 2, staging_possible(c), false, false};
    if (!cand[3]) cand[0] = cand[1] = cand[2] = true;
    cand[4] = cand[0] && c->nt_fixed == 0;
    cand[5] = cand[0] && c->nt_fixed == 0 && c->nscenes() == 1;
    const uint32_t nt0 = c->nt_fixed ? c->nt_fixed : 256u;   // threads of candidate 0
    const uint32_t nts[6] = {nt0, 256u, 256u, 256u, 128u, 512u};
    int rc = SPHGB_OK;
    for (int rep = 0; rep < 2 && rc == SPHGB_OK; rep++)
        for (uint32_t k = 0; k < 6 && rc == SPHGB_OK; k++) {
            if (!cand[k]) continue;
            const uint32_t lg = (k == 1 || k == 2) ? k : 0u;
            c->lpp_log2 = lg;
            c->staged = k == 3;
            c->solver_nt = nts[k];
            cudaEventRecord(e0, c->stream);
            rc = step_host_loop<T>(c);
            cudaEventRecord(e1, c->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            best[k] = std::min(best[k], ms);
            if (cudaMemcpy(c->sc, saved.data(), (S + 1) * sizeof(StepScalars), cudaMemcpyHostToDevice) != cudaSuccess)
                rc = fail(c, SPHGB_ERR_CUDA, "autotune: restoring the step scalars");
        }
    c->profile = prof;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (saved_pa) {
        const cudaError_t e = cudaMemcpy(c->pa, saved_pa, pa_bytes, cudaMemcpyDeviceToDevice);
        cudaFree(saved_pa);
        if (e != cudaSuccess && !rc) rc = fail(c, SPHGB_ERR_CUDA, "autotune: restoring the pressure accelerations");
    }
    if (rc) return rc;
    if (c->nbodies)
        CK(cudaMemcpy(c->bodies.acc, saved_acc.data(), saved_acc.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaGetLastError());
    // a block size other than 256 must win by 2 %: on the 1M dam break the trial step (one step
    // from the state at hand) put 128 and 512 within 1 % of 256, while over 20 steps of the
    // solve-heavy phase they ran 1.8 % and 0.7 % slower
    uint32_t pick = 0;
    for (uint32_t k = 0; k < 6; k++) {
        c->tune_ms[k] = cand[k] ? best[k] : 0.0f;
        const float score = k >= 4 ? best[k] / 0.98f : best[k];
        const float held = pick >= 4 ? best[pick] / 0.98f : best[pick];
        if (cand[k] && (!cand[pick] || score < held)) pick = k;
    }
    c->lpp_log2 = (pick == 1 || pick == 2) ? pick : 0u;
    c->staged = pick == 3;
    c->solver_nt = nts[pick];
    c->tuned = true;
    invalidate_graphs(c);
    return SPHGB_OK;
}

// The Bender2019 configurations this path supports: bodies given only as volume maps built for
// the current support radius, each in one scene of the batch, forces collected with one body per map.
int check_boundary_method(sphgb_ctx *c)
{
    if (c->boundary_method != 2) return SPHGB_OK;
    if (c->vmaps.empty()) return fail(c, SPHGB_ERR_STATE, "Bender2019 boundary without volume maps");
    for (const auto &m : c->vmaps)
        if (m.scene >= c->nscenes()) return fail(c, SPHGB_ERR_ARGUMENT, "a volume map belongs to a scene that is not uploaded");
    if (c->nb) return fail(c, SPHGB_ERR_STATE, "the Bender2019 boundary takes no boundary particles");
    if (c->nbodies && c->nbodies != c->vmaps.size())
        return fail(c, SPHGB_ERR_ARGUMENT, "with volume maps the bodies are the maps: one body per map");
    for (const auto &m : c->vmaps)
        if (m.support != 4.0 * c->prm.particle_radius)
            return fail(c, SPHGB_ERR_STATE, "a volume map was built for another particle radius");
    return SPHGB_OK;
}

// the bodies (maps in the order they were added) in scene order, stable within a scene
std::vector<uint32_t> vmap_order(const sphgb_ctx *c)
{
    std::vector<uint32_t> o(c->vmaps.size());
    for (uint32_t b = 0; b < o.size(); b++) o[b] = b;
    std::stable_sort(o.begin(), o.end(), [&](uint32_t a, uint32_t b) { return c->vmaps[a].scene < c->vmaps[b].scene; });
    return o;
}

// the maps as the step reads them (VMapDev<T>), in scene order
template <class T> std::vector<VMapDev<T>> vmap_dev_array(const sphgb_ctx *c)
{
    const std::vector<uint32_t> order = vmap_order(c);
    std::vector<VMapDev<T>> h(c->vmaps.size());
    for (size_t q = 0; q < c->vmaps.size(); q++) {
        const auto &m = c->vmaps[order[q]];
        VMapDev<T> &d = h[q];
        for (int k = 0; k < 3; k++) {
            d.dmin[k] = (T)m.dmin[k];
            d.dmax[k] = (T)m.dmax[k];
            d.cs[k] = (T)((m.dmax[k] - m.dmin[k]) / (double)m.res[k]);
            d.t[k] = (T)m.t[k];
            d.v[k] = (T)m.v[k];
            d.w[k] = (T)m.w[k];
            d.max_dist = (T)m.max_dist;
            d.res[k] = m.res[k];
        }
        for (int k = 0; k < 9; k++) d.R[k] = (T)m.R[k];
        d.pad = 0;
        d.coef = static_cast<const T *>(m.coef);
    }
    return h;
}

// uploaded after a map is added or removed or changes scene, and when the context is prepared:
// the maps in scene order and, for a batch, each scene's range and each map's body, scene and slot
template <class T> int upload_vmaps(sphgb_ctx *c)
{
    for (void **p : {&c->d_vmaps, &c->d_vmap_range, &c->d_vmap_info}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    c->vmaps_dirty = false;
    c->vmap_max = 0;
    if (c->vmaps.empty()) return SPHGB_OK;
    const std::vector<VMapDev<T>> h = vmap_dev_array<T>(c);
    CK(cudaMalloc(&c->d_vmaps, h.size() * sizeof(VMapDev<T>)));
    CK(cudaMemcpy(c->d_vmaps, h.data(), h.size() * sizeof(VMapDev<T>), cudaMemcpyHostToDevice));
    const uint32_t S = c->nscenes();
    std::vector<uint2> range(S, make_uint2(0u, 0u));
    std::vector<uint4> info(c->vmaps.size());
    const std::vector<uint32_t> order = vmap_order(c);
    for (uint32_t q = 0; q < order.size(); q++) {
        const uint32_t s = std::min(c->vmaps[order[q]].scene, S - 1);
        if (range[s].y == 0) range[s].x = q;
        info[q] = make_uint4(order[q], s, range[s].y, 0u);
        range[s].y++;
    }
    for (const uint2 &r : range) c->vmap_max = std::max(c->vmap_max, r.y);
    if (S > 1) {
        CK(cudaMalloc(&c->d_vmap_range, range.size() * sizeof(uint2)));
        CK(cudaMemcpy(c->d_vmap_range, range.data(), range.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&c->d_vmap_info, info.size() * sizeof(uint4)));
        CK(cudaMemcpy(c->d_vmap_info, info.data(), info.size() * sizeof(uint4), cudaMemcpyHostToDevice));
    }
    return SPHGB_OK;
}

// new poses and velocities, copied in place on the step stream before the next step (captured
// graphs keep the array's address)
template <class T> int refresh_vmaps(sphgb_ctx *c)
{
    c->vmaps_dirty = false;
    if (!c->d_vmaps || c->vmaps.empty()) return SPHGB_OK;
    const std::vector<VMapDev<T>> h = vmap_dev_array<T>(c);
    CK(cudaMemcpyAsync(c->d_vmaps, h.data(), h.size() * sizeof(VMapDev<T>), cudaMemcpyHostToDevice, c->stream));
    return SPHGB_OK;
}

// Buffers of the moving bodies (body allocations, made once per boundary count) and their
// contents from the prepared layout: rest positions (the uploaded positions, body coordinates),
// volumes (computed for the rest shape: a rigid body's particles keep them) and bodies, upload order.
template <class T> int prepare_body_motion(sphgb_ctx *c)
{
    if (!c->bmotion || c->bm_ready || !c->nb || !c->nbodies) return SPHGB_OK;
    const uint32_t nb = c->nb;
    int rc;
    if (c->bm_nb != nb) {
        const size_t vs = sizeof(v4_t<T>), tiles = (nb + kSortTile - 1) / kSortTile;
        auto al = [&](auto **p, size_t bytes) { return dalloc_into(c, c->body_allocs, p, bytes); };
        if ((rc = al(&c->d_bmot, (size_t)c->nbodies * sizeof(BodyMotionDev<T>))) || (rc = al(&c->bm_x0, nb * vs)) ||
            (rc = al(&c->bm_V0, nb * sizeof(T))) || (rc = al(&c->bm_xtmp, nb * vs)) || (rc = al(&c->bm_vtmp, nb * vs)) ||
            (rc = al(&c->vbs, nb * vs)) || (rc = al(&c->bm_body, nb * 4)) || (rc = al(&c->bm_k1, nb * 4)) ||
            (rc = al(&c->bm_k2, nb * 4)) || (rc = al(&c->bm_v1, nb * 4)) || (rc = al(&c->bm_v2, nb * 4)) ||
            (rc = al(&c->bm_cells, nb * 4)) || (rc = al(&c->bm_hist, (tiles + 1) * 256 * 4)) ||
            (rc = al(&c->bm_scene, nb * 4)))
            return rc;
        c->bm_nb = nb;
    }
    CK(cudaStreamSynchronize(c->stream));
    std::vector<v4_t<T>> x0(nb), xs(nb);
    std::vector<uint32_t> bid(nb);
    std::vector<T> V0(nb);
    CK(cudaMemcpy(xs.data(), c->xb, nb * sizeof(v4_t<T>), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(bid.data(), c->bid, nb * 4, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < nb; k++) V0[bid[k]] = (T)xs[k].w;
    for (uint32_t u = 0; u < nb; u++) {
        const double *p = c->hb.data() + 3 * (size_t)u;
        x0[u].x = (T)p[0];
        x0[u].y = (T)p[1];
        x0[u].z = (T)p[2];
        x0[u].w = T(0);
    }
    CK(cudaMemcpy(c->bm_x0, x0.data(), nb * sizeof(v4_t<T>), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->bm_V0, V0.data(), nb * sizeof(T), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->bm_body, c->body_of.data(), nb * 4, cudaMemcpyHostToDevice));
    std::vector<uint32_t> bs(nb, 0u);   // each boundary particle's scene (upload order)
    for (uint32_t s = 0; s < c->scn.size(); s++)
        for (uint32_t k = 0; k < c->scn[s].nb; k++) bs[c->scn[s].bstart + k] = s;
    CK(cudaMemcpy(c->bm_scene, bs.data(), nb * 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(c->vbs, 0, nb * sizeof(v4_t<T>)));
    c->bm_ready = true;
    c->bmot_dirty = true;
    invalidate_graphs(c);
    return SPHGB_OK;
}

// the bodies' poses and velocities, copied in place on the step stream before the next step
template <class T> int refresh_body_motion(sphgb_ctx *c)
{
    c->bmot_dirty = false;
    if (!c->d_bmot) return SPHGB_OK;
    std::vector<BodyMotionDev<T>> h(c->nbodies);
    for (uint32_t b = 0; b < c->nbodies; b++) {
        const double *q = c->bmot.data() + 18 * (size_t)b;
        for (int k = 0; k < 9; k++) h[b].R[k] = (T)q[k];
        for (int k = 0; k < 3; k++) {
            h[b].t[k] = (T)q[9 + k];
            h[b].v[k] = (T)q[12 + k];
            h[b].w[k] = (T)q[15 + k];
        }
    }
    CK(cudaMemcpyAsync(c->d_bmot, h.data(), h.size() * sizeof(BodyMotionDev<T>), cudaMemcpyHostToDevice, c->stream));
    return SPHGB_OK;
}

// Fluid phases: their particle counts cover the fluid; one scene; Weiler2018 (a system per fluid
// model over same-phase neighbours) and the learned warm start (trained on one rest density) are
// not available with several phases.
int check_phases(sphgb_ctx *c)
{
    if (c->phase_counts.size() <= 1) return SPHGB_OK;
    uint64_t total = 0;
    for (uint32_t n : c->phase_counts) total += n;
    if (total != c->n) return fail(c, SPHGB_ERR_STATE, "the fluid phases do not cover the uploaded fluid");
    if (c->nscenes() > 1) return fail(c, SPHGB_ERR_STATE, "fluid phases serve a single scene, not a batch");
    if (c->learned) return fail(c, SPHGB_ERR_ARGUMENT, "the learned warm start takes one fluid phase");
    return SPHGB_OK;
}

template <class T> int do_step(sphgb_ctx *c)
{
    int rc;
    if ((rc = check_boundary_method(c))) return rc;
    if ((rc = check_phases(c))) return rc;
    if (!c->prepared && (rc = prepare<T>(c))) return rc;
    if (c->vmaps_dirty && (rc = refresh_vmaps<T>(c))) return rc;
    if ((rc = prepare_body_motion<T>(c))) return rc;
    if (c->bmot_dirty && c->bm_ready && (rc = refresh_body_motion<T>(c))) return rc;
    if ((rc = upload_scalars(c))) return rc;
    if (!c->tuned) {
        if (c->lpp_fixed) {
            c->lpp_log2 = c->lpp_fixed == 1 ? 0u : (c->lpp_fixed == 2 ? 1u : 2u);
            c->solver_nt = c->nt_fixed ? c->nt_fixed : 256u;
            // the 128- and 512-thread passes are unstaged
            c->staged = c->lpp_log2 == 0 && staging_possible(c) && c->solver_nt == 256u;
            c->tuned = true;
            invalidate_graphs(c);
        } else if ((rc = autotune<T>(c))) {
            return rc;
        }
    }
    if (c->cfg.use_graph && !c->profile) {
        if (!c->graph_ok) {
            invalidate_graphs(c);
            if ((rc = build_graph<T>(c, 0, &c->exec[0]))) return rc;
            if ((rc = build_graph<T>(c, 1, &c->exec[1]))) return rc;
            c->graph_ok = true;
        }
        CK(cudaGraphLaunch(c->exec[c->parity], c->stream));
    } else {
        if ((rc = step_host_loop<T>(c))) return rc;
    }
    c->parity = 1 - c->parity;
    CK(cudaMemcpyAsync(c->hsc, c->sc, (c->nscenes() + 1) * sizeof(StepScalars), cudaMemcpyDeviceToHost, c->stream));
    c->step_pending = true;
    return SPHGB_OK;
}

// statistics of scene s from the host mirror (g: the global record)
void scene_stats(const sphgb_ctx *c, const StepScalars &h, const StepScalars &g, sphgb_stats *st)
{
    st->iterations = h.iters;
    st->iterations_v = h.iters_v;
    // fluid phases: the phases' systems' iterations summed, their largest final error
    const bool phases = c->phase_counts.size() > 1;
    st->visco_iterations = c->prm.viscosity_method == 6 ? (phases ? h.iters_cg_tot : h.iters_cg) : 0;
    st->max_fluid_neighbors = h.max_nf;
    st->max_boundary_neighbors = h.max_nb;
    st->flags = h.flags | g.flags;
    st->avg_density_err = h.avg_err;
    st->avg_density_err_v = h.avg_err_v;
    st->visco_error = c->prm.viscosity_method == 6 ? (phases ? std::max(h.cg_err_max, h.cg_err) : h.cg_err) : 0.0;
    st->dt_used = h.dt_used;
    st->dt_next = h.dt_next;
    st->time = h.time;
    st->kernel_launches = g.launches + (c->learned ? 1 : 0);   // the network forward counts as one
    st->learned_used = c->learned ? h.ws_used : 0;
    st->reserved = 0;
    for (int k = 0; k < 2; k++) {
        st->ws_residual_classic[k] = c->learned ? h.ws_rc[k] : 0.0;
        st->ws_residual_learned[k] = c->learned ? h.ws_rl[k] : 0.0;
    }
}

int fill_stats(sphgb_ctx *c, sphgb_stats *st)
{
    CK(cudaStreamSynchronize(c->stream));
    const uint32_t S = c->nscenes();
    const StepScalars &g = c->hsc[S];
    if (c->step_pending) {
        for (uint32_t s = 0; s < c->scn.size(); s++) {
            c->scn[s].dt = c->hsc[s].dt;
            c->scn[s].time = c->hsc[s].time;
            c->scn[s].prev_iters = c->hsc[s].prev_iters;
        }
        c->step_pending = false;
    }
    unsigned flags = g.flags;
    for (uint32_t s = 0; s < S; s++) flags |= c->hsc[s].flags;
    if (st) {
        // one scene: its statistics; a batch: scene 0's times, the maxima of counts and errors over the
        // scenes (the iterations the batch's loops executed), mean initial residuals, OR of flags
        scene_stats(c, c->hsc[0], g, st);
        for (uint32_t s = 1; s < S; s++) {
            sphgb_stats o;
            scene_stats(c, c->hsc[s], g, &o);
            st->iterations = std::max(st->iterations, o.iterations);
            st->iterations_v = std::max(st->iterations_v, o.iterations_v);
            st->visco_iterations = std::max(st->visco_iterations, o.visco_iterations);
            st->max_fluid_neighbors = std::max(st->max_fluid_neighbors, o.max_fluid_neighbors);
            st->max_boundary_neighbors = std::max(st->max_boundary_neighbors, o.max_boundary_neighbors);
            st->avg_density_err = std::max(st->avg_density_err, o.avg_density_err);
            st->avg_density_err_v = std::max(st->avg_density_err_v, o.avg_density_err_v);
            st->visco_error = std::max(st->visco_error, o.visco_error);
            st->learned_used |= o.learned_used;
            for (int k = 0; k < 2; k++) {
                st->ws_residual_classic[k] += o.ws_residual_classic[k];
                st->ws_residual_learned[k] += o.ws_residual_learned[k];
            }
        }
        for (int k = 0; k < 2; k++) {
            st->ws_residual_classic[k] /= S;
            st->ws_residual_learned[k] /= S;
        }
        st->flags = flags;
    }
    if (flags & kFlagOverflow)
        return fail(c, SPHGB_ERR_CAPACITY, "neighbour list capacity exceeded (raise max_fluid/boundary_neighbors)");
    if (flags & kFlagNonFinite) return fail(c, SPHGB_ERR_NONFINITE, "non-finite velocity");
    if (flags & kFlagLoopGuard) return fail(c, SPHGB_ERR_STATE, "a device solver loop exceeded its iteration bound");
    return SPHGB_OK;
}

int alloc_learned_buffers(sphgb_ctx *c);

int ensure_scalar_mirror(sphgb_ctx *c, size_t records)
{
    if (c->hsc_cap >= records) return SPHGB_OK;
    if (c->hsc) cudaFreeHost(c->hsc);
    c->hsc = nullptr;
    c->hsc_cap = 0;
    CK(cudaMallocHost(&c->hsc, records * sizeof(StepScalars)));
    std::memset(c->hsc, 0, records * sizeof(StepScalars));
    c->hsc_cap = records;
    return SPHGB_OK;
}

// (Re)allocate every per-particle buffer for the scenes with fluid counts `counts` and
// upload their state; x, v (and id) hold all scenes' particles in scene order.
template <class T> int init_scenes(sphgb_ctx *c, const double *x, const double *v, const uint32_t *id,
                                   const std::vector<uint32_t> &counts)
{
    int rc;
    free_all(c);
    c->feat = c->mlp_x = c->mlp_y = nullptr;
    c->kl = c->pa2 = nullptr;
    c->staging = nullptr;
    c->staging_bytes = 0;
    c->d_scenes = nullptr;
    c->d_blk = nullptr;
    c->have_fluid = false;
    const uint32_t S = (uint32_t)counts.size();
    std::vector<SceneHost> old = c->scn;
    c->scn.assign(S, SceneHost{});
    uint32_t u = 0, p = 0;
    for (uint32_t s = 0; s < S; s++) {
        SceneHost &h = c->scn[s];
        h.n = counts[s];
        h.ustart = u;
        h.pstart = p;
        h.dt = c->dt;
        h.time = 0.0;
        if (s < old.size()) { h.nb = old[s].nb; h.bstart = old[s].bstart; }
        for (int d = 0; d < 3; d++) { h.bmin[d] = s < old.size() ? old[s].bmin[d] : 0.0; h.bmax[d] = s < old.size() ? old[s].bmax[d] : 0.0; }
        u += h.n;
        p += S > 1 ? (h.n + kBlock - 1) / kBlock * kBlock : h.n;
    }
    c->n = u;
    c->np = p;
    const size_t N = std::max<uint32_t>(c->np, 1), NR = std::max<uint32_t>(c->n, 1);
    const size_t vs = vec_size(c), rs = real_size(c);
    for (int k = 0; k < 2; k++) {
        if ((rc = dalloc(c, &c->set_x[k], N * vs))) return rc;
        if ((rc = dalloc(c, &c->set_v[k], N * vs))) return rc;
        if ((rc = dalloc(c, &c->set_vdiff[k], N * vs))) return rc;
        if ((rc = dalloc(c, &c->set_kappa[k], N * rs))) return rc;
        if ((rc = dalloc(c, &c->set_kappa_v[k], N * rs))) return rc;
        if ((rc = dalloc(c, &c->set_id[k], N * 4))) return rc;
        c->set_xlo[k] = nullptr;
        if (!c->fp64 && (rc = dalloc(c, &c->set_xlo[k], N * sizeof(float4)))) return rc;
        // idle slots of a batch hold zeros
        CK(cudaMemset(c->set_x[k], 0, N * vs));
        CK(cudaMemset(c->set_v[k], 0, N * vs));
    }
    if ((rc = dalloc(c, &c->a, N * vs))) return rc;
    if ((rc = dalloc(c, &c->pa, N * vs))) return rc;
    c->xa = nullptr;
    if (!c->fp64 && (rc = dalloc(c, &c->xa, N * 2 * sizeof(float4)))) return rc;
    if ((rc = dalloc(c, &c->xk, N * vs))) return rc;
    if ((rc = dalloc(c, &c->bg, N * vs))) return rc;
    if ((rc = dalloc(c, &c->density, N * rs))) return rc;
    if ((rc = dalloc(c, &c->factor, N * rs))) return rc;
    if ((rc = dalloc(c, &c->dadv, N * rs))) return rc;
    if ((rc = dalloc(c, &c->nfc, N * 4))) return rc;
    if ((rc = dalloc(c, &c->nbc, N * 4))) return rc;
    const size_t NW = (N + 31) / 32 * 32;
    if ((rc = dalloc(c, &c->lf, NW * c->cfg.max_fluid_neighbors * 4))) return rc;
    if ((rc = dalloc(c, &c->lb, NW * c->cfg.max_boundary_neighbors * 4))) return rc;
    c->ll = c->stage_off = nullptr;
    c->stage_hdr = nullptr;
    c->stage_cell = nullptr;
    c->stage_src = nullptr;
    if (!c->fp64) {
        const size_t nblk = (N + kBlock - 1) / kBlock;
        if ((rc = dalloc(c, &c->ll, NW * c->cfg.max_fluid_neighbors * 2))) return rc;
        if ((rc = dalloc(c, &c->stage_hdr, nblk * sizeof(uint2)))) return rc;
        if ((rc = dalloc(c, &c->stage_cell, nblk * kStageCells * 4))) return rc;
        if ((rc = dalloc(c, &c->stage_off, nblk * kStageCells * 2))) return rc;
        if ((rc = dalloc(c, &c->stage_src, nblk * kStageCap * 4))) return rc;
    }
    if ((rc = dalloc(c, &c->key, NR * 4))) return rc;
    if ((rc = dalloc(c, &c->key2, NR * 4))) return rc;
    if ((rc = dalloc(c, &c->perm, NR * 4))) return rc;
    if ((rc = dalloc(c, &c->perm2, NR * 4))) return rc;
    if ((rc = dalloc(c, &c->cell0, N * 4))) return rc;
    if ((rc = dalloc(c, &c->cell1, N * 4))) return rc;
    for (int k = 0; k < 5; k++)
        if ((rc = dalloc(c, &c->cg[k], N * vs))) return rc;
    for (int k = 0; k < 2; k++)
        if ((rc = dalloc(c, &c->inv[k], N * vs))) return rc;
    const size_t blocks = (N + kBlock - 1) / kBlock;
    // reductions index partials by block: up to 4 blocks per kBlock slots (4 lanes per particle)
    if ((rc = dalloc(c, &c->partials, 4 * blocks * 4 * sizeof(double)))) return rc;
    const size_t nrec = (size_t)std::max<uint32_t>(S, 1) + 1;
    if ((rc = dalloc(c, &c->counters, std::max<size_t>(nrec * 4, 64)))) return rc;
    CK(cudaMemset(c->counters, 0, std::max<size_t>(nrec * 4, 64)));
    if ((rc = dalloc(c, &c->sc, nrec * sizeof(StepScalars)))) return rc;
    CK(cudaMemset(c->sc, 0, nrec * sizeof(StepScalars)));
    if ((rc = ensure_scalar_mirror(c, nrec))) return rc;
    const size_t tiles = (NR + kSortTile - 1) / kSortTile;
    if ((rc = dalloc(c, &c->hist, (tiles + 1) * 256 * 4))) return rc;
    if ((rc = dalloc(c, &c->inv_perm, NR * 4))) return rc;
    if (S > 1) {
        if ((rc = dalloc(c, &c->d_scenes, S * sizeof(SceneDev<T>)))) return rc;
        std::vector<uint4> blk(blocks);
        for (uint32_t s = 0; s < S; s++) {
            const SceneHost &h = c->scn[s];
            for (uint32_t b = h.pstart / kBlock; b < (h.pstart + h.n + kBlock - 1) / kBlock; b++)
                blk[b] = make_uint4(s, h.pstart, h.pstart + h.n, 0u);
        }
        if ((rc = dalloc(c, &c->d_blk, blocks * sizeof(uint4)))) return rc;
        CK(cudaMemcpy(c->d_blk, blk.data(), blocks * sizeof(uint4), cudaMemcpyHostToDevice));
        if ((rc = upload_scene_table<T>(c))) return rc;
    }
    // zero per-step fields so that downloads before the first step are defined
    CK(cudaMemset(c->a, 0, N * vs));
    CK(cudaMemset(c->pa, 0, N * vs));
    CK(cudaMemset(c->density, 0, N * rs));
    CK(cudaMemset(c->factor, 0, N * rs));
    CK(cudaMemset(c->dadv, 0, N * rs));
    CK(cudaMemset(c->nfc, 0, N * 4));
    CK(cudaMemset(c->nbc, 0, N * 4));
    // staging copy of x/v (double) and ids
    double *dx, *dv;
    uint32_t *did = nullptr;
    if ((rc = dalloc(c, &dx, NR * 3 * sizeof(double)))) return rc;
    if ((rc = dalloc(c, &dv, NR * 3 * sizeof(double)))) return rc;
    if (c->n) {
        CK(cudaMemcpy(dx, x, (size_t)c->n * 3 * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dv, v, (size_t)c->n * 3 * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (id) {
        if ((rc = dalloc(c, &did, NR * 4))) return rc;
        CK(cudaMemcpy(did, id, (size_t)c->n * 4, cudaMemcpyHostToDevice));
    }
    c->parity = 0;
    DevParams<T> P = make_params<T>(c);
    DevBufs<T> B = make_bufs<T>(c, 0);
    launch_init_state<T>(P, B, dx, dv, did, c->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    dfree(c->allocs, dx);
    dfree(c->allocs, dv);
    if (did) dfree(c->allocs, did);
    // extents
    for (SceneHost &h : c->scn) {
        for (int d = 0; d < 3; d++) {
            h.fmin[d] = h.n ? x[3 * (size_t)h.ustart + d] : 0.0;
            h.fmax[d] = h.fmin[d];
        }
        for (uint32_t i = h.ustart + 1; i < h.ustart + h.n; i++)
            for (int d = 0; d < 3; d++) {
                h.fmin[d] = std::min(h.fmin[d], x[3 * (size_t)i + d]);
                h.fmax[d] = std::max(h.fmax[d], x[3 * (size_t)i + d]);
            }
    }
    c->have_fluid = true;
    c->tuned = false;
    if ((c->learned || c->feat_on) && (rc = alloc_learned_buffers(c))) return rc;
    c->scalars_dirty = true;
    return SPHGB_OK;
}

// Host copy of the boundary particles (scene order) with per-scene counts; the device
// copy, its sort and the volumes are made by prepare().
int set_boundary(sphgb_ctx *c, const double *xb, const std::vector<uint32_t> &counts)
{
    size_t total = 0;
    for (uint32_t k : counts) total += k;
    if (total > 0xffffffffull) return fail(c, SPHGB_ERR_ARGUMENT, "too many boundary particles");
    c->hb.assign(xb, xb + 3 * total);
    c->nb = (uint32_t)total;
    // bodies are given per boundary particle: a boundary of another size drops them
    if (c->nbodies && c->body_of.size() != total) {
        if (c->stream) cudaStreamSynchronize(c->stream);
        free_bodies(c);
    }
    if (c->scn.size() < counts.size()) c->scn.resize(counts.size());
    uint32_t b = 0;
    for (uint32_t s = 0; s < c->scn.size(); s++) {
        SceneHost &h = c->scn[s];
        h.nb = s < counts.size() ? counts[s] : 0;
        h.bstart = b;
        for (int d = 0; d < 3; d++) {
            h.bmin[d] = h.nb ? xb[3 * (size_t)b + d] : 0.0;
            h.bmax[d] = h.bmin[d];
        }
        for (uint32_t i = b + 1; i < b + h.nb; i++)
            for (int d = 0; d < 3; d++) {
                h.bmin[d] = std::min(h.bmin[d], xb[3 * (size_t)i + d]);
                h.bmax[d] = std::max(h.bmax[d], xb[3 * (size_t)i + d]);
            }
        b += h.nb;
    }
    c->have_boundary = true;
    free_prepared(c);
    invalidate_graphs(c);
    return SPHGB_OK;
}

int ensure_staging(sphgb_ctx *c, size_t bytes)
{
    if (c->staging_bytes >= bytes) return SPHGB_OK;
    int rc = dalloc(c, &c->staging, bytes);
    if (rc) return rc;
    c->staging_bytes = bytes;
    return SPHGB_OK;
}

int field_components(int field)
{
    switch (field) {
    case SPHGB_FIELD_POSITION: case SPHGB_FIELD_VELOCITY: case SPHGB_FIELD_ACCELERATION:
    case SPHGB_FIELD_PRESSURE_ACCEL: case SPHGB_FIELD_VDIFF: case SPHGB_FIELD_BOUNDARY_POSITION:
    case SPHGB_FIELD_POSITION_HI: case SPHGB_FIELD_POSITION_LO:
        return 3;
    case SPHGB_FIELD_FEATURES:
        return 10;
    default:
        return 1;
    }
}

size_t dtype_size(int dt) { return dt == SPHGB_DTYPE_F64 ? 8 : 4; }

int alloc_learned_buffers(sphgb_ctx *c)
{
    if (c->feat) return SPHGB_OK;
    const size_t N = std::max<uint32_t>(c->np, 1);
    int rc;
    if ((rc = dalloc(c, &c->feat, N * 8 * sizeof(float)))) return rc;
    if ((rc = dalloc(c, &c->mlp_x, N * 10 * sizeof(float)))) return rc;
    if ((rc = dalloc(c, &c->mlp_y, N * 2 * sizeof(float)))) return rc;
    if ((rc = dalloc(c, &c->kl, N * real_size(c)))) return rc;
    if ((rc = dalloc(c, &c->pa2, N * vec_size(c)))) return rc;
    CK(cudaMemset(c->feat, 0, N * 8 * sizeof(float)));
    CK(cudaMemset(c->mlp_x, 0, N * 10 * sizeof(float)));
    return SPHGB_OK;
}

int check_finite(sphgb_ctx *c, const double *a, size_t m, const char *what)
{
    for (size_t k = 0; k < m; k++)
        if (!std::isfinite(a[k])) return fail(c, SPHGB_ERR_NONFINITE, std::string("non-finite ") + what);
    return SPHGB_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int sphgb_abi_version(void) { return SPHGB_ABI_VERSION; }

int sphgb_default_params(sphgb_params *p)
{
    if (!p) return SPHGB_ERR_ARGUMENT;
    *p = kDefaults;
    return SPHGB_OK;
}

int sphgb_create(const sphgb_config *cfg, sphgb_ctx **out)
{
    if (!cfg || !out) return SPHGB_ERR_ARGUMENT;
    if (cfg->abi_version != SPHGB_ABI_VERSION) return SPHGB_ERR_ARGUMENT;
    if (cfg->precision != SPHGB_PRECISION_FP32 && cfg->precision != SPHGB_PRECISION_FP64) return SPHGB_ERR_ARGUMENT;
    sphgb_ctx *c = new sphgb_ctx();
    c->cfg = *cfg;
    if (c->cfg.max_fluid_neighbors == 0) c->cfg.max_fluid_neighbors = 80;
    c->cfg.max_fluid_neighbors = (c->cfg.max_fluid_neighbors + 3u) / 4u * 4u;   // fluid-list layout: lanes of 4
    if (c->cfg.max_boundary_neighbors == 0) c->cfg.max_boundary_neighbors = 128;
    c->fp64 = cfg->precision == SPHGB_PRECISION_FP64;
    c->prm = kDefaults;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->body_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = configure_staged_kernels();
    if (e == cudaSuccess && ensure_scalar_mirror(c, 2) != SPHGB_OK) e = cudaErrorMemoryAllocation;
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (c->hsc) cudaFreeHost(c->hsc);
        if (c->stream) cudaStreamDestroy(c->stream);
        if (c->body_stream) cudaStreamDestroy(c->body_stream);
        delete c;
        return SPHGB_ERR_CUDA;
    }
    *out = c;
    return SPHGB_OK;
}

int sphgb_destroy(sphgb_ctx *c)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(c->cfg.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->export_thread.joinable()) c->export_thread.join();
    if (c->export_stream) cudaStreamSynchronize(c->export_stream);
    free_all(c);
    free_bodies(c);
    free_vmaps(c);
    if (c->hsc) cudaFreeHost(c->hsc);
    if (c->export_dev) cudaFree(c->export_dev);
    if (c->export_host) cudaFreeHost(c->export_host);
    for (cudaEvent_t e : {c->export_scattered, c->export_copied, c->export_start})
        if (e) cudaEventDestroy(e);
    if (c->export_stream) cudaStreamDestroy(c->export_stream);
    if (c->mlp_p) cudaFree(c->mlp_p);
    if (c->mlp_w) cudaFree(c->mlp_w);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->body_stream) cudaStreamDestroy(c->body_stream);
    delete c;
    return SPHGB_OK;
}

const char *sphgb_last_error(const sphgb_ctx *c) { return c ? c->err.c_str() : "null context"; }

int sphgb_set_params(sphgb_ctx *c, const sphgb_params *p)
{
    if (!c || !p) return SPHGB_ERR_ARGUMENT;
    if (!(p->particle_radius > 0) || !(p->density0 > 0)) return fail(c, SPHGB_ERR_ARGUMENT, "radius/density0 must be > 0");
    if (p->viscosity_method != 0 && p->viscosity_method != 6)
        return fail(c, SPHGB_ERR_ARGUMENT, "viscosity_method must be 0 (none) or 6 (Weiler et al. 2018)");
    if (p->cfl_method < 0 || p->cfl_method > 2) return fail(c, SPHGB_ERR_ARGUMENT, "cfl_method must be 0, 1 or 2");
    const bool radius_changed = c->prm.particle_radius != p->particle_radius;
    c->prm = *p;
    invalidate_graphs(c);
    // the cell grids and boundary volumes depend on the support radius
    if (radius_changed && c->prepared) c->prepared = false;
    return SPHGB_OK;
}

int sphgb_get_params(const sphgb_ctx *c, sphgb_params *p)
{
    if (!c || !p) return SPHGB_ERR_ARGUMENT;
    *p = c->prm;
    return SPHGB_OK;
}

int sphgb_upload_boundary(sphgb_ctx *c, const double *xb, uint32_t nb)
{
    if (!c || (!xb && nb)) return SPHGB_ERR_ARGUMENT;
    if (c->scn.size() > 1) return fail(c, SPHGB_ERR_STATE, "a batch of scenes takes its boundary in sphgb_upload_scenes");
    int rc = check_finite(c, xb, (size_t)nb * 3, "boundary position");
    if (rc) return rc;
    cudaSetDevice(c->cfg.device);
    return set_boundary(c, xb, std::vector<uint32_t>{nb});
}

int sphgb_upload_boundary_f32(sphgb_ctx *c, const float *xb, uint32_t nb)
{
    if (!c || (!xb && nb)) return SPHGB_ERR_ARGUMENT;
    std::vector<double> d((size_t)nb * 3);
    for (size_t k = 0; k < d.size(); k++) d[k] = xb[k];
    return sphgb_upload_boundary(c, d.data(), nb);
}

int sphgb_upload_fluid(sphgb_ctx *c, const double *x, const double *v, const uint32_t *id, uint32_t n)
{
    if (!c || (n && (!x || !v))) return SPHGB_ERR_ARGUMENT;
    if (id) {
        // ids index the host arrays on download: they must be a permutation of 0..n-1
        std::vector<char> seen(n, 0);
        for (uint32_t i = 0; i < n; i++) {
            if (id[i] >= n || seen[id[i]]) return fail(c, SPHGB_ERR_ARGUMENT, "particle ids must be a permutation of 0..n-1");
            seen[id[i]] = 1;
        }
    }
    for (size_t k = 0; k < (size_t)n * 3; k++)
        if (!std::isfinite(x[k]) || !std::isfinite(v[k])) return fail(c, SPHGB_ERR_NONFINITE, "non-finite fluid state");
    cudaSetDevice(c->cfg.device);
    if (c->scn.size() > 1) {
        // a single scene replaces a batch: the batch's boundary does not carry over
        c->scn.clear();
        c->hb.clear();
        c->nb = 0;
        c->have_boundary = false;
    }
    int rc = c->fp64 ? init_scenes<double>(c, x, v, id, {n}) : init_scenes<float>(c, x, v, id, {n});
    if (rc) return rc;
    c->scalars_dirty = true;
    return SPHGB_OK;
}

int sphgb_upload_fluid_f32(sphgb_ctx *c, const float *x, const float *v, const uint32_t *id, uint32_t n)
{
    if (!c || (n && (!x || !v))) return SPHGB_ERR_ARGUMENT;
    std::vector<double> dx((size_t)n * 3), dv((size_t)n * 3);
    for (size_t k = 0; k < dx.size(); k++) { dx[k] = x[k]; dv[k] = v[k]; }
    return sphgb_upload_fluid(c, dx.data(), dv.data(), id, n);
}

int sphgb_upload_scenes(sphgb_ctx *c, uint32_t nscenes, const uint32_t *n, const uint32_t *nb, const double *x,
                        const double *v, const double *xb)
{
    if (!c || nscenes == 0 || !n || !nb || !x || !v) return SPHGB_ERR_ARGUMENT;
    size_t nt = 0, nbt = 0;
    for (uint32_t s = 0; s < nscenes; s++) {
        if (n[s] == 0) return fail(c, SPHGB_ERR_ARGUMENT, "every scene needs at least one fluid particle");
        nt += n[s];
        nbt += nb[s];
    }
    if (nbt && !xb) return SPHGB_ERR_ARGUMENT;
    // slots of a batch are padded to whole blocks: the padded total must fit 32-bit indices
    size_t padded = 0;
    for (uint32_t s = 0; s < nscenes; s++) padded += (n[s] + kBlock - 1) / kBlock * (size_t)kBlock;
    if (padded >= 0xffffffffull || nbt >= 0xffffffffull) return fail(c, SPHGB_ERR_CAPACITY, "too many particles");
    int rc = check_finite(c, x, nt * 3, "fluid position");
    if (!rc) rc = check_finite(c, v, nt * 3, "fluid velocity");
    if (!rc && nbt) rc = check_finite(c, xb, nbt * 3, "boundary position");
    if (rc) return rc;
    cudaSetDevice(c->cfg.device);
    c->scn.clear();
    std::vector<uint32_t> counts(n, n + nscenes), bcounts(nb, nb + nscenes);
    rc = c->fp64 ? init_scenes<double>(c, x, v, nullptr, counts) : init_scenes<float>(c, x, v, nullptr, counts);
    if (rc) return rc;
    static const double kNone[3] = {0, 0, 0};
    rc = set_boundary(c, nbt ? xb : kNone, bcounts);
    if (rc) return rc;
    c->scalars_dirty = true;
    return SPHGB_OK;
}

int sphgb_num_scenes(const sphgb_ctx *c, uint32_t *nscenes)
{
    if (!c || !nscenes) return SPHGB_ERR_ARGUMENT;
    *nscenes = (uint32_t)c->scn.size();
    return SPHGB_OK;
}

int sphgb_scene_stats(sphgb_ctx *c, uint32_t first, uint32_t count, sphgb_stats *out)
{
    if (!c || (!out && count)) return SPHGB_ERR_ARGUMENT;
    if ((size_t)first + count > c->scn.size()) return fail(c, SPHGB_ERR_ARGUMENT, "scene index out of range");
    sphgb_stats agg;
    const int rc = fill_stats(c, &agg);
    const StepScalars &g = c->hsc[c->nscenes()];
    for (uint32_t k = 0; k < count; k++) scene_stats(c, c->hsc[first + k], g, out + k);
    return rc;
}

int sphgb_set_time_step(sphgb_ctx *c, double dt)
{
    if (!c || !(dt > 0)) return SPHGB_ERR_ARGUMENT;
    sphgb_stats st;
    if (c->step_pending) fill_stats(c, &st);
    c->dt = dt;
    for (SceneHost &h : c->scn) h.dt = dt;
    c->scalars_dirty = true;
    return SPHGB_OK;
}

int sphgb_get_time_step(const sphgb_ctx *c, double *dt)
{
    if (!c || !dt) return SPHGB_ERR_ARGUMENT;
    if (c->step_pending) {
        cudaStreamSynchronize(c->stream);
        *dt = c->hsc[0].dt;
    } else {
        *dt = c->scn.empty() ? c->dt : c->scn[0].dt;
    }
    return SPHGB_OK;
}

int sphgb_set_time(sphgb_ctx *c, double t)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    sphgb_stats st;
    if (c->step_pending) fill_stats(c, &st);
    for (SceneHost &h : c->scn) h.time = t;
    c->scalars_dirty = true;
    return SPHGB_OK;
}

int sphgb_step(sphgb_ctx *c, sphgb_stats *stats)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "sphgb_step before sphgb_upload_fluid");
    if (c->n == 0) return fail(c, SPHGB_ERR_STATE, "sphgb_step of a fluid model without particles");
    cudaSetDevice(c->cfg.device);
    if (c->step_pending && c->scalars_dirty) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    int rc = c->fp64 ? do_step<double>(c) : do_step<float>(c);
    if (rc) return rc;
    if (stats) return fill_stats(c, stats);
    return SPHGB_OK;
}

int sphgb_sync(sphgb_ctx *c, sphgb_stats *stats)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    return fill_stats(c, stats);
}

int sphgb_set_feature_output(sphgb_ctx *c, int on)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (on && !c->have_fluid) return fail(c, SPHGB_ERR_STATE, "upload the fluid first");
    cudaSetDevice(c->cfg.device);
    if (on) {
        int rc = alloc_learned_buffers(c);
        if (rc) return rc;
    }
    c->feat_on = on != 0;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_warmstart_mlp(sphgb_ctx *c, const sphgb_mlp *m)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(c->cfg.device);
    invalidate_graphs(c);
    if (!m) {
        c->learned = false;
        return SPHGB_OK;
    }
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "upload the fluid first");
    const float *mp;
    const void *mw;
    float scale[2];
    int dev;
    mlp_export(m, &mp, &mw, scale, &dev);
    if (dev != c->cfg.device) return fail(c, SPHGB_ERR_ARGUMENT, "network and context are on different devices");
    int rc = alloc_learned_buffers(c);
    if (rc) return rc;
    // the network copy outlives re-uploads of the fluid: not in the per-particle allocation list
    if (!c->mlp_p) CK(cudaMalloc(&c->mlp_p, (size_t)kMlpParams * 4));
    if (!c->mlp_w) CK(cudaMalloc(&c->mlp_w, (size_t)kMlpParams * 2));
    CK(cudaMemcpy(c->mlp_p, mp, (size_t)kMlpParams * 4, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(c->mlp_w, mw, (size_t)kMlpParams * 2, cudaMemcpyDeviceToDevice));
    c->ws_scale[0] = scale[0];
    c->ws_scale[1] = scale[1];
    c->learned = true;
    return SPHGB_OK;
}

int sphgb_set_warmstart_gate(sphgb_ctx *c, uint32_t div_sweeps, uint32_t pressure_sweeps)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    c->ws_gate[0] = div_sweeps;
    c->ws_gate[1] = pressure_sweeps;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_lanes_per_particle(sphgb_ctx *c, uint32_t lanes)
{
    if (!c || (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4)) return SPHGB_ERR_ARGUMENT;
    sphgb_stats st;
    if (c->step_pending) fill_stats(c, &st);
    c->lpp_fixed = lanes;
    c->tuned = false;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_solver_block_threads(sphgb_ctx *c, uint32_t threads)
{
    if (!c || (threads != 0 && threads != 128 && threads != 256 && threads != 512)) return SPHGB_ERR_ARGUMENT;
    if (threads == 512 && c->nscenes() > 1) return fail(c, SPHGB_ERR_ARGUMENT, "512-thread blocks need one scene");
    sphgb_stats st;
    if (c->step_pending) fill_stats(c, &st);
    c->nt_fixed = threads;
    c->tuned = false;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_get_solver_block_threads(const sphgb_ctx *c, uint32_t *threads, float trial_ms[3])
{
    if (!c || !threads) return SPHGB_ERR_ARGUMENT;
    const bool used = c->lpp_log2 == 0 && !(c->staged && !c->fp64 && c->ll);
    *threads = used && !(c->solver_nt == 512u && c->nscenes() > 1) ? c->solver_nt : 256u;
    if (trial_ms) {
        trial_ms[0] = c->tune_ms[4];
        trial_ms[1] = c->tune_ms[0];
        trial_ms[2] = c->tune_ms[5];
    }
    return SPHGB_OK;
}

int sphgb_set_neighbor_staging(sphgb_ctx *c, int mode)
{
    if (!c || mode < 0 || mode > 2) return SPHGB_ERR_ARGUMENT;
    sphgb_stats st;
    if (c->step_pending) fill_stats(c, &st);
    c->stage_mode = mode;
    c->tuned = false;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_get_neighbor_staging(sphgb_ctx *c, int *active, float *staged_fraction, float *trial_ms)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    const bool on = c->staged && !c->fp64 && c->lpp_log2 == 0 && c->ll;
    if (active) *active = on ? 1 : 0;
    if (trial_ms) *trial_ms = c->tune_ms[3];
    if (staged_fraction) {
        *staged_fraction = 0.0f;
        if (on && c->np) {
            // blocks of the last step's stage tables that hold particles, and how many were staged
            cudaSetDevice(c->cfg.device);
            const size_t nblk = (c->np + kBlock - 1) / kBlock;
            std::vector<uint2> hdr(nblk);
            CK(cudaStreamSynchronize(c->stream));
            CK(cudaMemcpy(hdr.data(), c->stage_hdr, nblk * sizeof(uint2), cudaMemcpyDeviceToHost));
            size_t used = 0, staged = 0;
            for (uint32_t s = 0; s < c->nscenes(); s++) {
                const uint32_t b0 = c->scn.empty() ? 0u : c->scn[s].pstart / kBlock;
                const uint32_t n = c->scn.empty() ? c->n : c->scn[s].n;
                for (uint32_t b = b0; b < b0 + (n + kBlock - 1) / kBlock && b < nblk; b++) {
                    used++;
                    staged += hdr[b].x != 0;
                }
            }
            *staged_fraction = used ? (float)staged / (float)used : 0.0f;
        }
    }
    return SPHGB_OK;
}

int sphgb_get_lanes_per_particle(const sphgb_ctx *c, uint32_t *lanes, float trial_ms[3])
{
    if (!c || !lanes) return SPHGB_ERR_ARGUMENT;
    *lanes = 1u << c->lpp_log2;
    if (trial_ms)
        for (int k = 0; k < 3; k++) trial_ms[k] = c->tune_ms[k];
    return SPHGB_OK;
}

int sphgb_set_boundary_bodies(sphgb_ctx *c, const uint32_t *body, uint32_t nbodies, const double *center,
                              const int *dynamic)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (nbodies && ((!body && c->nb) || !center)) return SPHGB_ERR_ARGUMENT;
    if (nbodies && !c->have_boundary) return fail(c, SPHGB_ERR_STATE, "no boundary uploaded");
    for (uint32_t k = 0; nbodies && k < c->nb; k++)
        if (body[k] >= nbodies) return fail(c, SPHGB_ERR_ARGUMENT, "body index out of range");
    int rc;
    if (nbodies && (rc = check_finite(c, center, 3 * (size_t)nbodies, "body reference point"))) return rc;
    cudaSetDevice(c->cfg.device);
    CK(cudaStreamSynchronize(c->stream));
    free_bodies(c);
    invalidate_graphs(c);
    // prepared again at the next step: the body tables (and, with volume maps, the block partials
    // of their forces)
    c->prepared = false;
    if (nbodies == 0) return SPHGB_OK;
    c->body_of.assign(body, body + (body ? c->nb : 0u));
    c->body_center.assign(center, center + 3 * (size_t)nbodies);
    c->body_dynamic.assign(nbodies, 1);
    if (dynamic)
        for (uint32_t b = 0; b < nbodies; b++) c->body_dynamic[b] = dynamic[b] != 0;
    c->nbodies = nbodies;
    c->bmot.assign(18 * (size_t)nbodies, 0.0);   // every body at rest in its uploaded pose
    for (uint32_t b = 0; b < nbodies; b++)
        for (int k = 0; k < 3; k++) c->bmot[18 * (size_t)b + 4 * k] = 1.0;
    double *acc, *cen;
    unsigned *cnt;
    int *dyn;
    if ((rc = dalloc_into(c, c->body_allocs, &acc, 6 * (size_t)nbodies * sizeof(double))) ||
        (rc = dalloc_into(c, c->body_allocs, &cen, 3 * (size_t)nbodies * sizeof(double))) ||
        (rc = dalloc_into(c, c->body_allocs, &cnt, (size_t)nbodies * sizeof(unsigned))) ||
        (rc = dalloc_into(c, c->body_allocs, &dyn, (size_t)nbodies * sizeof(int)))) {
        free_bodies(c);
        return rc;
    }
    CK(cudaMemset(acc, 0, 6 * (size_t)nbodies * sizeof(double)));
    CK(cudaMemset(cnt, 0, (size_t)nbodies * sizeof(unsigned)));
    CK(cudaMemcpy(cen, center, 3 * (size_t)nbodies * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dyn, c->body_dynamic.data(), (size_t)nbodies * sizeof(int), cudaMemcpyHostToDevice));
    c->bodies.acc = acc;
    c->bodies.center = cen;
    c->bodies.counters = cnt;
    c->bodies.dynamic = dyn;
    c->bodies.nbodies = nbodies;
    return SPHGB_OK;
}

int sphgb_boundary_forces(sphgb_ctx *c, double *force, double *torque)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (c->nbodies == 0) return SPHGB_OK;
    cudaSetDevice(c->cfg.device);
    std::vector<double> acc(6 * (size_t)c->nbodies);
    CK(cudaMemcpyAsync(acc.data(), c->bodies.acc, acc.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (uint32_t b = 0; b < c->nbodies; b++)
        for (int d = 0; d < 3; d++) {
            if (force) force[3 * (size_t)b + d] = acc[6 * (size_t)b + d];
            if (torque) torque[3 * (size_t)b + d] = acc[6 * (size_t)b + 3 + d];
        }
    return SPHGB_OK;
}

int sphgb_clear_boundary_forces(sphgb_ctx *c, int32_t body)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (body >= 0 && (uint32_t)body >= c->nbodies) return fail(c, SPHGB_ERR_ARGUMENT, "body index out of range");
    if (c->nbodies == 0) return SPHGB_OK;
    cudaSetDevice(c->cfg.device);
    if (body < 0) CK(cudaMemsetAsync(c->bodies.acc, 0, 6 * (size_t)c->nbodies * sizeof(double), c->stream));
    else CK(cudaMemsetAsync(c->bodies.acc + 6 * (size_t)body, 0, 6 * sizeof(double), c->stream));
    return SPHGB_OK;
}

namespace {
// register a map whose node fields f0 / f1 (device, FP64) are filled: per-cell coefficients and
// the device table; the prepared set is rebuilt at the next step
int add_vmap(sphgb_ctx *c, sphgb_ctx::VMap &m, uint32_t *body)
{
    const VMapLayout L(m.res[0], m.res[1], m.res[2]);
    const size_t bytes = (size_t)L.cells() * 64 * real_size(c);
    cudaError_t e = cudaMalloc(&m.coef, bytes);
    if (e == cudaSuccess)
        e = c->fp64 ? vmap_expand_device<double>(m.res, m.f0, m.f1, (double *)m.coef, c->stream)
                    : vmap_expand_device<float>(m.res, m.f0, m.f1, (float *)m.coef, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        for (void *p : {(void *)m.f0, (void *)m.f1, m.coef})
            if (p) cudaFree(p);
        return fail(c, SPHGB_ERR_CUDA, std::string("volume map: ") + cudaGetErrorString(e));
    }
    c->vmaps.push_back(m);
    if (body) *body = (uint32_t)c->vmaps.size() - 1;
    const int rc = c->fp64 ? upload_vmaps<double>(c) : upload_vmaps<float>(c);
    c->prepared = false;
    invalidate_graphs(c);
    return rc;
}

int vmap_init(sphgb_ctx *c, sphgb_ctx::VMap &m, const uint32_t res[3], const double *rotation, const double *translation)
{
    uint64_t cells = 1;
    for (int k = 0; k < 3; k++) {
        if (res[k] == 0 || res[k] > 1024) return fail(c, SPHGB_ERR_ARGUMENT, "map resolution must be 1..1024 per axis");
        m.res[k] = res[k];
        cells *= res[k];
    }
    const VMapLayout L(res[0], res[1], res[2]);
    if (L.nodes() >= 0x7fffffffull || cells >= 0x7fffffffull) return fail(c, SPHGB_ERR_ARGUMENT, "map too large");
    static const double kI[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, kZ[3] = {0, 0, 0};
    std::memcpy(m.R, rotation ? rotation : kI, sizeof(m.R));
    std::memcpy(m.t, translation ? translation : kZ, sizeof(m.t));
    if (cudaMalloc(&m.f0, L.nodes() * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&m.f1, L.nodes() * sizeof(double)) != cudaSuccess) {
        if (m.f0) cudaFree(m.f0);
        cudaGetLastError();
        return fail(c, SPHGB_ERR_CUDA, "cudaMalloc of a volume map");
    }
    return SPHGB_OK;
}
}  // namespace

int sphgb_add_volume_map(sphgb_ctx *c, const double *vertices, uint32_t nv, const uint32_t *faces, uint32_t nf,
                         const uint32_t resolution[3], double thickness, int invert, const double rotation[9],
                         const double translation[3], uint32_t order, uint32_t *body)
{
    if (!c || !vertices || !faces || nv == 0 || nf == 0 || !resolution) return SPHGB_ERR_ARGUMENT;
    for (size_t k = 0; k < 3 * (size_t)nf; k++)
        if (faces[k] >= nv) return fail(c, SPHGB_ERR_ARGUMENT, "face index out of range");
    int rc = check_finite(c, vertices, 3 * (size_t)nv, "mesh vertex");
    if (rc) return rc;
    if (!std::isfinite(thickness)) return fail(c, SPHGB_ERR_NONFINITE, "non-finite map thickness");
    cudaSetDevice(c->cfg.device);
    sphgb_ctx::VMap m;
    if ((rc = vmap_init(c, m, resolution, rotation, translation))) return rc;
    m.support = 4.0 * c->prm.particle_radius;
    vmap_domain(vertices, nv, m.support, thickness, m.dmin, m.dmax);
    {   // the CFL radius of a moving body (SimulatorBase.cpp:2706-2729)
        double com[3] = {0, 0, 0};
        for (uint32_t k = 0; k < nv; k++)
            for (int d = 0; d < 3; d++) com[d] += vertices[3 * (size_t)k + d];
        for (int d = 0; d < 3; d++) com[d] /= (double)nv;
        for (uint32_t k = 0; k < nv; k++) {
            const double dx = vertices[3 * (size_t)k] - com[0], dy = vertices[3 * (size_t)k + 1] - com[1],
                         dz = vertices[3 * (size_t)k + 2] - com[2];
            m.max_dist = std::max(m.max_dist, std::sqrt(dx * dx + dy * dy + dz * dz));
        }
    }
    cudaError_t e = vmap_build_device(vertices, nv, faces, nf, m.res, m.support, thickness, invert, order ? order : 30u,
                                      m.f0, m.f1, m.dmin, m.dmax, c->stream);
    if (e != cudaSuccess) {
        cudaFree(m.f0);
        cudaFree(m.f1);
        return fail(c, SPHGB_ERR_CUDA, std::string("volume map construction: ") + cudaGetErrorString(e));
    }
    return add_vmap(c, m, body);
}

int sphgb_add_volume_map_values(sphgb_ctx *c, const uint32_t resolution[3], const double dmin[3], const double dmax[3],
                                const double *distance, const double *volume, const double rotation[9],
                                const double translation[3], uint32_t *body)
{
    if (!c || !resolution || !dmin || !dmax || !distance || !volume) return SPHGB_ERR_ARGUMENT;
    for (int k = 0; k < 3; k++)
        if (!(dmax[k] > dmin[k])) return fail(c, SPHGB_ERR_ARGUMENT, "empty map box");
    cudaSetDevice(c->cfg.device);
    sphgb_ctx::VMap m;
    int rc = vmap_init(c, m, resolution, rotation, translation);
    if (rc) return rc;
    const size_t nodes = VMapLayout(m.res[0], m.res[1], m.res[2]).nodes();
    if ((rc = check_finite(c, distance, nodes, "map distance")) || (rc = check_finite(c, volume, nodes, "map volume"))) {
        cudaFree(m.f0);
        cudaFree(m.f1);
        return rc;
    }
    std::memcpy(m.dmin, dmin, sizeof(m.dmin));
    std::memcpy(m.dmax, dmax, sizeof(m.dmax));
    m.support = 4.0 * c->prm.particle_radius;
    if (cudaMemcpy(m.f0, distance, nodes * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m.f1, volume, nodes * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(m.f0);
        cudaFree(m.f1);
        return fail(c, SPHGB_ERR_CUDA, "volume map upload");
    }
    return add_vmap(c, m, body);
}

int sphgb_get_volume_map(sphgb_ctx *c, uint32_t body, uint32_t resolution[3], double dmin[3], double dmax[3],
                         double *distance, double *volume)
{
    if (!c || body >= c->vmaps.size()) return SPHGB_ERR_ARGUMENT;
    const auto &m = c->vmaps[body];
    for (int k = 0; k < 3; k++) {
        if (resolution) resolution[k] = m.res[k];
        if (dmin) dmin[k] = m.dmin[k];
        if (dmax) dmax[k] = m.dmax[k];
    }
    const size_t nodes = VMapLayout(m.res[0], m.res[1], m.res[2]).nodes();
    cudaSetDevice(c->cfg.device);
    if (distance) CK(cudaMemcpy(distance, m.f0, nodes * sizeof(double), cudaMemcpyDeviceToHost));
    if (volume) CK(cudaMemcpy(volume, m.f1, nodes * sizeof(double), cudaMemcpyDeviceToHost));
    return SPHGB_OK;
}

int sphgb_clear_volume_maps(sphgb_ctx *c)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(c->cfg.device);
    CK(cudaStreamSynchronize(c->stream));
    free_vmaps(c);
    c->prepared = false;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_fluid_phase_viscosity(sphgb_ctx *c, uint32_t nphases, const double *viscosity,
                                    const double *viscosity_boundary)
{
    if (!c || nphases > 8 || (nphases > 0 && (!viscosity || !viscosity_boundary))) return SPHGB_ERR_ARGUMENT;
    for (uint32_t k = 0; k < nphases; k++)
        if (!(std::isfinite(viscosity[k]) && viscosity[k] >= 0.0 && std::isfinite(viscosity_boundary[k]) &&
              viscosity_boundary[k] >= 0.0))
            return fail(c, SPHGB_ERR_ARGUMENT, "a phase's viscosity must be finite and non-negative");
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    c->phase_nu.assign(viscosity, viscosity + nphases);
    c->phase_nub.assign(viscosity_boundary, viscosity_boundary + nphases);
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_fluid_phase_xsph(sphgb_ctx *c, uint32_t nphases, const double *xsph, const double *xsph_boundary)
{
    if (!c || nphases > 8 || (nphases > 0 && (!xsph || !xsph_boundary))) return SPHGB_ERR_ARGUMENT;
    for (uint32_t k = 0; k < nphases; k++)
        if (!(std::isfinite(xsph[k]) && std::isfinite(xsph_boundary[k])))
            return fail(c, SPHGB_ERR_ARGUMENT, "a phase's XSPH coefficient must be finite");
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    c->phase_xs.assign(xsph, xsph + nphases);
    c->phase_xsb.assign(xsph_boundary, xsph_boundary + nphases);
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_fluid_phases(sphgb_ctx *c, uint32_t nphases, const uint32_t *counts, const double *density0)
{
    if (!c || nphases > 8 || (nphases > 1 && (!counts || !density0))) return SPHGB_ERR_ARGUMENT;
    for (uint32_t k = 0; k < nphases && nphases > 1; k++)
        if (!(std::isfinite(density0[k]) && density0[k] > 0.0))
            return fail(c, SPHGB_ERR_ARGUMENT, "a phase's rest density must be positive");
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    if (nphases > 1) {
        c->phase_counts.assign(counts, counts + nphases);
        c->phase_rho0.assign(density0, density0 + nphases);
    } else {
        c->phase_counts.clear();
        c->phase_rho0.clear();
    }
    c->prepared = false;   // the per-slot rest densities
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_body_motion(sphgb_ctx *c, uint32_t body, const double rotation[9], const double translation[3],
                          const double velocity[3], const double omega[3])
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (c->boundary_method == 2)
        return fail(c, SPHGB_ERR_ARGUMENT, "volume-map bodies move with sphgb_set_volume_map_motion");
    if (body >= c->nbodies || c->nb == 0)
        return fail(c, SPHGB_ERR_ARGUMENT, "no such body of boundary particles (sphgb_set_boundary_bodies)");
    int rc;
    if ((rotation && (rc = check_finite(c, rotation, 9, "body rotation"))) ||
        (translation && (rc = check_finite(c, translation, 3, "body translation"))) ||
        (velocity && (rc = check_finite(c, velocity, 3, "body velocity"))) ||
        (omega && (rc = check_finite(c, omega, 3, "body angular velocity"))))
        return rc;
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    cudaSetDevice(c->cfg.device);
    double *q = c->bmot.data() + 18 * (size_t)body;
    if (rotation) std::copy(rotation, rotation + 9, q);
    if (translation) std::copy(translation, translation + 3, q + 9);
    for (int k = 0; k < 3; k++) {
        q[12 + k] = velocity ? velocity[k] : 0.0;
        q[15 + k] = omega ? omega[k] : 0.0;
    }
    if (!c->bmotion) {   // from now on the boundary particles are placed and sorted every step
        c->bmotion = true;
        c->bm_ready = false;
        invalidate_graphs(c);
    }
    c->bmot_dirty = true;
    if (translation && c->bodies.center) {   // the body's torque is taken about its position
        std::copy(translation, translation + 3, c->body_center.begin() + 3 * (size_t)body);
        CK(cudaMemcpyAsync(const_cast<double *>(c->bodies.center) + 3 * (size_t)body,
                           c->body_center.data() + 3 * (size_t)body, 3 * sizeof(double), cudaMemcpyHostToDevice,
                           c->stream));
    }
    return SPHGB_OK;
}

int sphgb_set_volume_map_scene(sphgb_ctx *c, uint32_t body, uint32_t scene)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (body >= c->vmaps.size()) return fail(c, SPHGB_ERR_ARGUMENT, "no such volume map");
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    c->vmaps[body].scene = scene;
    c->prepared = false;   // the scene-ordered maps and the boundary points per particle
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_set_volume_map_motion(sphgb_ctx *c, uint32_t body, const double rotation[9], const double translation[3],
                                const double velocity[3], const double omega[3])
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (body >= c->vmaps.size()) return fail(c, SPHGB_ERR_ARGUMENT, "no such volume map");
    int rc;
    if ((rotation && (rc = check_finite(c, rotation, 9, "map rotation"))) ||
        (translation && (rc = check_finite(c, translation, 3, "map translation"))) ||
        (velocity && (rc = check_finite(c, velocity, 3, "body velocity"))) ||
        (omega && (rc = check_finite(c, omega, 3, "body angular velocity"))))
        return rc;
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    cudaSetDevice(c->cfg.device);
    sphgb_ctx::VMap &m = c->vmaps[body];
    if (rotation) std::copy(rotation, rotation + 9, m.R);
    if (translation) std::copy(translation, translation + 3, m.t);
    for (int k = 0; k < 3; k++) {
        m.v[k] = velocity ? velocity[k] : 0.0;
        m.w[k] = omega ? omega[k] : 0.0;
    }
    bool move = false;
    for (const auto &q : c->vmaps)
        for (int k = 0; k < 3; k++) move = move || q.v[k] != 0.0 || q.w[k] != 0.0;
    if (move != c->vmove) {   // the kernels' parameters change
        c->vmove = move;
        invalidate_graphs(c);
    }
    c->vmaps_dirty = true;
    // a body's torque is taken about its position
    if (translation && c->nbodies == c->vmaps.size() && c->bodies.center) {
        std::copy(translation, translation + 3, c->body_center.begin() + 3 * (size_t)body);
        CK(cudaMemcpyAsync(const_cast<double *>(c->bodies.center) + 3 * (size_t)body, c->body_center.data() + 3 * (size_t)body,
                           3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    return SPHGB_OK;
}

int sphgb_set_boundary_method(sphgb_ctx *c, int method)
{
    if (!c || (method != 0 && method != 2)) return SPHGB_ERR_ARGUMENT;
    if (method == c->boundary_method) return SPHGB_OK;
    c->boundary_method = method;
    c->prepared = false;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_get_stream(const sphgb_ctx *c, void **stream)
{
    if (!c || !stream) return SPHGB_ERR_ARGUMENT;
    *stream = (void *)c->stream;
    return SPHGB_OK;
}

int sphgb_profile_enable(sphgb_ctx *c, int on)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    c->profile = on != 0;
    return SPHGB_OK;
}

int sphgb_profile_reset(sphgb_ctx *c)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    for (int k = 0; k < K_COUNT; k++) { c->prof_count[k] = 0; c->prof_ms[k] = 0.0; }
    return SPHGB_OK;
}

int sphgb_profile_read(const sphgb_ctx *c, int index, const char **name, uint64_t *launches, double *total_ms)
{
    if (!c || index < 0 || index >= K_COUNT) return SPHGB_ERR_ARGUMENT;
    if (name) *name = kKernelNames[index];
    if (launches) *launches = c->prof_count[index];
    if (total_ms) *total_ms = c->prof_ms[index];
    return SPHGB_OK;
}

int sphgb_num_particles(const sphgb_ctx *c, uint32_t *n, uint32_t *nb)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    if (n) *n = c->n;
    if (nb) *nb = c->nb;
    return SPHGB_OK;
}

// The device's address of a buffer its kernels can read and write: page-locked host memory
// mapped into its address space (cudaHostAlloc, cudaHostRegister on a unified address space) or
// memory of the context's own device, else null.  Such a buffer is read or written by the
// transfer kernels themselves, with no staging copy.
void *device_addressable(const void *p, int device)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice && a.device == device) return a.devicePointer;
    return nullptr;
}

int sphgb_download_fields(sphgb_ctx *c, uint32_t count, const int *fields, void *const *dsts, int dtype)
{
    if (!c || (count && (!fields || !dsts))) return SPHGB_ERR_ARGUMENT;
    if (dtype < SPHGB_DTYPE_F32 || dtype > SPHGB_DTYPE_U32) return fail(c, SPHGB_ERR_ARGUMENT, "unknown dtype");
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    cudaSetDevice(c->cfg.device);
    // checks; fluid fields into mapped host memory or device memory are written in particle-id
    // order by the device, the others get a place in the staging buffer
    std::vector<size_t> off(count + 1, 0);
    std::vector<void *> direct(count, nullptr);
    bool bfields = false, any_direct = false;
    for (uint32_t k = 0; k < count; k++) {
        const int field = fields[k];
        if (!dsts[k]) return SPHGB_ERR_ARGUMENT;
        if (field < 0 || field > SPHGB_FIELD_OBJECT_ID) return fail(c, SPHGB_ERR_ARGUMENT, "unknown field");
        if (field == SPHGB_FIELD_FEATURES && !c->mlp_x) return fail(c, SPHGB_ERR_STATE, "features are not computed");
        const bool bfield = field == SPHGB_FIELD_BOUNDARY_VOLUME || field == SPHGB_FIELD_BOUNDARY_POSITION;
        bfields = bfields || bfield;
        if (!bfield) direct[k] = device_addressable(dsts[k], c->cfg.device);
        any_direct = any_direct || direct[k];
        const size_t m = bfield ? c->nb : c->n;
        off[k + 1] = off[k] + (direct[k] ? 0 : ((m * field_components(field) * dtype_size(dtype) + 255) & ~(size_t)255));
    }
    if (bfields && !c->prepared) {
        int rc = c->fp64 ? prepare<double>(c) : prepare<float>(c);
        if (rc) return rc;
    }
    if (off[count] == 0 && (!any_direct || c->n == 0)) return SPHGB_OK;
    if (off[count]) {
        int rc = ensure_staging(c, off[count]);
        if (rc) return rc;
    }
    // every field queued back to back, one wait: written straight to mapped host or device
    // memory, or scattered to particle-id order in the staging buffer and copied out
    auto emit = [&](auto P, auto B) -> int {
        if (any_direct && c->n) {   // the mapped fields, up to kFieldSetMax per launch
            launch_inverse_perm(P, B.id, c->inv_perm, c->stream);
            FieldSet F{};
            for (uint32_t k = 0; k <= count; k++) {
                if (F.n == kFieldSetMax || (k == count && F.n)) {
                    launch_gather_fields(P, B, F, dtype, c->inv_perm, c->stream);
                    CK(cudaGetLastError());
                    F.n = 0;
                }
                if (k == count || !direct[k]) continue;
                F.ptr[F.n] = direct[k];
                F.field[F.n] = fields[k];
                F.comps[F.n] = (uint32_t)field_components(fields[k]);
                F.n++;
            }
        }
        for (uint32_t k = 0; k < count; k++) {
            const int field = fields[k];
            const bool bfield = field == SPHGB_FIELD_BOUNDARY_VOLUME || field == SPHGB_FIELD_BOUNDARY_POSITION;
            const size_t bytes = (size_t)(bfield ? c->nb : c->n) * field_components(field) * dtype_size(dtype);
            if (bytes == 0 || direct[k]) continue;
            char *st = static_cast<char *>(c->staging) + off[k];
            launch_scatter_field(P, B, field, st, dtype, c->stream);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(dsts[k], st, bytes, cudaMemcpyDeviceToHost, c->stream));
        }
        return SPHGB_OK;
    };
    const int rc = c->fp64 ? emit(make_params<double>(c), make_bufs<double>(c, 0))
                           : emit(make_params<float>(c), make_bufs<float>(c, 0));
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

int sphgb_download(sphgb_ctx *c, int field, void *dst, int dtype)
{
    if (!c || !dst) return SPHGB_ERR_ARGUMENT;
    return sphgb_download_fields(c, 1u, &field, &dst, dtype);
}

int sphgb_upload_fields(sphgb_ctx *c, uint32_t count, const int *fields, const void *const *srcs, int dtype)
{
    if (!c || (count && (!fields || !srcs))) return SPHGB_ERR_ARGUMENT;
    for (uint32_t k = 0; k < count; k++) {
        const int field = fields[k];
        if (!srcs[k]) return SPHGB_ERR_ARGUMENT;
        if (field != SPHGB_FIELD_POSITION && field != SPHGB_FIELD_VELOCITY && field != SPHGB_FIELD_VDIFF &&
            field != SPHGB_FIELD_PRESSURE_RHO2 && field != SPHGB_FIELD_PRESSURE_RHO2_V &&
            field != SPHGB_FIELD_POSITION_HI && field != SPHGB_FIELD_POSITION_LO)
            return fail(c, SPHGB_ERR_ARGUMENT, "field is not uploadable");
    }
    if (dtype != SPHGB_DTYPE_F32 && dtype != SPHGB_DTYPE_F64) return fail(c, SPHGB_ERR_ARGUMENT, "bad dtype");
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    cudaSetDevice(c->cfg.device);
    sphgb_stats st;
    if (c->step_pending) fill_stats(c, &st);
    // fields in mapped host memory or device memory are read by the device directly, the others
    // staged
    std::vector<size_t> off(count + 1, 0);
    std::vector<const void *> in(count, nullptr);
    for (uint32_t k = 0; k < count; k++) {
        in[k] = device_addressable(srcs[k], c->cfg.device);
        off[k + 1] = off[k] + (in[k] ? 0 : (((size_t)c->n * field_components(fields[k]) * dtype_size(dtype) + 255) &
                                            ~(size_t)255));
    }
    if (c->n == 0 || count == 0) return SPHGB_OK;
    if (off[count]) {
        int rc = ensure_staging(c, off[count]);
        if (rc) return rc;
    }
    // every staged field copied in, the inverse permutation once, then each field written by id;
    // one wait
    for (uint32_t k = 0; k < count; k++) {
        if (in[k]) continue;
        in[k] = static_cast<const char *>(c->staging) + off[k];
        CK(cudaMemcpyAsync(const_cast<void *>(in[k]), srcs[k],
                           (size_t)c->n * field_components(fields[k]) * dtype_size(dtype), cudaMemcpyHostToDevice,
                           c->stream));
    }
    auto write = [&](auto P, auto B) {
        launch_inverse_perm(P, B.id, c->inv_perm, c->stream);
        FieldSet F{};   // up to kFieldSetMax fields per launch, in the order given
        for (uint32_t k = 0; k < count; k++) {
            F.ptr[F.n] = const_cast<void *>(in[k]);
            F.field[F.n] = fields[k];
            F.comps[F.n] = (uint32_t)field_components(fields[k]);
            if (++F.n == kFieldSetMax || k + 1 == count) {
                launch_upload_fields(P, B, F, dtype, c->inv_perm, c->stream);
                F.n = 0;
            }
        }
    };
    if (c->fp64) write(make_params<double>(c), make_bufs<double>(c, 0));
    else write(make_params<float>(c), make_bufs<float>(c, 0));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

int sphgb_upload_field(sphgb_ctx *c, int field, const void *src, int dtype)
{
    if (!c || !src) return SPHGB_ERR_ARGUMENT;
    return sphgb_upload_fields(c, 1u, &field, &src, dtype);
}

int sphgb_neighbors(sphgb_ctx *c, int kind, uint32_t *offsets, uint32_t *indices, size_t capacity)
{
    if (!c || !offsets || (kind != 0 && kind != 1)) return SPHGB_ERR_ARGUMENT;
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    cudaSetDevice(c->cfg.device);
    sphgb_stats st;
    if (c->step_pending) fill_stats(c, &st);
    const uint32_t n = c->n;
    std::vector<uint32_t> cnt(n);
    int rc = sphgb_download(c, kind == 0 ? SPHGB_FIELD_NUM_FLUID_NEIGHBORS : SPHGB_FIELD_NUM_BOUNDARY_NEIGHBORS,
                            cnt.data(), SPHGB_DTYPE_U32);
    if (rc) return rc;
    const uint32_t cap = kind == 0 ? c->cfg.max_fluid_neighbors : c->cfg.max_boundary_neighbors;
    offsets[0] = 0;
    for (uint32_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + std::min(cnt[i], cap);
    if (!indices) return SPHGB_OK;
    if (capacity < offsets[n]) return fail(c, SPHGB_ERR_CAPACITY, "index buffer too small");
    // the lists of the last step are indexed by the sorted order of that step,
    // which is the current state order (parity already flipped to it)
    uint32_t *doff, *dout;
    if ((rc = dalloc(c, &doff, ((size_t)n + 1) * 4))) return rc;
    if ((rc = dalloc(c, &dout, (size_t)std::max<uint32_t>(offsets[n], 1) * 4))) return rc;
    CK(cudaMemcpy(doff, offsets, ((size_t)n + 1) * 4, cudaMemcpyHostToDevice));
    const uint32_t *id = c->set_id[c->parity];
    if (c->fp64) launch_inverse_perm<double>(make_params<double>(c), id, c->inv_perm, c->stream);
    else launch_inverse_perm<float>(make_params<float>(c), id, c->inv_perm, c->stream);
    launch_lists_to_ids(kind == 0 ? c->lf : c->lb, kind == 0 ? c->nfc : c->nbc, cap, id, c->inv_perm, c->bid, kind,
                        c->lpp_log2, doff, dout, n, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(indices, dout, (size_t)offsets[n] * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    dfree(c->allocs, dout);
    dfree(c->allocs, doff);
    return SPHGB_OK;
}

}  // extern "C"

// ===========================================================================
// Particle export (legacy VTK, ParticleExporter_VTK.cpp:25-266) from the device copy
// ===========================================================================
namespace {

// the reference's field names (FluidModel.cpp:61-67, TimeStepDFSPH.cpp:49-53, Viscosity_Weiler2018.cpp:33)
const char *field_name(int f)
{
    switch (f) {
    case SPHGB_FIELD_POSITION: return "position";
    case SPHGB_FIELD_VELOCITY: return "velocity";
    case SPHGB_FIELD_ACCELERATION: return "acceleration";
    case SPHGB_FIELD_DENSITY: return "density";
    case SPHGB_FIELD_FACTOR: return "factor";
    case SPHGB_FIELD_DENSITY_ADV: return "advected density";
    case SPHGB_FIELD_PRESSURE_RHO2: return "p / rho^2";
    case SPHGB_FIELD_PRESSURE_RHO2_V: return "p_v / rho^2";
    case SPHGB_FIELD_PRESSURE_ACCEL: return "pressure acceleration";
    case SPHGB_FIELD_VDIFF: return "velocity difference";
    case SPHGB_FIELD_PARTICLE_ID: return "id";
    case SPHGB_FIELD_FACTOR_RAW: return "factor raw";
    case SPHGB_FIELD_NUM_FLUID_NEIGHBORS: return "fluid neighbors";
    case SPHGB_FIELD_NUM_BOUNDARY_NEIGHBORS: return "boundary neighbors";
    case SPHGB_FIELD_FEATURES: return "features";
    case SPHGB_FIELD_POSITION_HI: return "position high";
    case SPHGB_FIELD_POSITION_LO: return "position low";
    case SPHGB_FIELD_STATE: return "state";
    case SPHGB_FIELD_OBJECT_ID: return "object_id";
    default: return nullptr;
    }
}

bool is_uint_field(int f)
{
    return f == SPHGB_FIELD_PARTICLE_ID || f == SPHGB_FIELD_NUM_FLUID_NEIGHBORS || f == SPHGB_FIELD_NUM_BOUNDARY_NEIGHBORS ||
           f == SPHGB_FIELD_STATE || f == SPHGB_FIELD_OBJECT_ID;
}

std::string vtk_name(const char *name)
{
    std::string out;
    for (const char *p = name; *p; p++) out += (*p == ' ' || *p == '\t' || *p == '\n') ? '_' : *p;
    return out;
}

uint32_t be32(uint32_t v)
{
    return ((v & 0xffu) << 24) | ((v & 0xff00u) << 8) | ((v >> 8) & 0xff00u) | (v >> 24);
}

struct ExportChunk {
    int field;          // -1: positions
    size_t offset;      // bytes into the staging buffer
    size_t count;       // words
    int word;           // bytes per word
    int comps;
};

// Writer thread: waits for the device copy, then writes the file from pinned memory.
void write_vtk(sphgb_ctx *c, std::string path, uint32_t n, std::vector<ExportChunk> chunks, bool real64)
{
    if (cudaEventSynchronize(c->export_copied) != cudaSuccess) {
        c->export_rc = SPHGB_ERR_CUDA;
        c->export_err = "export: device copy failed";
        return;
    }
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) {
        c->export_rc = SPHGB_ERR_ARGUMENT;
        c->export_err = "export: cannot open " + path;
        return;
    }
    const char *real_str = real64 ? " double\n" : " float\n";
    const char *base = static_cast<const char *>(c->export_host);
    fprintf(f, "# vtk DataFile Version 4.1\nSPlisHSPlasH particle data\nBINARY\nDATASET UNSTRUCTURED_GRID\n");
    fprintf(f, "POINTS %u%s", n, real_str);
    fwrite(base + chunks[0].offset, 1, chunks[0].count * chunks[0].word, f);
    fprintf(f, "\nCELLS %u %u\n", n, 2 * n);
    // particles are vertex cells (1, index); written in pieces
    std::vector<uint32_t> buf;
    const uint32_t piece = 1u << 16;
    const uint32_t one = be32(1u);
    for (uint32_t a = 0; a < n; a += piece) {
        const uint32_t b = std::min(n, a + piece);
        buf.resize(2 * (size_t)(b - a));
        for (uint32_t i = a; i < b; i++) { buf[2 * (size_t)(i - a)] = one; buf[2 * (size_t)(i - a) + 1] = be32(i); }
        fwrite(buf.data(), 4, buf.size(), f);
    }
    fprintf(f, "\nCELL_TYPES %u\n", n);
    buf.assign(std::min<size_t>(n, piece), one);
    for (uint32_t a = 0; a < n; a += piece) fwrite(buf.data(), 4, std::min(n, a + piece) - a, f);
    fprintf(f, "\nPOINT_DATA %u\nSCALARS id unsigned_int 1\nLOOKUP_TABLE id_table\n", n);
    fwrite(base + chunks[1].offset, 1, chunks[1].count * chunks[1].word, f);
    fprintf(f, "\nFIELD FieldData %zu\n", chunks.size() - 2);
    for (size_t k = 2; k < chunks.size(); k++) {
        const ExportChunk &ch = chunks[k];
        fprintf(f, "%s %d %u%s", vtk_name(field_name(ch.field)).c_str(), ch.comps, n,
                is_uint_field(ch.field) ? " unsigned_int\n" : real_str);
        fwrite(base + ch.offset, 1, ch.count * ch.word, f);
        fprintf(f, "\n");
    }
    if (fclose(f) != 0) {
        c->export_rc = SPHGB_ERR_ARGUMENT;
        c->export_err = "export: write failed for " + path;
    }
}

// Writer thread of the BGEO export: waits for the device copy of the packed records
void write_bgeo(sphgb_ctx *c, std::string path, uint32_t n, uint32_t words, std::vector<BgeoAttr> attrs, int level)
{
    if (cudaEventSynchronize(c->export_copied) != cudaSuccess) {
        c->export_rc = SPHGB_ERR_CUDA;
        c->export_err = "export: device copy failed";
        return;
    }
    std::string err;
    const int rc = write_bgeo_file(path, c->export_host, n, words, attrs, level, err);
    if (rc) {
        c->export_rc = rc;
        c->export_err = err;
    }
}

int export_join(sphgb_ctx *c)
{
    if (c->export_thread.joinable()) c->export_thread.join();
    const int rc = c->export_rc;
    if (rc) c->err = c->export_err;
    c->export_rc = SPHGB_OK;
    return rc;
}

}  // namespace

extern "C" {

int sphgb_export_wait(sphgb_ctx *c)
{
    if (!c) return SPHGB_ERR_ARGUMENT;
    return export_join(c);
}

int sphgb_export_vtk(sphgb_ctx *c, const char *path, const int *fields, uint32_t nfields, int wait)
{
    if (!c || !path || (nfields && !fields)) return SPHGB_ERR_ARGUMENT;
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    cudaSetDevice(c->cfg.device);
    int rc = export_join(c);   // one export in flight at a time
    if (rc) return rc;
    for (uint32_t k = 0; k < nfields; k++) {
        const int f = fields[k];
        if (!field_name(f) || f == SPHGB_FIELD_POSITION)
            return fail(c, SPHGB_ERR_ARGUMENT, "field cannot be exported (boundary fields, or position twice)");
        if (f == SPHGB_FIELD_FEATURES && !c->mlp_x) return fail(c, SPHGB_ERR_STATE, "features are not computed");
    }
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    const uint32_t n = c->n;
    const int rword = c->fp64 ? 8 : 4;
    // staging layout: positions, ids, then the requested fields; every chunk 256-byte aligned
    std::vector<ExportChunk> chunks;
    size_t off = 0;
    auto add = [&](int field, int comps, int word) {
        chunks.push_back({field, off, (size_t)n * comps, word, comps});
        off += ((size_t)n * comps * word + 255) / 256 * 256;
    };
    add(-1, 3, rword);
    add(SPHGB_FIELD_PARTICLE_ID, 1, 4);
    for (uint32_t k = 0; k < nfields; k++)
        add(fields[k], field_components(fields[k]), is_uint_field(fields[k]) ? 4 : rword);
    const size_t bytes = std::max<size_t>(off, 256);
    if (c->export_dev_bytes < bytes) {
        if (c->export_dev) cudaFree(c->export_dev);
        c->export_dev = nullptr;
        c->export_dev_bytes = 0;
        CK(cudaMalloc(&c->export_dev, bytes));
        c->export_dev_bytes = bytes;
    }
    if (c->export_host_bytes < bytes) {
        if (c->export_host) cudaFreeHost(c->export_host);
        c->export_host = nullptr;
        c->export_host_bytes = 0;
        CK(cudaMallocHost(&c->export_host, bytes));
        c->export_host_bytes = bytes;
    }
    if (!c->export_stream) {
        CK(cudaStreamCreateWithFlags(&c->export_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->export_start, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->export_scattered, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->export_copied, cudaEventDisableTiming));
    }
    // the export reads the state the last step left; it follows that step on its own stream
    CK(cudaEventRecord(c->export_start, c->stream));
    CK(cudaStreamWaitEvent(c->export_stream, c->export_start, 0));
    char *dev = static_cast<char *>(c->export_dev);
    for (const ExportChunk &ch : chunks) {
        const int field = ch.field < 0 ? SPHGB_FIELD_POSITION : ch.field;
        const int dt = is_uint_field(field) ? SPHGB_DTYPE_U32 : (c->fp64 ? SPHGB_DTYPE_F64 : SPHGB_DTYPE_F32);
        if (c->fp64) {
            launch_scatter_field<double>(make_params<double>(c), make_bufs<double>(c, 0), field, dev + ch.offset, dt,
                                         c->export_stream);
        } else {
            launch_scatter_field<float>(make_params<float>(c), make_bufs<float>(c, 0), field, dev + ch.offset, dt,
                                        c->export_stream);
        }
        launch_byteswap(dev + ch.offset, ch.count, ch.word, c->export_stream);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->export_scattered, c->export_stream));
    // later steps write the state set only after the scatter has read it
    CK(cudaStreamWaitEvent(c->stream, c->export_scattered, 0));
    CK(cudaMemcpyAsync(c->export_host, c->export_dev, off, cudaMemcpyDeviceToHost, c->export_stream));
    CK(cudaEventRecord(c->export_copied, c->export_stream));
    c->export_rc = SPHGB_OK;
    c->export_thread = std::thread(write_vtk, c, std::string(path), n, chunks, c->fp64);
    return wait ? export_join(c) : SPHGB_OK;
}

int sphgb_field_id(const char *name)
{
    if (!name) return -1;
    for (int f = 0; f <= SPHGB_FIELD_OBJECT_ID; f++) {
        const char *fn = field_name(f);
        if (fn && std::strcmp(fn, name) == 0) return f;
    }
    return -1;
}

int sphgb_export_bgeo(sphgb_ctx *c, const char *path, const int *fields, uint32_t nfields, int level, int wait)
{
    if (!c || !path || (nfields && !fields)) return SPHGB_ERR_ARGUMENT;
    if (level < -1 || level > 9) return fail(c, SPHGB_ERR_ARGUMENT, "compression level must be -1 .. 9");
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    if (level != 0 && !bgeo_compression_available())
        return fail(c, SPHGB_ERR_STATE, "compressed BGEO needs zlib (libz.so.1), which could not be loaded");
    cudaSetDevice(c->cfg.device);
    int rc = export_join(c);   // one export in flight at a time
    if (rc) return rc;
    if (nfields + 2 > kBgeoMaxColumns) return fail(c, SPHGB_ERR_ARGUMENT, "too many fields");
    uint32_t words = 5;   // x, y, z, 1, id
    for (uint32_t k = 0; k < nfields; k++) {
        const int f = fields[k];
        if (!field_name(f) || f == SPHGB_FIELD_POSITION || f == SPHGB_FIELD_PARTICLE_ID)
            return fail(c, SPHGB_ERR_ARGUMENT, "field cannot be exported (boundary fields, position or id twice)");
        const int comps = field_components(f);
        if (comps != 1 && comps != 3)
            return fail(c, SPHGB_ERR_ARGUMENT, "BGEO carries scalar and 3-vector fields only");
        words += (uint32_t)comps;
    }
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    const uint32_t n = c->n;
    const int rword = c->fp64 ? 8 : 4;
    // device staging: the fields in particle-id order (256-byte aligned chunks), then the records
    std::vector<ExportChunk> chunks;
    size_t off = 0;
    auto add = [&](int field, int comps, int word) {
        chunks.push_back({field, off, (size_t)n * comps, word, comps});
        off += ((size_t)n * comps * word + 255) / 256 * 256;
    };
    add(-1, 3, rword);
    add(SPHGB_FIELD_PARTICLE_ID, 1, 4);
    for (uint32_t k = 0; k < nfields; k++)
        add(fields[k], field_components(fields[k]), is_uint_field(fields[k]) ? 4 : rword);
    const size_t rec_off = off, rec_bytes = (size_t)n * words * 4u;
    const size_t bytes = std::max<size_t>(rec_off + rec_bytes, 256);
    if (c->export_dev_bytes < bytes) {
        if (c->export_dev) cudaFree(c->export_dev);
        c->export_dev = nullptr;
        c->export_dev_bytes = 0;
        CK(cudaMalloc(&c->export_dev, bytes));
        c->export_dev_bytes = bytes;
    }
    if (c->export_host_bytes < std::max<size_t>(rec_bytes, 256)) {
        if (c->export_host) cudaFreeHost(c->export_host);
        c->export_host = nullptr;
        c->export_host_bytes = 0;
        CK(cudaMallocHost(&c->export_host, std::max<size_t>(rec_bytes, 256)));
        c->export_host_bytes = std::max<size_t>(rec_bytes, 256);
    }
    if (!c->export_stream) {
        CK(cudaStreamCreateWithFlags(&c->export_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->export_start, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->export_scattered, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->export_copied, cudaEventDisableTiming));
    }
    CK(cudaEventRecord(c->export_start, c->stream));
    CK(cudaStreamWaitEvent(c->export_stream, c->export_start, 0));
    char *dev = static_cast<char *>(c->export_dev);
    std::vector<BgeoColumn> cols;
    std::vector<BgeoAttr> attrs;
    for (const ExportChunk &ch : chunks) {
        const int field = ch.field < 0 ? SPHGB_FIELD_POSITION : ch.field;
        const bool u = is_uint_field(field);
        const int dt = u ? SPHGB_DTYPE_U32 : (c->fp64 ? SPHGB_DTYPE_F64 : SPHGB_DTYPE_F32);
        if (c->fp64) {
            launch_scatter_field<double>(make_params<double>(c), make_bufs<double>(c, 0), field, dev + ch.offset, dt,
                                         c->export_stream);
        } else {
            launch_scatter_field<float>(make_params<float>(c), make_bufs<float>(c, 0), field, dev + ch.offset, dt,
                                        c->export_stream);
        }
        cols.push_back({dev + ch.offset, (uint32_t)ch.comps, u ? 2u : (c->fp64 ? 1u : 0u)});
        if (ch.field < 0) cols.push_back({nullptr, 1u, 3u});   // the position's w = 1
        else attrs.push_back({ch.field == SPHGB_FIELD_PARTICLE_ID ? std::string("id") : std::string(field_name(ch.field)),
                              (uint32_t)ch.comps, u});
    }
    launch_bgeo_pack(cols.data(), (uint32_t)cols.size(), n, reinterpret_cast<uint32_t *>(dev + rec_off),
                     c->export_stream);
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->export_scattered, c->export_stream));
    CK(cudaStreamWaitEvent(c->stream, c->export_scattered, 0));
    if (rec_bytes) CK(cudaMemcpyAsync(c->export_host, dev + rec_off, rec_bytes, cudaMemcpyDeviceToHost, c->export_stream));
    CK(cudaEventRecord(c->export_copied, c->export_stream));
    c->export_rc = SPHGB_OK;
    c->export_thread = std::thread(write_bgeo, c, std::string(path), n, words, attrs, level);
    return wait ? export_join(c) : SPHGB_OK;
}

}  // extern "C"

// ===========================================================================
// State files (SimulatorBase::saveState / loadState, SimulatorBase.cpp:1689-1870), written
// from and read into the device copy.  Little-endian binary:
//   "SPHGBST1", uint32 abi, precision, scenes S, lanes_log2 (0xffffffff: not chosen yet),
//   sphgb_params, per scene {uint32 n, nb, prev_iters, pad; double dt, time, fmin[3], fmax[3]},
//   double boundary positions [nb x 3] (upload order),
//   uint32 ids [n] in device slot order, then in device slot order: position high part [n x 3]
//   (float in FP32 mode, double in FP64 mode), position low part [n x 3] (float), velocity,
//   velocity difference [n x 3], p / rho^2, p_v / rho^2 [n] (Real).
// Saving the slot order and the grid extents keeps the next radix sort and cell grid identical,
// so a loaded context continues bit for bit.
// ===========================================================================
namespace {

constexpr char kStateMagic[8] = {'S', 'P', 'H', 'G', 'B', 'S', 'T', '1'};

struct StateScene {
    uint32_t n, nb, prev_iters, pad;
    double dt, time, fmin[3], fmax[3];
};

// device slot order of the particles: the id of every occupied slot, scene by scene
int slot_ids(sphgb_ctx *c, std::vector<uint32_t> &ids)
{
    ids.resize(c->n);
    const uint32_t *dev = c->set_id[c->parity];
    if (c->scn.size() <= 1) {
        if (c->n) CK(cudaMemcpy(ids.data(), dev, (size_t)c->n * 4, cudaMemcpyDeviceToHost));
        return SPHGB_OK;
    }
    for (const SceneHost &h : c->scn)
        CK(cudaMemcpy(ids.data() + h.ustart, dev + h.pstart, (size_t)h.n * 4, cudaMemcpyDeviceToHost));
    return SPHGB_OK;
}

template <class V> bool put_vec(FILE *f, const std::vector<V> &v) { return fwrite(v.data(), sizeof(V), v.size(), f) == v.size(); }
template <class V> bool get_vec(FILE *f, std::vector<V> &v) { return fread(v.data(), sizeof(V), v.size(), f) == v.size(); }

// field in id order -> the same field in slot order
template <class V> std::vector<V> to_slots(const std::vector<V> &byid, const std::vector<uint32_t> &ids, int comps)
{
    std::vector<V> out(byid.size());
    for (size_t k = 0; k < ids.size(); k++)
        for (int q = 0; q < comps; q++) out[k * comps + q] = byid[(size_t)ids[k] * comps + q];
    return out;
}

}  // namespace

extern "C" {

int sphgb_save_state(sphgb_ctx *c, const char *path)
{
    if (!c || !path) return SPHGB_ERR_ARGUMENT;
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    cudaSetDevice(c->cfg.device);
    int rc;
    if (c->step_pending) {
        sphgb_stats st;
        fill_stats(c, &st);
    }
    const uint32_t n = c->n;
    std::vector<uint32_t> ids;
    if ((rc = slot_ids(c, ids))) return rc;
    const int rdt = c->fp64 ? SPHGB_DTYPE_F64 : SPHGB_DTYPE_F32;
    // fields in id order (Real or float), reordered to slot order
    auto grab_real = [&](int field, int comps, std::vector<char> &out) -> int {
        const size_t w = c->fp64 ? 8 : 4;
        std::vector<char> byid((size_t)n * comps * w);
        int r = n ? sphgb_download(c, field, byid.data(), rdt) : SPHGB_OK;
        if (r) return r;
        out.resize(byid.size());
        for (size_t k = 0; k < n; k++)
            std::memcpy(out.data() + k * comps * w, byid.data() + (size_t)ids[k] * comps * w, comps * w);
        return SPHGB_OK;
    };
    std::vector<char> xhi, vel, vdiff, kp, kv;
    std::vector<float> xlo_id((size_t)n * 3);
    if ((rc = grab_real(SPHGB_FIELD_POSITION_HI, 3, xhi))) return rc;
    if (n && (rc = sphgb_download(c, SPHGB_FIELD_POSITION_LO, xlo_id.data(), SPHGB_DTYPE_F32))) return rc;
    if ((rc = grab_real(SPHGB_FIELD_VELOCITY, 3, vel))) return rc;
    if ((rc = grab_real(SPHGB_FIELD_VDIFF, 3, vdiff))) return rc;
    if ((rc = grab_real(SPHGB_FIELD_PRESSURE_RHO2, 1, kp))) return rc;
    if ((rc = grab_real(SPHGB_FIELD_PRESSURE_RHO2_V, 1, kv))) return rc;
    const std::vector<float> xlo = to_slots(xlo_id, ids, 3);

    FILE *f = fopen(path, "wb");
    if (!f) return fail(c, SPHGB_ERR_ARGUMENT, std::string("cannot open ") + path);
    const uint32_t S = (uint32_t)c->scn.size();
    const uint32_t hdr[4] = {SPHGB_ABI_VERSION, c->fp64 ? 1u : 0u, S, c->tuned ? c->lpp_log2 : 0xffffffffu};
    bool ok = fwrite(kStateMagic, 1, 8, f) == 8 && fwrite(hdr, 4, 4, f) == 4 && fwrite(&c->prm, sizeof(sphgb_params), 1, f) == 1;
    for (uint32_t s = 0; s < S && ok; s++) {
        const SceneHost &h = c->scn[s];
        StateScene r{h.n, h.nb, h.prev_iters, 0, h.dt, h.time, {h.fmin[0], h.fmin[1], h.fmin[2]},
                     {h.fmax[0], h.fmax[1], h.fmax[2]}};
        ok = fwrite(&r, sizeof r, 1, f) == 1;
    }
    ok = ok && put_vec(f, c->hb) && put_vec(f, ids) && put_vec(f, xhi) && put_vec(f, xlo) && put_vec(f, vel) &&
         put_vec(f, vdiff) && put_vec(f, kp) && put_vec(f, kv);
    if (fclose(f) != 0) ok = false;
    return ok ? SPHGB_OK : fail(c, SPHGB_ERR_ARGUMENT, std::string("write failed: ") + path);
}

int sphgb_load_state(sphgb_ctx *c, const char *path)
{
    if (!c || !path) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(c->cfg.device);
    FILE *f = fopen(path, "rb");
    if (!f) return fail(c, SPHGB_ERR_ARGUMENT, std::string("cannot open ") + path);
    struct Closer { FILE *f; ~Closer() { fclose(f); } } closer{f};
    char magic[8];
    uint32_t hdr[4];
    sphgb_params prm;
    if (fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kStateMagic, 8) != 0 || fread(hdr, 4, 4, f) != 4 ||
        fread(&prm, sizeof prm, 1, f) != 1)
        return fail(c, SPHGB_ERR_ARGUMENT, "not a state file of this library");
    if (hdr[0] != SPHGB_ABI_VERSION) return fail(c, SPHGB_ERR_ARGUMENT, "state file of another ABI version");
    if ((hdr[1] != 0) != c->fp64) return fail(c, SPHGB_ERR_ARGUMENT, "state file of the other precision");
    const uint32_t S = hdr[2];
    if (S == 0 || S > (1u << 24)) return fail(c, SPHGB_ERR_ARGUMENT, "bad scene count in state file");
    std::vector<StateScene> sc(S);
    if (!get_vec(f, sc)) return fail(c, SPHGB_ERR_ARGUMENT, "truncated state file");
    size_t n = 0, nb = 0;
    std::vector<uint32_t> counts(S), bcounts(S);
    for (uint32_t s = 0; s < S; s++) {
        counts[s] = sc[s].n;
        bcounts[s] = sc[s].nb;
        n += sc[s].n;
        nb += sc[s].nb;
    }
    if (n >= 0xffffffffull || nb >= 0xffffffffull) return fail(c, SPHGB_ERR_ARGUMENT, "bad particle counts in state file");
    const size_t w = c->fp64 ? 8 : 4;
    std::vector<double> hb(nb * 3);
    std::vector<uint32_t> ids(n);
    std::vector<char> xhi(n * 3 * w), vel(n * 3 * w), vdiff(n * 3 * w), kp(n * w), kv(n * w);
    std::vector<float> xlo(n * 3);
    if (!get_vec(f, hb) || !get_vec(f, ids) || !get_vec(f, xhi) || !get_vec(f, xlo) || !get_vec(f, vel) ||
        !get_vec(f, vdiff) || !get_vec(f, kp) || !get_vec(f, kv))
        return fail(c, SPHGB_ERR_ARGUMENT, "truncated state file");
    std::vector<char> seen(n, 0);
    for (uint32_t id : ids) {
        if (id >= n || seen[id]) return fail(c, SPHGB_ERR_ARGUMENT, "particle ids in the state file are not a permutation");
        seen[id] = 1;
    }
    int rc;
    if ((rc = sphgb_set_params(c, &prm))) return rc;
    // fluid in the saved slot order with the saved ids (positions / velocities as double)
    std::vector<double> x(n * 3), v(n * 3);
    for (size_t k = 0; k < n * 3; k++) {
        double hi, vv;
        if (c->fp64) { std::memcpy(&hi, xhi.data() + k * 8, 8); std::memcpy(&vv, vel.data() + k * 8, 8); }
        else {
            float a, b;
            std::memcpy(&a, xhi.data() + k * 4, 4);
            std::memcpy(&b, vel.data() + k * 4, 4);
            hi = a;
            vv = b;
        }
        x[k] = hi;
        v[k] = vv;
    }
    c->scn.clear();
    c->hb.clear();
    c->nb = 0;
    c->have_boundary = false;
    rc = c->fp64 ? init_scenes<double>(c, x.data(), v.data(), ids.data(), counts)
                 : init_scenes<float>(c, x.data(), v.data(), ids.data(), counts);
    if (rc) return rc;
    static const double kNone[3] = {0, 0, 0};
    if ((rc = set_boundary(c, nb ? hb.data() : kNone, bcounts))) return rc;
    // exact fields in id order
    auto by_id = [&](const std::vector<char> &slots, int comps) {
        std::vector<char> out(slots.size());
        const size_t e = comps * w;
        for (size_t k = 0; k < n; k++) std::memcpy(out.data() + (size_t)ids[k] * e, slots.data() + k * e, e);
        return out;
    };
    std::vector<float> xlo_id(n * 3);
    for (size_t k = 0; k < n; k++)
        for (int q = 0; q < 3; q++) xlo_id[(size_t)ids[k] * 3 + q] = xlo[k * 3 + q];
    const int rdt = c->fp64 ? SPHGB_DTYPE_F64 : SPHGB_DTYPE_F32;
    if (n) {
        const std::vector<char> a = by_id(xhi, 3), b = by_id(vdiff, 3), d = by_id(kp, 1), e = by_id(kv, 1);
        if ((rc = sphgb_upload_field(c, SPHGB_FIELD_POSITION_HI, a.data(), rdt))) return rc;
        if ((rc = sphgb_upload_field(c, SPHGB_FIELD_POSITION_LO, xlo_id.data(), SPHGB_DTYPE_F32))) return rc;
        if ((rc = sphgb_upload_field(c, SPHGB_FIELD_VDIFF, b.data(), rdt))) return rc;
        if ((rc = sphgb_upload_field(c, SPHGB_FIELD_PRESSURE_RHO2, d.data(), rdt))) return rc;
        if ((rc = sphgb_upload_field(c, SPHGB_FIELD_PRESSURE_RHO2_V, e.data(), rdt))) return rc;
    }
    // per-scene step size, time, CFL history and the grid extents fixed at the original upload
    for (uint32_t s = 0; s < S; s++) {
        SceneHost &h = c->scn[s];
        h.dt = sc[s].dt;
        h.time = sc[s].time;
        h.prev_iters = sc[s].prev_iters;
        for (int d = 0; d < 3; d++) { h.fmin[d] = sc[s].fmin[d]; h.fmax[d] = sc[s].fmax[d]; }
    }
    if (hdr[3] <= 2) {   // the lanes per particle the saved context ran with
        c->lpp_log2 = hdr[3];
        c->staged = c->lpp_log2 == 0 && staging_possible(c);
        c->tuned = true;
    }
    c->dt = c->scn[0].dt;
    c->scalars_dirty = true;
    invalidate_graphs(c);
    return SPHGB_OK;
}

int sphgb_save_particle_state(sphgb_ctx *c, const char *path, int level)
{
    if (!c || !path) return SPHGB_ERR_ARGUMENT;
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    if (c->nscenes() != 1 || c->phase_counts.size() > 1)
        return fail(c, SPHGB_ERR_STATE, "a particle state file holds one fluid model of one scene");
    // the storeData fields of FluidModel, TimeStepDFSPH and Viscosity_Weiler2018, in that order
    // (FluidModel.cpp:61-66, TimeStepDFSPH.cpp:51-52, Viscosity_Weiler2018.cpp:33); the position
    // and "id" are the exporter's first attributes
    std::vector<int> fields = {SPHGB_FIELD_STATE, SPHGB_FIELD_OBJECT_ID, SPHGB_FIELD_VELOCITY,
                               SPHGB_FIELD_PRESSURE_RHO2, SPHGB_FIELD_PRESSURE_RHO2_V};
    if (c->prm.viscosity_method == 6) fields.push_back(SPHGB_FIELD_VDIFF);
    return sphgb_export_bgeo(c, path, fields.data(), (uint32_t)fields.size(), level, 1);
}

int sphgb_load_particle_state(sphgb_ctx *c, const char *path)
{
    if (!c || !path) return SPHGB_ERR_ARGUMENT;
    if (!c->have_fluid) return fail(c, SPHGB_ERR_STATE, "no fluid uploaded");
    if (c->nscenes() != 1 || c->phase_counts.size() > 1)
        return fail(c, SPHGB_ERR_STATE, "a particle state file holds one fluid model of one scene");
    BgeoPoints pts;
    std::string err;
    int rc = read_bgeo_file(path, pts, err);
    if (rc) return fail(c, rc, err.c_str());
    const uint32_t n = c->n;
    if (pts.n != n) return fail(c, SPHGB_ERR_ARGUMENT, "the file's point count differs from the fluid's");
    // record r -> particle id (the "id" attribute; the record order without one)
    std::vector<uint32_t> id(n);
    for (uint32_t r = 0; r < n; r++) id[r] = r;
    auto find = [&](const char *name, uint32_t comps, bool integer) -> const std::vector<uint32_t> * {
        for (size_t a = 0; a < pts.attrs.size(); a++)
            if (pts.attrs[a].name == name && pts.attrs[a].comps == comps && pts.attrs[a].integer == integer)
                return &pts.values[a];
        return nullptr;
    };
    if (const std::vector<uint32_t> *ids = find("id", 1, true)) {
        std::vector<char> seen(n, 0);
        for (uint32_t r = 0; r < n; r++) {
            const uint32_t d = (*ids)[r];
            if (d >= n || seen[d]) return fail(c, SPHGB_ERR_ARGUMENT, "the file's ids are not a permutation of 0 .. n-1");
            seen[d] = 1;
            id[r] = d;
        }
    }
    if (const std::vector<uint32_t> *state = find("state", 1, true))
        for (uint32_t r = 0; r < n; r++)
            if ((*state)[r] != 0u) return fail(c, SPHGB_ERR_ARGUMENT, "only Active particles (state 0) are supported");
    std::vector<double> buf;
    auto put = [&](int field, const std::vector<uint32_t> &v, uint32_t comps) -> int {
        buf.assign((size_t)n * comps, 0.0);
        for (uint32_t r = 0; r < n; r++)
            for (uint32_t k = 0; k < comps; k++) {
                float x;
                std::memcpy(&x, &v[(size_t)r * comps + k], 4);
                buf[(size_t)id[r] * comps + k] = (double)x;
            }
        return sphgb_upload_field(c, field, buf.data(), SPHGB_DTYPE_F64);
    };
    {
        std::vector<uint32_t> pos(pts.position.size());
        std::memcpy(pos.data(), pts.position.data(), pos.size() * 4);
        if ((rc = put(SPHGB_FIELD_POSITION, pos, 3))) return rc;
    }
    const struct { const char *name; int field; uint32_t comps; } map[] = {
        {"velocity", SPHGB_FIELD_VELOCITY, 3}, {"p / rho^2", SPHGB_FIELD_PRESSURE_RHO2, 1},
        {"p_v / rho^2", SPHGB_FIELD_PRESSURE_RHO2_V, 1}, {"velocity difference", SPHGB_FIELD_VDIFF, 3}};
    for (const auto &m : map)
        if (const std::vector<uint32_t> *v = find(m.name, m.comps, false))
            if ((rc = put(m.field, *v, m.comps))) return rc;
    return SPHGB_OK;
}

}  // extern "C"
