// sm_103a kernels of the DFSPH time step.  One thread per fluid slot, in the
// cell-sorted order of the current step.  Neighbour lists are built once per
// step (fused with densities, the DFSPH factor and the divergence source) and
// then re-read by every later pass; kernel gradients are recomputed from the
// positions in each pass (the whole position array stays in L2).
//
// Every launch covers all scenes of the context.  Scene s owns the slots
// [begin_s, end_s) of whole thread blocks, so all threads of a block belong to
// one scene: per-scene reductions, step sizes and loop decisions are block
// uniform.  Slots past a scene's last particle are idle (they hold no particle,
// appear in no cell and in no list).
//
// Reference restated (SPlisHSPlasH 2.16.0): TimeStep.cpp:35-169,
// DFSPH/TimeStepDFSPH.cpp:117-706 and the scalar kernels :1106-1420,
// XSPH.cpp:138-216, Viscosity/Viscosity_Weiler2018.cpp:271-443,605-742,891-1254,
// Simulation.cpp:395-493, BoundaryModel_Akinci2012.cpp:48-75.
#include "sph_ctx.h"

#include "../../include/sphgb300.h"

namespace sphgb {

namespace {

inline unsigned grid_for(uint32_t n) { return (n + kBlock - 1) / kBlock; }

// ---- slots, scenes and lanes per particle ---------------------------------
// A particle kernel runs LPP lanes per particle (LPP = 1 everywhere except the
// neighbour passes, which take LPP in {1, 2, 4}): the kBlock threads of a block
// cover kBlock / LPP consecutive slots, and the LPP lanes of a particle walk
// interleaved parts of its fluid list and combine their partial sums with warp
// shuffles.  A block never spans two scenes (scenes start at multiples of kBlock).
struct SlotInfo {
    uint32_t b;            // block (units of kBlock / LPP slots)
    uint32_t s;            // scene
    uint32_t i;            // slot
    uint32_t l;            // lane of the particle (0 .. LPP-1)
    uint32_t begin, end;   // the scene's slots holding particles
    bool act;              // slot i holds a particle
};

// NT: threads per block (kBlock except in the two solver passes, which may run 128 or 512); a
// block of 512 covers two scene tiles and runs for one scene only.
template <int LPP = 1, int NT = kBlock, class T> __device__ __forceinline__ SlotInfo slot_info(const DevParams<T> &P)
{
    constexpr uint32_t SPB = NT / LPP;                            // slots per block
    constexpr uint32_t PER = SPB <= kBlock ? kBlock / SPB : 1u;   // blocks per scene-table entry
    SlotInfo q;
    q.b = blockIdx.x;
    q.i = q.b * SPB + threadIdx.x / LPP;
    q.l = threadIdx.x % LPP;
    if (SPB <= kBlock && P.nscenes > 1) {
        const uint4 b = __ldg(P.blk + q.b / PER);
        q.s = b.x;
        q.begin = b.y;
        q.end = b.z;
    } else {
        q.s = 0;
        q.begin = 0;
        q.end = P.s0.n;
    }
    q.act = q.i < q.end;   // blocks never span scenes: i >= begin
    return q;
}

// reduction slot of the scene of this block
template <int LPP = 1, int NT = kBlock, class T>
__device__ __forceinline__ ReduceSlot scene_reduce(const DevParams<T> &P, const DevBufs<T> &B, const SlotInfo &q)
{
    constexpr uint32_t SPB = NT / LPP;
    constexpr uint32_t PER = SPB <= kBlock ? kBlock / SPB : 1u;
    ReduceSlot r;
    r.partials = B.partials;
    r.counter = B.counters + q.s;
    if (SPB <= kBlock && P.nscenes > 1) {
        // every block of the scene's padded slot range [begin, begin + kBlock * ceil(n / kBlock))
        // takes part, also those that hold no particle
        r.first = q.begin / SPB;
        r.count = (q.end - q.begin + kBlock - 1) / kBlock * PER;
    } else {
        r.first = 0;
        r.count = gridDim.x;
    }
    return r;
}

// sum over the LPP lanes of a particle (all 32 lanes of the warp must call it)
template <int LPP, class T> __device__ __forceinline__ T gsum(T v)
{
#pragma unroll
    for (int o = LPP >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int LPP, class T> __device__ __forceinline__ V3<T> gsum3(V3<T> v)
{
    return V3<T>{gsum<LPP>(v.x), gsum<LPP>(v.y), gsum<LPP>(v.z)};
}

// Loop decision of the batch.  Called by the thread that finalized a scene's
// reduction, after it stored the scene's own decision in sc[s].cont; the last
// scene to arrive stores the OR over all scenes in the global record and in the
// graph's loop condition.  A loop stopped by the guard stays stopped.
// The scenes that call it are every scene (all_scenes: the first kernel of a loop) or the scenes
// live at the launch, whose number the previous decision left in the global record: the blocks
// of a scene whose loop has stopped return before any work and never get here.  The last scene
// to decide counts the scenes that continue for the next launch.
template <class T>
__device__ __forceinline__ void batch_decide(const DevParams<T> &P, const DevBufs<T> &B, cudaGraphConditionalHandle h,
                                             int use_handle, bool all_scenes)
{
    unsigned any;
    if (P.nscenes == 1) {
        any = B.sc[0].cont;
    } else {
        const unsigned expect = all_scenes ? P.nscenes : __ldcg(&B.gsc->live);
        __threadfence();
        const unsigned t = atomicAdd(B.counters + P.nscenes, 1u);
        if (t != expect - 1) return;
        __threadfence();
        any = 0;
        for (uint32_t s = 0; s < P.nscenes; s++) any += __ldcg(&B.sc[s].cont) != 0u ? 1u : 0u;
        B.counters[P.nscenes] = 0;
        B.gsc->live = any;
    }
    if (B.gsc->flags & kFlagLoopGuard) any = 0;
    B.gsc->cont = any ? 1u : 0u;
    if (use_handle) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// ---- list access --------------------------------------------------------
// Boundary lists: warp-interleaved, entry k of particle i at (i / 32) 32 cap + 32 k + i % 32.
__device__ __forceinline__ const uint32_t *list_ptr(const uint32_t *L, uint32_t i, uint32_t cap)
{
    return L + (size_t)(i >> 5) * cap * 32u + (i & 31u);
}
__device__ __forceinline__ uint32_t *list_ptr(uint32_t *L, uint32_t i, uint32_t cap)
{
    return L + (size_t)(i >> 5) * cap * 32u + (i & 31u);
}
// local fluid lists (staged passes): the warp-interleaved layout, entry k at + 32 k
__device__ __forceinline__ const uint16_t *ll_ptr(const uint16_t *L, uint32_t i, uint32_t cap)
{
    return L + (size_t)(i >> 5) * cap * 32u + (i & 31u);
}
// Fluid lists in the layout of the neighbour passes' lanes per particle (lpp = 1 << lpp_log2):
// entry k of particle i at (i / G) G cap + 32 (k / lpp) + lpp (i % G) + k % lpp, G = 32 / lpp,
// so that one step of a warp (G particles x lpp entries) reads 32 consecutive words; lpp = 1
// is the warp-interleaved layout of the boundary lists.  cap is a multiple of 4.
__device__ __forceinline__ size_t fl_index(uint32_t i, uint32_t k, uint32_t cap, uint32_t lpp_log2)
{
    const uint32_t lpp = 1u << lpp_log2, G = 32u >> lpp_log2;
    return (size_t)(i / G) * G * cap + 32u * (k >> lpp_log2) + lpp * (i % G) + (k & (lpp - 1u));
}
// first entry of lane l of particle i; the lane's following entries are 32 words apart
template <int LPP> __device__ __forceinline__ const uint32_t *fl_lane(const uint32_t *L, uint32_t i, uint32_t l, uint32_t cap)
{
    constexpr uint32_t G = 32u / LPP;
    return L + (size_t)(i / G) * G * cap + LPP * (i % G) + l;
}
// entries of lane l among cnt entries dealt round-robin to LPP lanes
template <int LPP> __device__ __forceinline__ uint32_t lane_count(uint32_t cnt, uint32_t l)
{
    return cnt > l ? (cnt - l + LPP - 1) / LPP : 0u;
}

// gradW(r) = c r from the squared distance.  FP32: one reciprocal square root
// (MUFU) instead of a square root and a division; FP64: exact sqrt and division.
__device__ __forceinline__ float grad_coef_d2(const Kernel<float> &K, float d2)
{
    const float rinv = rsqrtf(fmaxf(d2, 1e-36f));
    const float rl = d2 * rinv;
    const float q = rl * K.invh;
    float c;
    if (q <= 0.5f) {
        c = K.l * K.invh2 * (3.0f * q - 2.0f);
    } else {
        const float f = 1.0f - q;
        c = -K.l * f * f * K.invh * rinv;
    }
    return (rl > 1.0e-9f && q <= 1.0f) ? c : 0.0f;
}
__device__ __forceinline__ double grad_coef_d2(const Kernel<double> &K, double d2)
{
    return kernel_gradW_coef(K, sqrt(d2));
}

// W(r) and the gradient coefficient from the squared distance (FP32: one rsqrt)
__device__ __forceinline__ void kernel_W_coef_d2(const Kernel<float> &K, float d2, float &W, float &c)
{
    const float rinv = rsqrtf(fmaxf(d2, 1e-36f));
    const float rl = d2 * rinv;
    const float q = rl * K.invh;
    if (q <= 0.5f) {
        const float q2 = q * q;
        W = K.k * (6.0f * q2 * q - 6.0f * q2 + 1.0f);
        c = K.l * K.invh2 * (3.0f * q - 2.0f);
    } else {
        const float f = 1.0f - q;
        W = K.k * (2.0f * f * f * f);
        c = -K.l * f * f * K.invh * rinv;
    }
    if (!(q <= 1.0f)) W = 0.0f;
    if (!(rl > 1.0e-9f && q <= 1.0f)) c = 0.0f;
}
__device__ __forceinline__ void kernel_W_coef_d2(const Kernel<double> &K, double d2, double &W, double &c)
{
    const double rl = sqrt(d2);
    W = kernel_W(K, rl);
    c = kernel_gradW_coef(K, rl);
}

// rest density of the particle in slot i: its fluid phase's (FluidModel::getDensity0), else density0
template <class T> __device__ __forceinline__ T rho0_at(const DevParams<T> &P, const DevBufs<T> &B, uint32_t i)
{
    return P.nphase > 1 ? B.r0[i] : P.rho0;
}
// Weiler2018 coefficients nu, nu_b of phase k, without dynamic indexing of the parameter arrays
template <class T> __device__ __forceinline__ void phase_visc(const DevParams<T> &P, uint32_t k, T &nu, T &nub)
{
    nu = P.phase_nu[0];
    nub = P.phase_nub[0];
#pragma unroll
    for (uint32_t q = 1; q < 8; q++)
        if (q == k) {
            nu = P.phase_nu[q];
            nub = P.phase_nub[q];
        }
}
// XSPH coefficients of phase k (fluid, boundary)
template <class T> __device__ __forceinline__ void phase_xsph(const DevParams<T> &P, uint32_t k, T &xs, T &xsb)
{
    xs = P.phase_xs[0];
    xsb = P.phase_xsb[0];
#pragma unroll
    for (uint32_t q = 1; q < 8; q++)
        if (q == k) {
            xs = P.phase_xs[q];
            xsb = P.phase_xsb[q];
        }
}
// particles of phase k (counted, rest density) without dynamic indexing of the parameter arrays
template <class T> __device__ __forceinline__ void phase_info(const DevParams<T> &P, int k, uint32_t &count, T &rho0)
{
    count = P.phase_count[0];
    rho0 = P.phase_rho0[0];
#pragma unroll
    for (int q = 1; q < 8; q++)
        if (q == k) {
            count = P.phase_count[q];
            rho0 = P.phase_rho0[q];
        }
}

template <class T> __device__ __forceinline__ V3<T> diff3(const v4_t<T> &a, const v4_t<T> &b)
{
    return V3<T>{(T)a.x - (T)b.x, (T)a.y - (T)b.y, (T)a.z - (T)b.z};
}

// A list entry: read once per pass, so it is not kept in L1, where it would displace the
// neighbour records that the gathers reuse
__device__ __forceinline__ uint32_t ld_list(const uint32_t *p)
{
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ld_list(const uint16_t *p) { return __ldg(p); }
// ... and one that the reading thread itself wrote earlier in the same kernel (the list build):
// a coherent load, also without L1 allocation
__device__ __forceinline__ uint32_t ld_own_list(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.global.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Neighbour loop with U independent index loads, then U dependent gathers, then
// U computations, so that each thread keeps several loads in flight.  Idx: uint32_t for
// the lists of global slots, uint16_t for the local lists of the staged passes.  OWN: the
// list was written by this thread in the same kernel.
template <int U, uint32_t STRIDE = 32u, bool OWN = false, class Idx, class Ld, class Cp>
__device__ __forceinline__ void nbr_loop(const Idx *__restrict__ L, uint32_t cnt, Ld ld, Cp cp)
{
    auto idx = [&](uint32_t k) -> uint32_t {
        if constexpr (OWN) return ld_own_list(L + k * STRIDE);
        else return ld_list(L + k * STRIDE);
    };
    uint32_t k = 0;
    for (; k + U <= cnt; k += U) {
        uint32_t j[U];
#pragma unroll
        for (int u = 0; u < U; u++) j[u] = idx(k + u);
        decltype(ld(0u)) d[U];
#pragma unroll
        for (int u = 0; u < U; u++) d[u] = ld(j[u]);
#pragma unroll
        for (int u = 0; u < U; u++) cp(j[u], d[u]);
    }
    for (; k < cnt; k++) {
        const uint32_t jj = idx(k);
        cp(jj, ld(jj));
    }
}

// The fluid neighbours of particle i that lane l of its LPP lanes handles
template <int LPP, int U, class T, class Ld, class Cp>
__device__ __forceinline__ void fluid_loop(const DevParams<T> &P, const DevBufs<T> &B, uint32_t i, uint32_t l, Ld ld, Cp cp)
{
    const uint32_t nf = min(B.nf[i], P.capf);
    nbr_loop<U>(fl_lane<LPP>(B.lf, i, l, P.capf), lane_count<LPP>(nf, l), ld, cp);
}
// ... and its boundary neighbours (warp-interleaved boundary list, entries l, l + LPP, ...)
template <int LPP, class T, class Cp>
__device__ __forceinline__ void boundary_loop(const DevParams<T> &P, const DevBufs<T> &B, uint32_t i, uint32_t l, Cp cp)
{
    const uint32_t nb = min(B.nbn[i], P.capb);
    const uint32_t *L = list_ptr(B.lb, i, P.capb) + 32u * l;
    const uint32_t cnt = lane_count<LPP>(nb, l);
    for (uint32_t k = 0; k < cnt; k++) {
        const uint32_t j = ld_list(L + k * 32u * LPP);
        cp(j, ldv(B.xb, j));
    }
}

constexpr int kUnroll = 4;

__device__ __forceinline__ void cell_coords(uint32_t c, int dimx, int dimy, int &cx, int &cy, int &cz)
{
    cx = (int)(c % (uint32_t)dimx);
    const uint32_t t = c / (uint32_t)dimx;
    cy = (int)(t % (uint32_t)dimy);
    cz = (int)(t / (uint32_t)dimy);
}

// cell of x in the scene's grid, clamped into the grid (border cells absorb outliers)
template <class T> __device__ __forceinline__ void cell_of(const SceneDev<T> &S, const v4_t<T> &x, int &cx, int &cy, int &cz)
{
    cx = (int)floor(((T)x.x - S.ox) * S.inv_cell);
    cy = (int)floor(((T)x.y - S.oy) * S.inv_cell);
    cz = (int)floor(((T)x.z - S.oz) * S.inv_cell);
    cx = min(max(cx, 0), S.dimx - 1);
    cy = min(max(cy, 0), S.dimy - 1);
    cz = min(max(cz, 0), S.dimz - 1);
}

// the maps of scene s: first map and count in the scene-ordered map array
template <class T> __device__ __forceinline__ uint2 scene_maps(const DevParams<T> &P, uint32_t s)
{
    return P.vmap_range ? P.vmap_range[s] : make_uint2(0u, P.nvmaps);
}

template <class T> __device__ __forceinline__ uint32_t local_cell(const SceneDev<T> &S, int cx, int cy, int cz)
{
    return ((uint32_t)cz * (uint32_t)S.dimy + (uint32_t)cy) * (uint32_t)S.dimx + (uint32_t)cx;
}

// block-wide max of two counters, one atomic per block (all threads of the block call it)
__device__ __forceinline__ void block_max_atomic(uint32_t a, uint32_t b, unsigned *da, unsigned *db)
{
    // per warp, without a block barrier (the warps of the list build finish at very different
    // times); the atomic only where the warp's maximum exceeds the value already there
    a = __reduce_max_sync(0xffffffffu, a);
    b = __reduce_max_sync(0xffffffffu, b);
    if ((threadIdx.x & 31) == 0) {
        if (a > __ldcg(da)) atomicMax(da, a);
        if (b > __ldcg(db)) atomicMax(db, b);
    }
}

// ==========================================================================
// neighbour structure
// ==========================================================================
// Sort keys of the particles: (scene << Morton bits) | Morton code of the cell in
// the scene's grid, one entry per particle in upload order of the scenes
// (compact: idle slots have no entry).
template <class T>
__global__ void __launch_bounds__(kBlock) k_keys(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    const SceneDev<T> S = scene_get(P, q.s);
    int cx, cy, cz;
    cell_of(S, ldv(B.x, q.i), cx, cy, cz);
    const uint32_t u = S.ustart + (q.i - q.begin);
    B.key[u] = S.key_prefix | morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
    B.perm[u] = q.i;
    B.cellid[q.i] = S.cell_off + local_cell(S, cx, cy, cz);
}

// physical reorder: slot p of scene s receives the particle ranked (p - begin_s) in the scene's sorted keys
template <class T>
__global__ void __launch_bounds__(kBlock) k_gather(DevParams<T> P, DevBufs<T> B, const uint32_t *__restrict__ perm)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    const uint32_t ustart = P.nscenes > 1 ? P.scenes[q.s].ustart : 0u;
    const uint32_t k = q.i;
    const uint32_t s = perm[ustart + (k - q.begin)];
    stv(B.x2, k, ldv(B.x, s));
    stv(B.v2, k, ldv(B.v, s));
    stv(B.vdiff2, k, ldv(B.vdiff, s));
    if (B.xlo) B.xlo2[k] = B.xlo[s];
    B.kappa2[k] = B.kappa[s];
    B.kappa_v2[k] = B.kappa_v[s];
    B.id2[k] = B.id[s];
    B.cellid2[k] = B.cellid[s];
    if (P.nphase > 1) {   // the phase and rest density of the particle now in slot k
        stv(B.a, k, ldv(B.pa, s));   // its last pressure acceleration, put back by the list build
        const uint32_t id = B.id[s];
        uint32_t ph = 0;
        T r0 = P.phase_rho0[0];
#pragma unroll
        for (int q = 0; q < 7; q++)
            if (q + 1 < (int)P.nphase && id >= P.phase_end[q]) {
                ph = (uint32_t)(q + 1);
                r0 = P.phase_rho0[q + 1];
            }
        B.ph[k] = ph;
        B.r0[k] = r0;
    }
}

// first / one-past-last slot of every non-empty cell (cells of a scene are sorted within the scene's slots)
template <class T>
__global__ void __launch_bounds__(kBlock) k_cell_ranges(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    const uint32_t k = q.i;
    const uint32_t c = B.cellid[k];
    if (k == q.begin || B.cellid[k - 1] != c) B.cstart[c] = k;
    if (k + 1 == q.end || B.cellid[k + 1] != c) B.cend[c] = k + 1;
}

// the same for a flat sorted array without idle entries (boundary particles)
__global__ void __launch_bounds__(kBlock) k_cell_ranges_flat(const uint32_t *__restrict__ cellid, uint32_t *__restrict__ cstart,
                                                              uint32_t *__restrict__ cend, uint32_t n)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t c = cellid[k];
    if (k == 0 || cellid[k - 1] != c) cstart[c] = k;
    if (k == n - 1 || cellid[k + 1] != c) cend[c] = k + 1;
}

// ---- neighbourhood staging ----------------------------------------------------
// Exclusive block scan (kBlock threads) of two counters, with their block totals.
__device__ __forceinline__ void block_scan2(uint32_t a, uint32_t b, uint32_t &ea, uint32_t &eb, uint32_t &ta,
                                            uint32_t &tb)
{
    __shared__ uint32_t wa[kBlock / 32], wb[kBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t ia = a, ib = b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ya = __shfl_up_sync(0xffffffffu, ia, o), yb = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) { ia += ya; ib += yb; }
    }
    if (lane == 31) { wa[warp] = ia; wb[warp] = ib; }
    __syncthreads();
    uint32_t oa = 0, ob = 0;
    ta = tb = 0;
#pragma unroll
    for (int w = 0; w < kBlock / 32; w++) {
        if (w < warp) { oa += wa[w]; ob += wb[w]; }
        ta += wa[w];
        tb += wb[w];
    }
    ea = oa + ia - a;
    eb = ob + ib - b;
    __syncthreads();
}

// Stage table of a block of kBlock slots (one lane per particle): the cells of the union of its
// particles' 27-cell neighbourhoods that hold fluid, in ascending cell index, with the offset of
// each cell's first particle in the block's staged array.  The union is marked in a bitmap over
// the block's bounding box of cells dilated by one cell; a block over the limits of kStageCap,
// kStageCells or kStageBoxCells gets cells = 0 (not staged).
template <class T>
__global__ void __launch_bounds__(kBlock) k_stage_table(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    const SceneDev<T> S = scene_get(P, q.s);
    __shared__ int box[6];
    __shared__ uint32_t bits[kStageBoxCells / 32];
    if (threadIdx.x < 3) {
        box[threadIdx.x] = 0x7fffffff;
        box[3 + threadIdx.x] = -1;
    }
    __syncthreads();
    int cx = 0, cy = 0, cz = 0;
    if (q.act) {
        cell_coords(B.cellid[q.i] - S.cell_off, S.dimx, S.dimy, cx, cy, cz);
        atomicMin(&box[0], cx);
        atomicMin(&box[1], cy);
        atomicMin(&box[2], cz);
        atomicMax(&box[3], cx);
        atomicMax(&box[4], cy);
        atomicMax(&box[5], cz);
    }
    __syncthreads();
    uint32_t vol = 0;
    int lx = 0, ly = 0, lz = 0, ex = 0, ey = 0;
    if (box[3] >= 0) {
        lx = max(box[0] - 1, 0);
        ly = max(box[1] - 1, 0);
        lz = max(box[2] - 1, 0);
        ex = min(box[3] + 1, S.dimx - 1) - lx + 1;
        ey = min(box[4] + 1, S.dimy - 1) - ly + 1;
        const int ez = min(box[5] + 1, S.dimz - 1) - lz + 1;
        vol = (uint32_t)ex * (uint32_t)ey * (uint32_t)ez;
    }
    if (vol == 0 || vol > kStageBoxCells) {   // block uniform
        if (threadIdx.x == 0) B.stage_hdr[q.b] = make_uint2(0u, 0u);
        return;
    }
    for (uint32_t w = threadIdx.x; w < kStageBoxCells / 32; w += kBlock) bits[w] = 0u;
    __syncthreads();
    if (q.act) {
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int x = cx + dx - lx, y = cy + dy - ly, z = cz + dz - lz;
                    // outside the dilated box means outside the grid
                    if (x < 0 || y < 0 || z < 0 || x >= ex || y >= ey || (uint32_t)((z * ey + y) * ex + x) >= vol)
                        continue;
                    const uint32_t b = (uint32_t)((z * ey + y) * ex + x);
                    atomicOr(&bits[b >> 5], 1u << (b & 31u));
                }
    }
    __syncthreads();
    // each thread takes kStageBoxCells / kBlock consecutive box cells: count, scan, write
    constexpr uint32_t PER = kStageBoxCells / kBlock;
    const uint32_t b0 = threadIdx.x * PER;
    auto cell_at = [&](uint32_t b) {
        const uint32_t x = b % (uint32_t)ex, t = b / (uint32_t)ex;
        return S.cell_off + local_cell(S, lx + (int)x, ly + (int)(t % (uint32_t)ey), lz + (int)(t / (uint32_t)ey));
    };
    uint32_t nc = 0, nr = 0;
    for (uint32_t k = 0; k < PER; k++) {
        const uint32_t b = b0 + k;
        if (b >= vol) break;
        if (!((bits[b >> 5] >> (b & 31u)) & 1u)) continue;
        const uint32_t c = cell_at(b);
        const uint32_t st = B.cstart[c];
        if (st == kEmpty) continue;
        nc++;
        nr += B.cend[c] - st;
    }
    uint32_t pc, pr, tc, tr;
    block_scan2(nc, nr, pc, pr, tc, tr);
    if (tc == 0 || tc > kStageCells || tr > kStageCap) {   // block uniform
        if (threadIdx.x == 0) B.stage_hdr[q.b] = make_uint2(0u, 0u);
        return;
    }
    uint32_t *cells = B.stage_cell + (size_t)q.b * kStageCells;
    uint16_t *offs = B.stage_off + (size_t)q.b * kStageCells;
    uint32_t *src = B.stage_src + (size_t)q.b * kStageCap;
    for (uint32_t k = 0; k < PER; k++) {
        const uint32_t b = b0 + k;
        if (b >= vol) break;
        if (!((bits[b >> 5] >> (b & 31u)) & 1u)) continue;
        const uint32_t c = cell_at(b);
        const uint32_t st = B.cstart[c];
        if (st == kEmpty) continue;
        const uint32_t en = B.cend[c];
        cells[pc] = c;
        offs[pc] = (uint16_t)pr;
        for (uint32_t j = st; j < en; j++) src[pr + (j - st)] = j;
        pc++;
        pr += en - st;
    }
    if (threadIdx.x == 0) B.stage_hdr[q.b] = make_uint2(tc, tr);
}

// position of cell c in a block's stage table (ascending cell ids; c is present)
__device__ __forceinline__ uint32_t stage_find(const uint32_t *cells, uint32_t n, uint32_t c)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (cells[mid] <= c) lo = mid;
        else hi = mid;
    }
    return lo;
}

// TimeStep::computeVolumeAndBoundaryX (TimeStep.cpp:219-340), static bodies: for every body in
// turn, the volume-map sample at R^T (x_i - t) gives the distance phi, its gradient (the normal
// n = R grad phi / |.|) and the volume V.  For 0 < phi < h and V > 0 the particle gets the boundary
// point x_j = x_i - max(phi + r / 2, 2 r) n with volume V_j = V; a particle inside a body
// (phi <= 0) is moved by min(2 r - phi, r / 10) along n and stops (the reference's fallback for
// too large steps), and the next body sees it moved.  The boundary sums of the step then treat
// (x_j, V_j) like one boundary particle per body (forall_volume_maps, Simulation.h:79-89).
template <class T>
__global__ void __launch_bounds__(kBlock) k_vmap_boundary(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    const uint32_t i = q.i;
    const T r = (T)P.radius, hs = P.K.h;
    const uint2 mr = scene_maps(P, q.s);
    for (uint32_t b = 0; b < mr.y; b++) {   // b: the map's slot among the scene's maps
        const VMapDev<T> &m = P.vmaps[mr.x + b];
        v4_t<T> x = ldv(B.x, i);
        const T dx[3] = {(T)x.x - m.t[0], (T)x.y - m.t[1], (T)x.z - m.t[2]};
        T local[3];
#pragma unroll
        for (int k = 0; k < 3; k++) local[k] = m.R[k] * dx[0] + m.R[3 + k] * dx[1] + m.R[6 + k] * dx[2];
        T sdf = T(0), vol = T(0), g[3] = {T(0), T(0), T(0)};
        V3<T> xj = mk3<T>(0, 0, 0);
        T V = T(0);
        if (vmap_sample<T>(m, local, sdf, g, vol)) {
            const V3<T> nrm = mk3<T>(m.R[0] * g[0] + m.R[1] * g[1] + m.R[2] * g[2],
                                     m.R[3] * g[0] + m.R[4] * g[1] + m.R[5] * g[2],
                                     m.R[6] * g[0] + m.R[7] * g[1] + m.R[8] * g[2]);
            const T nl = dev_sqrt(dot(nrm, nrm));
            if (sdf > T(0) && sdf < hs) {
                if (vol > T(0) && nl > T(1.0e-9)) {
                    const T d = fmax(sdf + T(0.5) * r, T(2) * r);
                    xj = sub(xyz<T>(x), scl(nrm, d / nl));
                    V = vol;
                }
            } else if (sdf <= T(0) && nl > T(1.0e-5)) {
                const T delta = fmin(T(2) * r - sdf, T(0.1) * r);
                const V3<T> mv = scl(nrm, delta / nl);
                if (B.xlo) {   // double-float position
                    const float4 lo = B.xlo[i];
                    const double px = (double)x.x + (double)lo.x + (double)mv.x;
                    const double py = (double)x.y + (double)lo.y + (double)mv.y;
                    const double pz = (double)x.z + (double)lo.z + (double)mv.z;
                    x.x = (T)px; x.y = (T)py; x.z = (T)pz;
                    B.xlo[i] = make_float4((float)(px - (double)x.x), (float)(py - (double)x.y),
                                           (float)(pz - (double)x.z), 0.f);
                } else {
                    x.x += mv.x; x.y += mv.y; x.z += mv.z;
                }
                stv(B.x, i, x);
                v4_t<T> v = ldv(B.v, i);
                v.x = T(0); v.y = T(0); v.z = T(0);
                stv(B.v, i, v);
            }
        }
        stv(B.bx, b * P.np + i, pack(xj, V));
    }
}

// BoundaryModel::getPointVelocity (BoundaryModel.h:78-84): velocity w x (p - t) + v of point p of
// the body of volume map m
template <class T> __device__ __forceinline__ V3<T> vmap_point_velocity(const VMapDev<T> &m, const V3<T> &p)
{
    const T dx = p.x - m.t[0], dy = p.y - m.t[1], dz = p.z - m.t[2];
    return mk3<T>(m.w[1] * dz - m.w[2] * dy + m.v[0], m.w[2] * dx - m.w[0] * dz + m.v[1],
                  m.w[0] * dy - m.w[1] * dx + m.v[2]);
}

// Build the fluid and boundary neighbour lists of particle i and, in the same
// kernel, compute (TimeStep.cpp:116-169) the density, (TimeStepDFSPH.cpp:1106-1186)
// the DFSPH factor alpha, (TimeStepDFSPH.cpp:1247-1295) the divergence source and
// (TimeStepDFSPH.cpp:402-463) the warm-started kappa_v.
//
// Phase 1 scans the 27 surrounding cells with the exact predicate only and appends
// accepted indices to the lists (cells whose box is farther than h are skipped).
// Phase 2 walks the fresh lists densely for the kernel sums, so the kernel math
// does not run inside the divergent candidate loop.
// With the block's stage table (tn cells, in shared memory) phase 1 also writes the local
// list: the same entries as the fluid list, as indices into the block's staged array.
template <class T>
__device__ __forceinline__ void build_one(const DevParams<T> &P, const DevBufs<T> &B, const SceneDev<T> &S,
                                          uint32_t scene, StepScalars *sc, uint32_t i, uint32_t &nf_out, uint32_t &nb_out,
                                          const uint32_t *tcell, const uint16_t *toff, uint32_t tn)
{
    const v4_t<T> xi = ldv(B.x, i);
    int cx, cy, cz;
    cell_coords(B.cellid[i] - S.cell_off, S.dimx, S.dimy, cx, cy, cz);
    const T cs = T(1) / S.inv_cell;
    // squared distances from x_i to the lower / upper face of its cell, per axis
    T slo[3], shi[3];
    {
        const T px[3] = {(T)xi.x - S.ox, (T)xi.y - S.oy, (T)xi.z - S.oz};
        const int c3[3] = {cx, cy, cz};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const T lo = px[d] - (T)c3[d] * cs;
            const T hi = (T)(c3[d] + 1) * cs - px[d];
            slo[d] = lo > T(0) ? lo * lo : T(0);
            shi[d] = hi > T(0) ? hi * hi : T(0);
        }
    }
    const T cull = P.K.h2 * T(1.001);

    uint32_t *Lf = B.lf + fl_index(i, 0, P.capf, P.lpp_log2);   // entry k at fl_index(i, k, ...)
    uint32_t *Lb = list_ptr(B.lb, i, P.capb);
    uint16_t *Ll = tn ? B.ll + (size_t)(i >> 5) * P.capf * 32u + (i & 31u) : nullptr;   // one lane per particle
    const uint32_t lpp = 1u << P.lpp_log2;
    uint32_t nf = 0, nb = 0;
    for (int dz = -1; dz <= 1; dz++) {
        const int z = cz + dz;
        if (z < 0 || z >= S.dimz) continue;
        const T sz = dz < 0 ? slo[2] : (dz > 0 ? shi[2] : T(0));
        const bool inner_z = z > 0 && z < S.dimz - 1;
        for (int dy = -1; dy <= 1; dy++) {
            const int y = cy + dy;
            if (y < 0 || y >= S.dimy) continue;
            const T syz = sz + (dy < 0 ? slo[1] : (dy > 0 ? shi[1] : T(0)));
            const bool inner_yz = inner_z && y > 0 && y < S.dimy - 1;
            // the row's three cells (dx = -1, 0, 1): their fluid and boundary ranges are loaded
            // together, so their latencies overlap; a culled or outside cell gets an empty range
            uint32_t rc[3], rfs[3], rfe[3], rbs[3], rbe[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const int dx = k - 1, x = cx + dx;
                // border cells may hold clamped particles outside their box: never culled
                const bool inner = inner_yz && x > 0 && x < S.dimx - 1;
                const bool use = x >= 0 && x < S.dimx &&
                                 !(inner && syz + (dx < 0 ? slo[0] : (dx > 0 ? shi[0] : T(0))) > cull);
                rc[k] = use ? S.cell_off + local_cell(S, x, y, z) : 0u;
                rfs[k] = use ? B.cstart[rc[k]] : kEmpty;
                rfe[k] = use ? B.cend[rc[k]] : 0u;
                rbs[k] = use ? B.bcstart[rc[k]] : kEmpty;
                rbe[k] = use ? B.bcend[rc[k]] : 0u;
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const uint32_t c = rc[k];
                uint32_t s = rfs[k];
                if (s != kEmpty) {
                    const uint32_t e = rfe[k];
                    // staged index of slot j: lbase + j.  The stage table holds every fluid cell
                    // this loop visits; should a cell be missing, the block falls back to the
                    // unstaged passes (its stage header is cleared) and no local index is used.
                    uint32_t lbase = 0u;
                    if (Ll) {
                        const uint32_t pos = stage_find(tcell, tn, c);
                        if (tcell[pos] == c) {
                            lbase = (uint32_t)toff[pos] - s;
                        } else {
                            B.stage_hdr[i / kBlock] = make_uint2(0u, 0u);   // the block of slot i
                            Ll = nullptr;
                        }
                    }
                    auto accept = [&](uint32_t j) {
                        if (nf < P.capf) {
                            Lf[32u * (nf >> P.lpp_log2) + (nf & (lpp - 1u))] = j;
                            if (Ll) Ll[32u * nf] = (uint16_t)(lbase + j);
                        }
                        nf++;
                    };
                    // two candidates per iteration, both loads in flight before either test; the
                    // appends keep the order j, j + 1
                    uint32_t j = s;
                    for (; j + 1u < e; j += 2u) {
                        const v4_t<T> xa = ldv(B.x, j), xb = ldv(B.x, j + 1u);
                        T ddx, ddy, ddz;
                        const bool ia = pair_d2(xi, xa, ddx, ddy, ddz) < P.K.h2 && j != i;
                        const bool ib = pair_d2(xi, xb, ddx, ddy, ddz) < P.K.h2 && j + 1u != i;
                        if (ia) accept(j);
                        if (ib) accept(j + 1u);
                    }
                    if (j < e) {
                        T ddx, ddy, ddz;
                        if (j != i && pair_d2(xi, ldv(B.x, j), ddx, ddy, ddz) < P.K.h2) accept(j);
                    }
                }
                s = rbs[k];
                if (s != kEmpty) {
                    const uint32_t e = rbe[k];
                    auto accept = [&](uint32_t j) {
                        if (nb < P.capb) Lb[nb * 32u] = j;
                        nb++;
                    };
                    uint32_t j = s;
                    for (; j + 1u < e; j += 2u) {
                        const v4_t<T> xa = ldv(B.xb, j), xb = ldv(B.xb, j + 1u);
                        T ddx, ddy, ddz;
                        const bool ia = pair_d2(xi, xa, ddx, ddy, ddz) < P.K.h2;
                        const bool ib = pair_d2(xi, xb, ddx, ddy, ddz) < P.K.h2;
                        if (ia) accept(j);
                        if (ib) accept(j + 1u);
                    }
                    if (j < e) {
                        T ddx, ddy, ddz;
                        if (pair_d2(xi, ldv(B.xb, j), ddx, ddy, ddz) < P.K.h2) accept(j);
                    }
                }
            }
        }
    }

    // phase 2: kernel sums over the accepted neighbours
    const V3<T> vi = xyz<T>(ldv(B.v, i));
    T wf = T(0), wb = T(0), gsq = T(0), divf = T(0), divb = T(0);
    V3<T> gf = mk3<T>(0, 0, 0), gb = mk3<T>(0, 0, 0);
    struct XV {
        v4_t<T> x, v;
    };
    // the own list, sub-list by sub-list (entries l, l + lpp, ... are 32 words apart)
    const uint32_t nfc = min(nf, P.capf);
    for (uint32_t l = 0; l < lpp; l++)
        nbr_loop<kUnroll, 32u, true>(Lf + l, nfc > l ? (nfc - l + lpp - 1u) >> P.lpp_log2 : 0u,
                          [&](uint32_t j) { return XV{ldv(B.x, j), ldv(B.v, j)}; },
                          [&](uint32_t, const XV &d) {
                              const V3<T> r = diff3<T>(xi, d.x);
                              T W, c;
                              kernel_W_coef_d2(P.K, dot(r, r), W, c);
                              wf += W;
                              const V3<T> g = scl(r, c);
                              gsq += dot(g, g);
                              gf = add(gf, g);
                              divf += dot(sub(vi, xyz<T>(d.v)), g);
                          });
    // moving boundaries: sum V_j W v_j (XSPH) and sum V_j v_j . gradW (divergence source, density
    // advection), both fixed for the step
    V3<T> bvw = mk3<T>(0, 0, 0);
    T bvg = T(0);
    auto boundary_term = [&](uint32_t j, const v4_t<T> &xj) {
        const V3<T> r = diff3<T>(xi, xj);
        T W, c;
        kernel_W_coef_d2(P.K, dot(r, r), W, c);
        const T Vb = (T)xj.w;
        wb += Vb * W;
        const V3<T> g = scl(r, c * Vb);
        gb = add(gb, g);
        divb += dot(vi, g);
        if (P.bmove) {   // boundary particle j of a moving body
            const V3<T> vj = xyz<T>(ldv(B.vbs, j));
            bvw = add(bvw, scl(vj, Vb * W));
            bvg += dot(vj, g);
        }
    };
    nbr_loop<kUnroll, 32u, true>(Lb, min(nb, P.capb), [&](uint32_t j) { return ldv(B.xb, j); }, boundary_term);
    // Bender2019: the volume-map sample of each body, x_j with V_j in w, where V_j > 0; a moving
    // body's point velocity v_j enters the same sums
    const uint2 mr = scene_maps(P, scene);
    for (uint32_t b = 0; b < mr.y; b++) {
        const v4_t<T> xj = ldv(B.bx, b * P.np + i);
        if ((T)xj.w > T(0)) {
            boundary_term(b, xj);
            if (P.vmove) {
                const V3<T> vj = vmap_point_velocity<T>(P.vmaps[mr.x + b], xyz<T>(xj));
                const V3<T> r = diff3<T>(xi, xj);
                T W, c;
                kernel_W_coef_d2(P.K, dot(r, r), W, c);
                bvw = add(bvw, scl(vj, (T)xj.w * W));
                bvg += dot(vj, scl(r, c * (T)xj.w));
            }
        }
    }
    if (P.vmove || P.bmove) {
        divb -= bvg;
        stv(B.bv, i, pack(bvw, bvg));
    }
    B.nf[i] = nf;
    B.nbn[i] = nb;
    if (nf > P.capf || nb > P.capb) atomicOr(&sc->flags, kFlagOverflow);
    nf_out = nf;
    nb_out = nb;

    // density: rho0 * (V W0 + sum_f V W + sum_b Vb W)
    const T rho = rho0_at(P, B, i) * (P.V * P.K.w0 + P.V * wf + wb);
    B.density[i] = rho;
    // the fused XSPH and viscosity set-up pass gathers rho_j in the w lane of the
    // velocity-difference record (the kick overwrites it at the end of the step)
    if (P.visc_on) store_w(B.vdiff, i, rho);
    // factor: 1 / (sum_f |V gradW|^2 + |sum_f V gradW + sum_b Vb gradW|^2)
    const V3<T> gpi = add(scl(gf, P.V), gb);
    const T sum_grad = P.V * P.V * gsq + dot(gpi, gpi);
    const T alpha = sum_grad > P.eps ? T(1) / sum_grad : T(0);
    B.factor[i] = alpha;
    // divergence source (unclamped, as stored by computeDensityChange) and kappa_v warm start
    const T dsrc = divf * P.V + divb;
    B.dadv[i] = dsrc;
    T kv = B.kappa_v[i];
    if (P.div_on) {
        T densityAdv = dsrc > T(0) ? dsrc : T(0);
        if (nf + nb < 20u) densityAdv = T(0);
        const T invH = T(1) / (T)sc->dt;
        kv = densityAdv > T(0) ? T(0.5) * (kv < T(0.5) ? kv : T(0.5)) * invH : T(0);
        B.kappa_v[i] = kv;
    }
    // boundary sums are fixed for the step (static boundary, fixed positions): every
    // later pass uses them instead of re-walking the boundary list
    stv(B.bg, i, pack(gb, wb));
    if (P.feat_on) {
        // raw warm-start features, dimensionless and O(1): density deviation, velocity divergence
        // x dt, neighbour count, whether the particle carried pressure in the last step (the
        // previous kappa itself enters relative to its neighbourhood, in k_features),
        // displacement per step in diameters
        const float h = (float)sc->dt;
        float *f = B.feat + (size_t)i * 8;
        f[0] = 100.0f * ((float)rho / (float)P.rho0 - 1.0f);
        f[1] = 100.0f * (float)dsrc * h;
        f[2] = (float)(nf + nb) * (1.0f / 40.0f) - 1.0f;
        f[3] = B.kappa[i] > T(0) ? 1.0f : 0.0f;
        f[4] = 10.0f * sqrtf((float)dot(vi, vi)) * h / (float)(2.0 * P.radius);
    }
    v4_t<T> xk = xi;
    xk.w = kv;
    stv(B.xk, i, xk);
    // FP32: the position half of the Jacobi pass's (x, a) record, fixed for the step; the
    // pressure-acceleration passes write only the acceleration half
    if constexpr (sizeof(T) == 4) B.xa[2 * (size_t)i] = xi;
    if (P.nphase > 1) {   // fluid phases: each particle's last pressure acceleration, in its new slot
        const v4_t<T> a = ldv(B.a, i);
        stv(B.pa, i, a);
        if constexpr (sizeof(T) == 4)   // a pass writes only its own phase's accelerations
            B.xa[2 * (size_t)i + 1] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.0f);
    }
}

// ST: the instance that may write the staged passes' local lists.  Without staging the instance
// compiled without that code is used (0.49 against 0.53 ms at 1M particles).
template <class T, bool ST>
__global__ void __launch_bounds__(kBlock) k_build(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    StepScalars *const sc = B.sc + q.s;
    if constexpr (!ST) {
        uint32_t nf = 0, nb = 0;
        if (q.act) build_one(P, B, scene_get(P, q.s), q.s, sc, q.i, nf, nb, nullptr, nullptr, 0u);
        block_max_atomic(nf, nb, &sc->max_nf, &sc->max_nb);
        return;
    }
    __shared__ uint32_t tcell[kStageCells];
    __shared__ uint16_t toff[kStageCells];
    uint32_t tn = 0;
    if (P.staged) {   // block uniform
        tn = B.stage_hdr[q.b].x;
        for (uint32_t k = threadIdx.x; k < tn; k += kBlock) {
            tcell[k] = B.stage_cell[(size_t)q.b * kStageCells + k];
            toff[k] = B.stage_off[(size_t)q.b * kStageCells + k];
        }
        __syncthreads();
    }
    uint32_t nf = 0, nb = 0;
    if (q.act) build_one(P, B, scene_get(P, q.s), q.s, sc, q.i, nf, nb, tcell, toff, tn);
    block_max_atomic(nf, nb, &sc->max_nf, &sc->max_nb);
}

// ==========================================================================
// DFSPH solver passes
// ==========================================================================
// The neighbour passes run LPP lanes per particle.  All 32 lanes of a warp reach the
// lane sums (gsum): inactive slots contribute zeros, and only whole blocks return early.

// computePressureAccel, scalar path (TimeStepDFSPH.cpp:1299-1367):
// a_i = -V sum_j [|k_i + k_j| > eps] (k_i + k_j) gradW_ij - [|k_i| > eps] k_i sum_b V_b gradW_ib
// with kappa of the running solver read from xk.w and the boundary sum from bg.
// Every lane of the particle returns the full acceleration.
// Staged (sx != null, one lane per particle): the neighbours' xk records come from the block's
// shared copy through the local list, in the order of the fluid list, so the sums are the same.
template <int LPP, bool MP = false, class T>
__device__ __forceinline__ V3<T> pressure_accel_g(const DevParams<T> &P, const DevBufs<T> &B, const SlotInfo &q,
                                                  const v4_t<T> *sx = nullptr)
{
    V3<T> acc = mk3<T>(0, 0, 0);
    T pi = T(0);
    v4_t<T> xi{};
    if (q.act) {
        xi = ldv(B.xk, q.i);
        pi = (T)xi.w;
        const T r0i = MP ? B.r0[q.i] : T(1);
        auto cp = [&](uint32_t j, const v4_t<T> &xj) {
            // kappa_i + density0_j / density0_i kappa_j (TimeStepDFSPH.cpp:1312); one phase: ratio 1
            const T psum = MP ? pi + (B.r0[j] / r0i) * (T)xj.w : pi + (T)xj.w;
            if (fabs(psum) > P.eps) {
                const V3<T> r = diff3<T>(xi, xj);
                const T c = grad_coef_d2(P.K, dot(r, r)) * psum;
                acc = add(acc, scl(r, c));
            }
        };
        if (LPP == 1 && sx)
            nbr_loop<kUnroll>(ll_ptr(B.ll, q.i, P.capf), min(B.nf[q.i], P.capf), [&](uint32_t m) { return sx[m]; }, cp);
        else
            fluid_loop<LPP, kUnroll>(P, B, q.i, q.l, [&](uint32_t j) { return ldv(B.xk, j); }, cp);
    }
    acc = gsum3<LPP>(acc);
    V3<T> ai = scl(acc, -P.V);
    if (q.act && fabs(pi) > P.eps) ai = sub(ai, scl(xyz<T>(ldv(B.bg, q.i)), pi));
    return ai;
}

// resident blocks per SM the FP32 one-lane pressure-acceleration pass is compiled for (a register
// cap of 42): measured 11 % faster at 1M particles than the unconstrained 43-44 registers (5
// blocks); tighter caps spill
template <class T, int LPP> constexpr int kPressureMinBlocks = (sizeof(T) == 4 && LPP == 1) ? 6 : 1;

// Copy the block's staged records to shared memory: rec = load(slot) for every slot of the
// block's staged list, then store(local index, rec); CH loads in flight per thread.  Returns
// false, without copying, for a block that is not staged or has more than cap records.  Every
// thread of the block calls it (it synchronises the block).
template <class Ld, class St>
__device__ __forceinline__ bool stage_in(const DevBufs<float> &B, uint32_t blk, uint32_t cap, Ld load, St store)
{
    const uint2 hdr = B.stage_hdr[blk];
    if (hdr.x == 0 || hdr.y > cap) return false;   // block uniform
    const uint32_t *src = B.stage_src + (size_t)blk * kStageCap;
    constexpr uint32_t CH = 4;
#pragma unroll 1
    for (uint32_t base = threadIdx.x; base < hdr.y; base += CH * kBlock) {
        uint32_t slot[CH];
#pragma unroll
        for (uint32_t r = 0; r < CH; r++) slot[r] = base + r * kBlock < hdr.y ? src[base + r * kBlock] : 0u;
        decltype(load(0u)) rec[CH];
#pragma unroll
        for (uint32_t r = 0; r < CH; r++)
            if (base + r * kBlock < hdr.y) rec[r] = load(slot[r]);
#pragma unroll
        for (uint32_t r = 0; r < CH; r++)
            if (base + r * kBlock < hdr.y) store(base + r * kBlock, rec[r]);
    }
    __syncthreads();
    return true;
}

// Termination guard of a device-side loop: the first kernel of every loop body
// counts body executions; past the bound (which the solvers' own decisions never
// reach) it clears the loop condition and raises a flag that also overrides the
// decision of the same body, so a loop can never run on if its convergence
// decision was lost.
__device__ __forceinline__ void loop_guard(StepScalars *gsc, unsigned limit, cudaGraphConditionalHandle h, int use_handle)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned g = ++gsc->loop_guard;
        if (g > limit) {
            gsc->flags |= kFlagLoopGuard;
            gsc->cont = 0;
            if (use_handle) cudaGraphSetConditional(h, 0u);
        }
    }
}

// a scene whose solver loop already stopped skips the remaining bodies of the batch's loop
// (uniform over a block: a block belongs to one scene)
template <class T> __device__ __forceinline__ bool scene_live(const DevParams<T> &P, const StepScalars *sc)
{
    return P.nscenes == 1 || sc->cont != 0u;
}

// One 32-byte record (two float4) with a single 256-bit load; p must be 32-byte aligned and
// not written during the kernel.
struct F8 {
    float4 a, b;
};
__device__ __forceinline__ F8 ld_f8(const float4 *p)
{
    F8 r;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y), "=f"(r.b.z), "=f"(r.b.w)
        : "l"(p));
    return r;
}

// Pressure accelerations of the running solver.  FP32: the acceleration half of the (x_i, a_i)
// record that the Jacobi pass gathers with one 256-bit load per neighbour.
// NT: threads per block (the same resident threads per SM at every size); the staged variant runs
// with kBlock only
template <class T, int LPP, bool MP = false, int NT = kBlock>
__global__ void __launch_bounds__(NT, kPressureMinBlocks<T, LPP> * kBlock / NT)
    k_pressure_accel(DevParams<T> P, DevBufs<T> B, unsigned limit, cudaGraphConditionalHandle h, int use_handle,
                     int phase)
{
    count_launch(&B.gsc->launches);
    if (phase <= 0) loop_guard(B.gsc, limit, h, use_handle);   // once per loop body
    SlotInfo q = slot_info<LPP, NT>(P);
    if (!scene_live(P, B.sc + q.s)) return;   // block uniform
    // fluid phases: this launch updates the particles of one phase; the others keep their last a
    if (phase >= 0 && q.act && B.ph[q.i] != (uint32_t)phase) q.act = false;
    V3<T> a;
    if constexpr (LPP == 1 && sizeof(T) == 4 && NT == kBlock) {
        extern __shared__ float4 stage_f4[];   // kStageCap records when staged
        if (P.staged && stage_in(B, q.b, kStageCap, [&](uint32_t j) { return ldv(B.xk, j); },
                                 [&](uint32_t m, const float4 &r) { stage_f4[m] = r; }))
            a = pressure_accel_g<LPP, MP>(P, B, q, stage_f4);
        else
            a = pressure_accel_g<LPP, MP>(P, B, q);
    } else {
        a = pressure_accel_g<LPP, MP>(P, B, q);
    }
    if (!q.act || q.l != 0) return;
    if constexpr (sizeof(T) == 4) {
        B.xa[2 * (size_t)q.i + 1] = make_float4(a.x, a.y, a.z, 0.0f);   // x half: written by the list build
    } else {
        stv(B.pa, q.i, pack(a, T(0)));
    }
}

// compute_aij_pj, scalar path (TimeStepDFSPH.cpp:1370-1420):
// V sum_j (a_i - a_j).gradW_ij + a_i . sum_b V_b gradW_ib, on every lane of the particle.
// FP32: x_j and a_j from the packed record, one 256-bit load per neighbour; staged (s0 != null,
// one lane per particle): from the block's shared copy, three float2 arrays (x, y), (z, a_x),
// (a_y, a_z), through the local list.
template <int LPP>
__device__ __forceinline__ float aij_pj_g(const DevParams<float> &P, const DevBufs<float> &B, const SlotInfo &q,
                                          const float2 *s0 = nullptr, const float2 *s1 = nullptr,
                                          const float2 *s2 = nullptr)
{
    float accf = 0.0f;
    V3<float> ai = mk3<float>(0, 0, 0);
    if (q.act) {
        const F8 me = ld_f8(B.xa + 2 * (size_t)q.i);
        const float4 xi = me.a;
        ai = xyz<float>(me.b);
        auto cp = [&](uint32_t, const F8 &d) {
            const V3<float> r = diff3<float>(xi, d.a);
            const float c = grad_coef_d2(P.K, dot(r, r));
            accf += c * dot(sub(ai, xyz<float>(d.b)), r);
        };
        if (LPP == 1 && s0)
            nbr_loop<kUnroll>(ll_ptr(B.ll, q.i, P.capf), min(B.nf[q.i], P.capf),
                              [&](uint32_t m) {
                                  const float2 u = s0[m], v = s1[m], w = s2[m];
                                  F8 r;
                                  r.a = make_float4(u.x, u.y, v.x, 0.0f);
                                  r.b = make_float4(v.y, w.x, w.y, 0.0f);
                                  return r;
                              },
                              cp);
        else
            fluid_loop<LPP, kUnroll>(P, B, q.i, q.l, [&](uint32_t j) { return ld_f8(B.xa + 2 * (size_t)j); }, cp);
    }
    accf = gsum<LPP>(accf);
    return q.act ? accf * P.V + dot(ai, xyz<float>(ldv(B.bg, q.i))) : 0.0f;
}
template <int LPP>
__device__ __forceinline__ double aij_pj_g(const DevParams<double> &P, const DevBufs<double> &B, const SlotInfo &q)
{
    double accf = 0.0;
    V3<double> ai = mk3<double>(0, 0, 0);
    if (q.act) {
        const dquad xi = ldv(B.x, q.i);
        ai = xyz<double>(ldv(B.pa, q.i));
        struct XA {
            dquad x, a;
        };
        fluid_loop<LPP, kUnroll>(P, B, q.i, q.l, [&](uint32_t j) { return XA{ldv(B.x, j), ldv(B.pa, j)}; },
                                 [&](uint32_t, const XA &d) {
                                     const V3<double> r = diff3<double>(xi, d.x);
                                     const double c = grad_coef_d2(P.K, dot(r, r));
                                     accf += c * dot(sub(ai, xyz<double>(d.a)), r);
                                 });
    }
    accf = gsum<LPP>(accf);
    return q.act ? accf * P.V + dot(ai, xyz<double>(ldv(B.bg, q.i))) : 0.0;
}

// Book one iteration of a scene's solver with average error avg and take its loop decision:
// the while conditions of TimeStepDFSPH.cpp:477 (divergence: at least one iteration, error
// below maxErrorV percent of rho0 per second) and :324 (pressure: at least minIterations,
// error below maxError percent of rho0), both capped by the maximum iteration count.
// With fluid phases the caller passes chk = every phase met its tolerance (phase_chk = 0 or 1).
template <class T, bool DIV>
__device__ __forceinline__ void solver_decide(const DevParams<T> &P, StepScalars *sc, double avg, unsigned inc = 1,
                                              int phase_chk = -1)
{
    unsigned it;
    bool cont;
    if (DIV) {
        it = (sc->iters_v += inc);
        sc->avg_err_v = avg;
        const double eta = (1.0 / sc->dt) * P.max_error_v * 0.01 * (double)P.rho0;
        const bool chk = phase_chk >= 0 ? phase_chk != 0 : avg <= eta;
        cont = (!chk || it < 1u) && it < P.max_iter_v;
    } else {
        it = (sc->iters += inc);
        sc->avg_err = avg;
        const double eta = P.max_error * 0.01 * (double)P.rho0;
        const bool chk = phase_chk >= 0 ? phase_chk != 0 : avg <= eta;
        cont = (!chk || it < P.min_iter) && it < P.max_iter;
    }
    sc->cont = cont ? 1u : 0u;
}

// divergenceSolveIteration (TimeStepDFSPH.cpp:621-706) / pressureSolveIteration (:544-619):
// Jacobi update of kappa_v / kappa plus the FP64 average-error reduction and the
// loop decision (the while conditions of :477 and :324), per scene.
// resident blocks per SM the FP32 one-lane Jacobi pass is compiled for (a register cap of 40):
// measured 0.6 % faster per step on the 1M dam break than the unconstrained 44 registers (5 blocks)
template <class T, int LPP> constexpr int kJacobiMinBlocks = (sizeof(T) == 4 && LPP == 1) ? 6 : 1;

template <class T, bool DIV, int LPP, int NT = kBlock>
__global__ void __launch_bounds__(NT, kJacobiMinBlocks<T, LPP> * kBlock / NT)
    k_jacobi(DevParams<T> P, DevBufs<T> B, cudaGraphConditionalHandle handle, int use_handle, int phase)
{
    count_launch(&B.gsc->launches);
    SlotInfo q = slot_info<LPP, NT>(P);
    // fluid phases: this launch updates the particles of one phase (TimeStepDFSPH.cpp:322-339)
    if (phase >= 0 && q.act && B.ph[q.i] != (uint32_t)phase) q.act = false;
    StepScalars *const sc = B.sc + q.s;
    // a scene whose loop has stopped: its blocks return at once (block uniform; batch_decide
    // expects only the live scenes)
    if (!scene_live(P, sc)) return;
    double err = 0.0;
    {
        T apj;
        if constexpr (LPP == 1 && sizeof(T) == 4 && NT == kBlock) {
            extern __shared__ float2 stage_f2[];   // 3 x kStageCapJacobi when staged
            float2 *s0 = stage_f2, *s1 = stage_f2 + kStageCapJacobi, *s2 = stage_f2 + 2 * kStageCapJacobi;
            if (P.staged && stage_in(B, q.b, kStageCapJacobi, [&](uint32_t j) { return ld_f8(B.xa + 2 * (size_t)j); },
                                     [&](uint32_t m, const F8 &r) {
                                         s0[m] = make_float2(r.a.x, r.a.y);
                                         s1[m] = make_float2(r.a.z, r.b.x);
                                         s2[m] = make_float2(r.b.y, r.b.z);
                                     }))
                apj = aij_pj_g<LPP>(P, B, q, s0, s1, s2);
            else
                apj = aij_pj_g<LPP>(P, B, q);
        } else {
            apj = aij_pj_g<LPP>(P, B, q);
        }
        if (q.act && q.l == 0) {
            const uint32_t i = q.i;
            const double hd = DIV ? sc->dt : sc->dt_next;
            const T h = (T)hd;
            T *kap = DIV ? B.kappa_v : B.kappa;
            if (DIV) {
                apj *= h;
                const T si = -B.dadv[i];
                T residuum = (si - apj) < T(0) ? (si - apj) : T(0);
                if (B.nf[i] + B.nbn[i] < 20u) residuum = T(0);
                const T fac = B.factor[i] * (T(1) / h);
                const T kv = kap[i] - T(0.5) * (si - apj) * fac;
                kap[i] = kv > T(0) ? kv : T(0);
                store_w(B.xk, i, kap[i]);
                err = -(double)rho0_at(P, B, i) * (double)residuum;
            } else {
                apj *= h * h;
                const T si = T(1) - B.dadv[i];
                const T residuum = (si - apj) < T(0) ? (si - apj) : T(0);
                const T fac = B.factor[i] * (T(1) / (h * h));
                const T kv = kap[i] - T(0.5) * (si - apj) * fac;
                kap[i] = kv > T(0) ? kv : T(0);
                store_w(B.xk, i, kap[i]);
                err = -(double)rho0_at(P, B, i) * (double)residuum;
            }
        }
    }
    DSum<1> mine;
    mine.v[0] = err;
    const DevParams<T> &PP = P;
    const DevBufs<T> &BB = B;
    const uint32_t n_s = q.end - q.begin;
    const int ph = phase;
    grid_sum_finalize<1>(mine, scene_reduce<LPP, NT>(P, B, q), [&](const DSum<1> &tot) {
        if (ph < 0) {
            solver_decide<T, DIV>(PP, sc, n_s ? tot.v[0] / (double)n_s : 0.0);
            batch_decide(PP, BB, handle, use_handle, false);
        } else {   // one phase's average error against its own tolerance; the last phase decides
            uint32_t cnt;
            T r0;
            phase_info(PP, ph, cnt, r0);
            const double avg = cnt ? tot.v[0] / (double)cnt : 0.0;
            const double eta = DIV ? (1.0 / sc->dt) * PP.max_error_v * 0.01 * (double)r0 : PP.max_error * 0.01 * (double)r0;
            const unsigned ok = avg <= eta ? (1u << ph) : 0u;
            sc->phase_ok = ph == 0 ? ok : (sc->phase_ok | ok);
            if (ph + 1 == (int)PP.nphase) {
                solver_decide<T, DIV>(PP, sc, avg, 1u, sc->phase_ok == (1u << PP.nphase) - 1u);
                batch_decide(PP, BB, handle, use_handle, false);
            }
        }
    });
}

// final pressure acceleration and velocity update of both solvers
// (TimeStepDFSPH.cpp:500-520 and :345-363)
template <class T, bool DIV, int LPP, bool MP = false>
__global__ void __launch_bounds__(kBlock) k_solver_finalize(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info<LPP>(P);
    const V3<T> a = pressure_accel_g<LPP, MP>(P, B, q);
    // fluid phases: the next solver's first iteration reads the other phases' last a in the record
    if constexpr (sizeof(T) == 4 && MP)
        if (q.act && q.l == 0) B.xa[2 * (size_t)q.i + 1] = make_float4(a.x, a.y, a.z, 0.0f);
    if (!q.act || q.l != 0) return;
    const StepScalars *sc = B.sc + q.s;
    const T h = (T)(DIV ? sc->dt : sc->dt_next);
    stv(B.pa, q.i, pack(a, T(0)));
    v4_t<T> v = ldv(B.v, q.i);
    v.x += h * a.x;
    v.y += h * a.y;
    v.z += h * a.z;
    stv(B.v, q.i, v);
}

__global__ void k_step_begin(StepScalars *sc, StepScalars *gsc, uint32_t nscenes)
{
    for (uint32_t s = threadIdx.x; s < nscenes; s += blockDim.x) {
        StepScalars &r = sc[s];
        r.flags = 0;
        r.max_nf = 0;
        r.max_nb = 0;
        r.maxvel_bits = 0;
        r.maxvel_bits64 = 0ull;
        r.iters_cg = 0;
        r.cg_err = 0.0;
        r.cg_state = 1;
    }
    if (threadIdx.x == 0) {
        gsc->launches = 1;
        gsc->flags = 0;
        gsc->loop_guard = 0;
    }
}

__global__ void k_loop_begin(StepScalars *sc, StepScalars *gsc, uint32_t nscenes, int div, unsigned max_iter)
{
    count_launch(&gsc->launches);
    const unsigned cont = max_iter > 0 ? 1u : 0u;
    for (uint32_t s = threadIdx.x; s < nscenes; s += blockDim.x) {
        StepScalars &r = sc[s];
        if (div) { r.iters_v = 0; r.avg_err_v = 0.0; }
        else { r.iters = 0; r.avg_err = 0.0; }
        r.cont = cont;
    }
    if (threadIdx.x == 0) {
        gsc->cont = cont;
        gsc->live = cont ? nscenes : 0u;
        gsc->loop_guard = 0;
    }
}

// ==========================================================================
// non-pressure forces
// ==========================================================================
// clearAccelerations (TimeStep.cpp:35-50) + XSPH::step scalar path (XSPH.cpp:138-211).
// Also finishes the divergence solve's kappa_v *= h (TimeStepDFSPH.cpp:522-540),
// which must wait until no thread reads kappa_v of its neighbours any more.
// Gravity plus the XSPH acceleration of particle i from its fluid sum acc (XSPH.cpp:138-216),
// kappa_v h (divergence solve on) and, with viscosity, the Weiler2018 warm start in cg_x.
template <class T>
__device__ __forceinline__ void xsph_finish(const DevParams<T> &P, const DevBufs<T> &B, uint32_t s, uint32_t i,
                                            V3<T> acc, T xs, T xsb, int div_on)
{
    const T h = (T)B.sc[s].dt;
    const T invH = T(1) / h;
    const V3<T> vi = xyz<T>(ldv(B.v, i));
    V3<T> ai = mk3<T>(P.gx, P.gy, P.gz);
    if (xs != T(0)) ai = sub(ai, scl(acc, invH * xs));
    if (xsb != T(0)) {
        // sum_b (rho0 V_b / rho_i) W_ib from the per-step boundary sum
        const T r0i = rho0_at(P, B, i);
        const T wsum = r0i * (T)ldv(B.bg, i).w / B.density[i];
        if (P.vmove || P.bmove) {   // moving boundaries: (v_i - v_b) W
            const V3<T> dv = sub(scl(vi, (T)ldv(B.bg, i).w), xyz<T>(ldv(B.bv, i)));
            ai = sub(ai, scl(dv, invH * xsb * r0i / B.density[i]));
        } else {
            ai = sub(ai, scl(vi, invH * xsb * wsum));
        }
    }
    stv(B.a, i, pack(ai, T(0)));
    if (div_on) B.kappa_v[i] *= h;
    if (P.visc_on) {
        // Weiler2018 warm start g = v + vDiff (Viscosity_Weiler2018.cpp:1247-1250) with the
        // operator weight d mu m_i / rho_i in w
        // (fluid phases: mu = nu rho0 and m_i = V rho0 of the particle's phase)
        T wi;
        if (P.nphase > 1) {
            const T r0 = B.r0[i];
            T nu, nub;
            phase_visc(P, B.ph[i], nu, nub);
            wi = P.vd * (nu * r0) * (P.V * r0) / B.density[i];
        } else {
            wi = P.vd * P.mu * P.mass / B.density[i];
        }
        stv(B.cg_x, i, pack(add(vi, xyz<T>(ldv(B.vdiff, i))), wi));
    }
}

template <class T, int LPP>
__global__ void __launch_bounds__(kBlock) k_xsph(DevParams<T> P, DevBufs<T> B, int div_on)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info<LPP>(P);
    V3<T> acc = mk3<T>(0, 0, 0);
    T xs = P.xsph, xsb = P.xsph_b;   // fluid phases: the particle's model's coefficients
    if (P.nphase > 1 && q.act) phase_xsph(P, B.ph[q.i], xs, xsb);
    if (q.act && xs != T(0)) {
        const v4_t<T> xi = ldv(B.x, q.i);
        const V3<T> vi = xyz<T>(ldv(B.v, q.i));
        struct XVR {
            v4_t<T> x, v;
            T rho;
        };
        fluid_loop<LPP, kUnroll>(P, B, q.i, q.l, [&](uint32_t j) { return XVR{ldv(B.x, j), ldv(B.v, j), B.density[j]}; },
                                 [&](uint32_t j, const XVR &d) {
                                     const V3<T> r = diff3<T>(xi, d.x);
                                     const T mj = P.nphase > 1 ? P.V * B.r0[j] : P.mass;
                                     const T w = (mj / d.rho) * kernel_W(P.K, dev_sqrt(dot(r, r)));
                                     acc = add(acc, scl(sub(vi, xyz<T>(d.v)), w));
                                 });
    }
    acc = gsum3<LPP>(acc);
    if (!q.act || q.l != 0) return;
    xsph_finish(P, B, q.s, q.i, acc, xs, xsb, div_on);
}

// ---- Weiler et al. 2018 ---------------------------------------------------
// Operator (Viscosity_Weiler2018.cpp:271-443):
//   (A v)_i = v_i - dt/rho_i * sum_j w_j ((v_i - v_j).x_ij) / (|x_ij|^2 + 0.01 h^2) gradW_ij
// with w_j = d mu m_j / rho_j, constant during the solve.  Since gradW_ij = c_ij x_ij the
// diagonal block (diagonalMatrixElement :605-742) I - dt/rho_i sum_j w_j c_ij x_ij x_ij^T /
// (|x_ij|^2 + 0.01 h^2) is symmetric: 6 entries, and its inverse is symmetric too.
// w_j travels in the w lane of the CG direction p (and of the warm start in cg_x), so one
// 16-byte gather per neighbour gives both the vector and the weight.

// The four samples that stand for a volume-map boundary point x_j in the Weiler2018 boundary term
// (Viscosity_Weiler2018.cpp:205-255, 383-430, 697-740, 1031-1080): x_j -+ t1 h/2 and x_j -+ t2 h/2
// with t1 = n x v / |.|, t2 = n x t1 / |.|, n = (x_j - x_i) / |.| and v = e_x, or e_y when
// |n . e_x| > 0.999 (MathFunctions::getOrthogonalVectors, MathFunctions.cpp:234-247); each stands
// for a quarter of V_j.  visit(x_k) for each; none when |x_i - x_j| <= 1e-4.
template <class T, class Vis>
__device__ __forceinline__ void vmap_samples(const v4_t<T> &xi, const v4_t<T> &xj, T h, Vis visit)
{
    V3<T> n = sub(xyz<T>(xj), xyz<T>(xi));
    const T nl = dev_sqrt(dot(n, n));
    if (!(nl > T(1.0e-4))) return;
    n = scl(n, T(1) / nl);
    const V3<T> v = fabs(n.x) > T(0.999) ? mk3<T>(0, 1, 0) : mk3<T>(1, 0, 0);
    V3<T> t1 = mk3<T>(n.y * v.z - n.z * v.y, n.z * v.x - n.x * v.z, n.x * v.y - n.y * v.x);
    V3<T> t2 = mk3<T>(n.y * t1.z - n.z * t1.y, n.z * t1.x - n.x * t1.z, n.x * t1.y - n.y * t1.x);
    t1 = scl(t1, T(1) / dev_sqrt(dot(t1, t1)));
    t2 = scl(t2, T(1) / dev_sqrt(dot(t2, t2)));
    const T d = T(0.5) * h;
    const V3<T> c = xyz<T>(xj);
    visit(sub(c, scl(t1, d)));
    visit(add(c, scl(t1, d)));
    visit(sub(c, scl(t2, d)));
    visit(add(c, scl(t2, d)));
}

// Boundary term of the operator (mub != 0), this lane's share:
// sum_b d mub (rho0 V_b / rho_i) (v_i.x_ib) / (...) gradW_ib.
template <int LPP, class T>
__device__ __forceinline__ V3<T> weiler_boundary(const DevParams<T> &P, const DevBufs<T> &B, const SlotInfo &q,
                                                 const v4_t<T> &xi, T rhoi, V3<T> vi)
{
    V3<T> acc = mk3<T>(0, 0, 0);
    const T eps2 = T(0.01) * P.h2;
    boundary_loop<LPP>(P, B, q.i, q.l, [&](uint32_t, const v4_t<T> &xj) {
        const V3<T> r = diff3<T>(xi, xj);
        const T r2 = dot(r, r);
        const T f = P.vd * P.mub * (P.rho0 * (T)xj.w / rhoi) * dot(vi, r) / (r2 + eps2);
        acc = add(acc, scl(r, grad_coef_d2(P.K, r2) * f));
    });
    // volume maps: four samples per body, a quarter of V_j each and no rho0 / rho_i factor (as in
    // the reference's Bender2019 branches); lane 0 only, the lanes' shares are summed
    const uint2 mr = scene_maps(P, q.s);
    if (q.l == 0)
        for (uint32_t b = 0; b < mr.y; b++) {
            const v4_t<T> xj = ldv(B.bx, b * P.np + q.i);
            if (!((T)xj.w > T(0))) continue;
            const T vol = T(0.25) * (T)xj.w;
            vmap_samples<T>(xi, xj, P.K.h, [&](const V3<T> &xk) {
                const V3<T> r = sub(xyz<T>(xi), xk);
                const T r2 = dot(r, r);
                const T f = P.vd * P.mub * vol * dot(vi, r) / (r2 + eps2);
                acc = add(acc, scl(r, grad_coef_d2(P.K, r2) * f));
            });
        }
    return acc;
}

// Symmetric 3x3 stored as (m00, m01, m02, m11) and (m12, m22, -, -).
template <class T> __device__ __forceinline__ V3<T> sym_mul(const v4_t<T> &a, const v4_t<T> &b, V3<T> v)
{
    return V3<T>{(T)a.x * v.x + (T)a.y * v.y + (T)a.z * v.z, (T)a.y * v.x + (T)a.w * v.y + (T)b.x * v.z,
                 (T)a.z * v.x + (T)b.x * v.y + (T)b.y * v.z};
}

// Set-up of the CG solve (Viscosity_Weiler2018.cpp:891-926): block-Jacobi inverse of the
// diagonal blocks (inverse taken in MatrixFreeSolver.h:231-244), b = v (computeRHS :1091-1254,
// static boundary), warm start g = v + vDiff (already in cg_x), r = b - A g, p = M^-1 r, and
// the first reductions of Eigen's conjugate_gradient (ConjugateGradient.h:29-70), one pass.
// MP (fluid phases): the system of phase `phase` alone (Viscosity_Weiler2018 is per fluid model and
// sums over forall_fluid_neighbors_in_same_phase); the other phases' particles get p = 0 with
// weight 0, so the matrix-vector passes of this phase need no neighbour test.
// XS (one fluid phase): the XSPH pass fused in.  The neighbours' warm start g_j = v_j + vDiff_j and
// weight w_j = d mu m / rho_j are formed here, with the same operations as k_xsph stores them in
// cg_x, from one walk of the list that gathers (x_j, v_j, vDiff_j | rho_j); the XSPH sum takes v_j
// and rho_j from the same records, and the particle's own XSPH results are written as k_xsph does.
template <class T, int LPP, bool MP = false, bool XS = false>
__global__ void __launch_bounds__(kBlock) k_visc_setup(DevParams<T> P, DevBufs<T> B, cudaGraphConditionalHandle handle,
                                                        int use_handle, int phase)
{
    static_assert(!(MP && XS), "the fused XSPH pass serves a single fluid phase");
    count_launch(&B.gsc->launches);
    SlotInfo q = slot_info<LPP>(P);
    bool other = false;   // a slot of another phase
    if (MP && q.act && B.ph[q.i] != (uint32_t)phase) {
        other = true;
        q.act = false;
    }
    StepScalars *const sc = B.sc + q.s;
    DSum<3> mine;
    mine.v[0] = mine.v[1] = mine.v[2] = 0.0;
    T m[6] = {0, 0, 0, 0, 0, 0};   // m00 m01 m02 m11 m12 m22
    V3<T> acc = mk3<T>(0, 0, 0);
    V3<T> bb = mk3<T>(0, 0, 0);    // moving volume-map bodies: boundary term of the right-hand side (lane 0)
    V3<T> axs = mk3<T>(0, 0, 0);   // XS: the XSPH sum
    v4_t<T> xi{}, gi4{};
    T rhoi = T(1);
    if (q.act) {
        const uint32_t i = q.i;
        xi = ldv(B.x, i);
        rhoi = B.density[i];
        const T eps2 = T(0.01) * P.h2;
        // the operator term of neighbour j with its warm start g_j and weight w_j
        auto op = [&](const V3<T> &r, T r2, T wj, const V3<T> &gi, const V3<T> &gj) {
            const T f = wj / (r2 + eps2) * grad_coef_d2(P.K, r2);
            m[0] += f * r.x * r.x; m[1] += f * r.x * r.y; m[2] += f * r.x * r.z;
            m[3] += f * r.y * r.y; m[4] += f * r.y * r.z; m[5] += f * r.z * r.z;
            acc = add(acc, scl(r, f * dot(sub(gi, gj), r)));
        };
        if constexpr (XS) {
            const V3<T> vi = xyz<T>(ldv(B.v, i));
            gi4 = pack(add(vi, xyz<T>(ldv(B.vdiff, i))), P.vd * P.mu * P.mass / rhoi);
            const V3<T> gi = xyz<T>(gi4);
            const bool xs_on = P.xsph != T(0);
            struct XVD {
                v4_t<T> x, v, d;
            };
            fluid_loop<LPP, kUnroll>(P, B, i, q.l,
                                     [&](uint32_t j) { return XVD{ldv(B.x, j), ldv(B.v, j), ldv(B.vdiff, j)}; },
                                     [&](uint32_t, const XVD &d) {
                                         const V3<T> r = diff3<T>(xi, d.x);
                                         const T r2 = dot(r, r);
                                         const T rhoj = (T)d.d.w;
                                         if (xs_on) {
                                             const T w = (P.mass / rhoj) * kernel_W(P.K, dev_sqrt(r2));
                                             axs = add(axs, scl(sub(vi, xyz<T>(d.v)), w));
                                         }
                                         op(r, r2, P.vd * P.mu * P.mass / rhoj, gi,
                                            add(xyz<T>(d.v), xyz<T>(d.d)));
                                     });
        } else {
            gi4 = ldv(B.cg_x, i);
            const V3<T> gi = xyz<T>(gi4);
            struct XG {
                v4_t<T> x, g;
            };
            fluid_loop<LPP, kUnroll>(P, B, i, q.l, [&](uint32_t j) { return XG{ldv(B.x, j), ldv(B.cg_x, j)}; },
                                     [&](uint32_t j, const XG &d) {
                                         if (MP && B.ph[j] != (uint32_t)phase) return;
                                         const V3<T> r = diff3<T>(xi, d.x);
                                         op(r, dot(r, r), (T)d.g.w, gi, xyz<T>(d.g));
                                     });
        }
        if (P.mub != T(0)) {
            boundary_loop<LPP>(P, B, i, q.l, [&](uint32_t j, const v4_t<T> &xj) {
                const V3<T> r = diff3<T>(xi, xj);
                const T r2 = dot(r, r);
                const T f = P.vd * P.mub * (P.rho0 * (T)xj.w / rhoi) / (r2 + eps2) * grad_coef_d2(P.K, r2);
                m[0] += f * r.x * r.x; m[1] += f * r.x * r.y; m[2] += f * r.x * r.z;
                m[3] += f * r.y * r.y; m[4] += f * r.y * r.z; m[5] += f * r.z * r.z;
                // computeRHS (:1130-1138): the boundary particle's velocity
                if (P.bmove) bb = add(bb, scl(r, f * dot(xyz<T>(ldv(B.vbs, j)), r)));
            });
            const uint2 mr = scene_maps(P, q.s);
            if (q.l == 0)   // volume maps: the four samples of each body (diagonalMatrixElement :697-740)
                for (uint32_t b = 0; b < mr.y; b++) {
                    const v4_t<T> xj = ldv(B.bx, b * P.np + i);
                    if (!((T)xj.w > T(0))) continue;
                    const T vol = T(0.25) * (T)xj.w;
                    vmap_samples<T>(xi, xj, P.K.h, [&](const V3<T> &xk) {
                        const V3<T> r = sub(xyz<T>(xi), xk);
                        const T r2 = dot(r, r);
                        const T f = P.vd * P.mub * vol / (r2 + eps2) * grad_coef_d2(P.K, r2);
                        m[0] += f * r.x * r.x; m[1] += f * r.x * r.y; m[2] += f * r.x * r.z;
                        m[3] += f * r.y * r.y; m[4] += f * r.y * r.z; m[5] += f * r.z * r.z;
                        // computeRHS (:1191-1243): the samples' velocities
                        if (P.vmove) bb = add(bb, scl(r, f * dot(vmap_point_velocity<T>(P.vmaps[mr.x + b], xk), r)));
                    });
                }
            acc = add(acc, weiler_boundary<LPP>(P, B, q, xi, rhoi, xyz<T>(gi4)));
        }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) m[k] = gsum<LPP>(m[k]);
    acc = gsum3<LPP>(acc);
    if (P.bmove) bb = gsum3<LPP>(bb);   // the lanes' shares of the boundary list
    if constexpr (XS) axs = gsum3<LPP>(axs);
    if (q.act && q.l == 0) {
        const uint32_t i = q.i;
        if constexpr (XS) xsph_finish(P, B, q.s, i, axs, P.xsph, P.xsph_b, P.div_on);
        const T dt = (T)sc->dt;
        const V3<T> gi = xyz<T>(gi4);
        const T s = dt / rhoi;
        const T a = T(1) - s * m[0], b = -s * m[1], c = -s * m[2], d = T(1) - s * m[3], e = -s * m[4],
                f = T(1) - s * m[5];
        const T A00 = d * f - e * e, A01 = c * e - b * f, A02 = b * e - c * d;
        const T A11 = a * f - c * c, A12 = b * c - a * e, A22 = a * d - b * b;
        const T id = T(1) / (a * A00 + b * A01 + c * A02);
        v4_t<T> i0, i1;
        i0.x = A00 * id; i0.y = A01 * id; i0.z = A02 * id; i0.w = A11 * id;
        i1.x = A12 * id; i1.y = A22 * id; i1.z = 0; i1.w = 0;
        stv(B.inv0, i, i0);
        stv(B.inv1, i, i1);

        V3<T> vi = xyz<T>(ldv(B.v, i));   // b = v_i - dt / rho_i (boundary velocity term)
        if (P.vmove || P.bmove) vi = sub(vi, scl(bb, s));
        const V3<T> Ag = sub(gi, scl(acc, s));
        const V3<T> r = sub(vi, Ag);
        const V3<T> p = sym_mul<T>(i0, i1, r);
        stv(B.cg_r, i, pack(r, T(0)));
        stv(B.cg_p, i, pack(p, (T)gi4.w));
        mine.v[0] = (double)dot(vi, vi);
        mine.v[1] = (double)dot(r, r);
        mine.v[2] = (double)dot(r, p);
    }
    if (MP && other && q.l == 0) stv(B.cg_p, q.i, pack(mk3<T>(0, 0, 0), T(0)));
    const double tol = P.visc_tol;
    const unsigned maxit = P.visc_max_iter;
    const DevParams<T> &PP = P;
    const DevBufs<T> &BB = B;
    grid_sum_finalize<3>(mine, scene_reduce<LPP>(P, B, q), [&](const DSum<3> &tot) {
        if (phase <= 0) {   // the step's first system
            sc->iters_cg_tot = 0;
            sc->cg_zero = 0;
            sc->cg_err_max = 0.0;
        } else if (sc->cg_err > sc->cg_err_max) {   // the phase before this one
            sc->cg_err_max = sc->cg_err;
        }
        sc->cg_rhs2 = tot.v[0];
        sc->iters_cg = 0;
        sc->cg_err = 0.0;
        BB.gsc->loop_guard = 0;
        if (tot.v[0] == 0.0) {
            sc->cg_state = 2;
            if (phase >= 0) sc->cg_zero |= 1u << phase;
        } else {
            double thr = tol * tol * tot.v[0];
            if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
            sc->cg_thresh = thr;
            sc->cg_res2 = tot.v[1];
            if (tot.v[1] < thr) {
                sc->cg_state = 1;
                sc->cg_err = sqrt(tot.v[1] / tot.v[0]);
            } else {
                sc->cg_state = 0;
                sc->cg_absnew = tot.v[2];
            }
        }
        const bool cont = sc->cg_state == 0 && maxit > 0;
        if (sc->cg_state == 0 && maxit == 0) sc->cg_err = sqrt(tot.v[1] / tot.v[0]);
        sc->cont = cont ? 1u : 0u;
        batch_decide(PP, BB, handle, use_handle, true);
    });
}

// tmp = A p and p.tmp -> alpha (ConjugateGradient.h:74-76)
template <class T, int LPP>
__global__ void __launch_bounds__(kBlock) k_cg_matvec(DevParams<T> P, DevBufs<T> B, cudaGraphConditionalHandle h,
                                                       int use_handle, int phase)
{
    count_launch(&B.gsc->launches);
    loop_guard(B.gsc, P.visc_max_iter + 1, h, use_handle);
    SlotInfo q = slot_info<LPP>(P);
    if (phase >= 0 && q.act && B.ph[q.i] != (uint32_t)phase) q.act = false;   // fluid phases
    StepScalars *const sc = B.sc + q.s;
    if (!scene_live(P, sc)) return;   // block uniform: a scene whose CG has stopped
    DSum<1> mine;
    mine.v[0] = 0.0;
    {
        V3<T> acc = mk3<T>(0, 0, 0), pi = mk3<T>(0, 0, 0);
        T rhoi = T(1);
        if (q.act) {
            const uint32_t i = q.i;
            const v4_t<T> xi = ldv(B.x, i);
            rhoi = B.density[i];
            const T eps2 = T(0.01) * P.h2;
            pi = xyz<T>(ldv(B.cg_p, i));
            struct XP {
                v4_t<T> x, p;
            };
            fluid_loop<LPP, kUnroll>(P, B, i, q.l, [&](uint32_t j) { return XP{ldv(B.x, j), ldv(B.cg_p, j)}; },
                                     [&](uint32_t, const XP &d) {
                                         const V3<T> r = diff3<T>(xi, d.x);
                                         const T r2 = dot(r, r);
                                         const T f = (T)d.p.w / (r2 + eps2) * grad_coef_d2(P.K, r2);
                                         acc = add(acc, scl(r, f * dot(sub(pi, xyz<T>(d.p)), r)));
                                     });
            if (P.mub != T(0)) acc = add(acc, weiler_boundary<LPP>(P, B, q, xi, rhoi, pi));
        }
        acc = gsum3<LPP>(acc);
        if (q.act && q.l == 0) {
            const T dt = (T)sc->dt;
            const V3<T> t = sub(pi, scl(acc, dt / rhoi));
            stv(B.cg_t, q.i, pack(t, T(0)));
            mine.v[0] = (double)dot(pi, t);
        }
    }
    grid_sum_finalize<1>(mine, scene_reduce<LPP>(P, B, q),
                         [&](const DSum<1> &tot) { sc->cg_alpha = sc->cg_absnew / tot.v[0]; });
}

// x += alpha p; r -= alpha tmp; |r|^2; z = M^-1 r; r.z -> beta (ConjugateGradient.h:77-88).
// Element arithmetic in the bulk precision, sums accumulated in FP64.
template <class T>
__global__ void __launch_bounds__(kBlock) k_cg_update(DevParams<T> P, DevBufs<T> B, cudaGraphConditionalHandle handle,
                                                       int use_handle, int phase)
{
    count_launch(&B.gsc->launches);
    SlotInfo q = slot_info(P);
    if (phase >= 0 && q.act && B.ph[q.i] != (uint32_t)phase) q.act = false;   // fluid phases
    StepScalars *const sc = B.sc + q.s;
    if (!scene_live(P, sc)) return;   // block uniform: a scene whose CG has stopped
    DSum<2> mine;
    mine.v[0] = mine.v[1] = 0.0;
    if (q.act) {
        const uint32_t i = q.i;
        const T alpha = (T)sc->cg_alpha;
        const V3<T> p = xyz<T>(ldv(B.cg_p, i));
        const V3<T> t = xyz<T>(ldv(B.cg_t, i));
        v4_t<T> x4 = ldv(B.cg_x, i);
        V3<T> x = add(xyz<T>(x4), scl(p, alpha));
        const V3<T> r = sub(xyz<T>(ldv(B.cg_r, i)), scl(t, alpha));
        const V3<T> z = sym_mul<T>(ldv(B.inv0, i), ldv(B.inv1, i), r);
        x4.x = x.x; x4.y = x.y; x4.z = x.z;
        stv(B.cg_x, i, x4);
        stv(B.cg_r, i, pack(r, T(0)));
        stv(B.cg_z, i, pack(z, T(0)));
        mine.v[0] = (double)dot(r, r);
        mine.v[1] = (double)dot(r, z);
    }
    const unsigned maxit = P.visc_max_iter;
    const DevParams<T> &PP = P;
    const DevBufs<T> &BB = B;
    grid_sum_finalize<2>(mine, scene_reduce(P, B, q), [&](const DSum<2> &tot) {
        {
            sc->cg_res2 = tot.v[0];
            sc->cg_err = sqrt(tot.v[0] / sc->cg_rhs2);
            bool cont;
            if (tot.v[0] < sc->cg_thresh) {
                sc->cg_state = 1;
                cont = false;
            } else {
                const double absOld = sc->cg_absnew;
                sc->cg_absnew = tot.v[1];
                sc->cg_beta = tot.v[1] / absOld;
                sc->iters_cg += 1;
                sc->iters_cg_tot += 1;
                cont = sc->iters_cg < maxit;
            }
            sc->cont = cont ? 1u : 0u;
        }
        batch_decide(PP, BB, handle, use_handle, false);
    });
}

// p = z + beta p (ConjugateGradient.h:88) for scenes whose CG continues; the weight in p.w is kept
template <class T>
__global__ void __launch_bounds__(kBlock) k_cg_p(DevParams<T> P, DevBufs<T> B, int phase)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    if (phase >= 0 && B.ph[q.i] != (uint32_t)phase) return;   // fluid phases
    const StepScalars *sc = B.sc + q.s;
    if (sc->cg_state != 0 || sc->cont == 0) return;
    const uint32_t i = q.i;
    const T beta = (T)sc->cg_beta;
    const V3<T> z = xyz<T>(ldv(B.cg_z, i));
    v4_t<T> p = ldv(B.cg_p, i);
    p.x = z.x + beta * (T)p.x;
    p.y = z.y + beta * (T)p.y;
    p.z = z.z + beta * (T)p.z;
    stv(B.cg_p, i, p);
}

// ==========================================================================
// viscosity forces + CFL + velocity kick
// ==========================================================================
// applyForces (Viscosity_Weiler2018.cpp:928-936): a += (x - v)/dt, vDiff = x - v;
// updateTimeStepSizeCFL (Simulation.cpp:415-492): max |v + a h|^2 over the scene's particles;
// kick v += h a (TimeStepDFSPH.cpp:192-208).  The scene's last block computes its dt_next.
template <class T>
__global__ void __launch_bounds__(kBlock) k_kick(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    StepScalars *const sc = B.sc + q.s;
    T m = T(0);                  // |v + a h|^2 in the context's precision
    const double hd = sc->dt;
    if (q.act) {
        const uint32_t i = q.i;
        const T h = (T)hd;
        V3<T> a = xyz<T>(ldv(B.a, i));
        v4_t<T> v4 = ldv(B.v, i);
        const V3<T> v = xyz<T>(v4);
        if (P.visc_on) {
            // a zero right-hand side has the solution 0 (per phase with fluid phases)
            const bool zero = P.nphase > 1 ? ((sc->cg_zero >> B.ph[i]) & 1u) != 0u : sc->cg_state == 2;
            const V3<T> x = zero ? mk3<T>(0, 0, 0) : xyz<T>(ldv(B.cg_x, i));
            const V3<T> dv = sub(x, v);
            a = add(a, scl(dv, T(1) / h));
            stv(B.vdiff, i, pack(dv, T(0)));
            stv(B.a, i, pack(a, T(0)));
        }
        const V3<T> vn = add(v, scl(a, h));
        const T m2 = dot(vn, vn);
        if (!(m2 <= T(3.0e38))) atomicOr(&sc->flags, kFlagNonFinite);
        m = m2;
        if (!(m >= T(0))) m = T(0);
        v4.x = vn.x; v4.y = vn.y; v4.z = vn.z;
        stv(B.v, i, v4);
    }
    // block max -> atomicMax on the bits (non-negative floats / doubles order like unsigned integers)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ T wm[32];
    __shared__ bool amLast;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wm[warp] = m;
    __syncthreads();
    const ReduceSlot rs = scene_reduce(P, B, q);
    if (threadIdx.x == 0) {
        T bm = T(0);
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) bm = fmax(bm, wm[w]);
        if constexpr (sizeof(T) == 8) atomicMax(&sc->maxvel_bits64, (unsigned long long)__double_as_longlong((double)bm));
        else atomicMax(&sc->maxvel_bits, __float_as_uint((float)bm));
        __threadfence();
        const unsigned t = atomicAdd(rs.counter, 1u);
        amLast = (t == rs.count - 1);
    }
    __syncthreads();
    if (amLast && threadIdx.x == 0) {
        __threadfence();
        double maxVel;
        if constexpr (sizeof(T) == 8) {
            maxVel = __longlong_as_double((long long)atomicAdd(&sc->maxvel_bits64, 0ull));
            sc->maxvel_bits64 = 0ull;
        } else {
            maxVel = (double)__uint_as_float(atomicAdd(&sc->maxvel_bits, 0u));
            sc->maxvel_bits = 0;
        }
        *rs.counter = 0;
        double hn = hd;
        if (P.cfl_method != 0) {
            // moving volume-map bodies: |w x (maxDist, 0, 0) + v| against the squared fluid speeds,
            // as the reference compares them (Simulation.cpp:466-476, SimulatorBase.cpp:1670-1687)
            if (P.vmove) {
                const uint2 mr = scene_maps(P, q.s);
                for (uint32_t b = mr.x; b < mr.x + mr.y; b++) {
                    const VMapDev<T> &m = P.vmaps[b];
                    const double vx = (double)m.v[0], vy = (double)m.v[1] + (double)m.w[2] * (double)m.max_dist,
                                 vz = (double)m.v[2] - (double)m.w[1] * (double)m.max_dist;
                    maxVel = fmax(maxVel, sqrt(vx * vx + vy * vy + vz * vz));
                }
            }
            if (maxVel < 1.0e-9) maxVel = 1.0e-9;
            hn = P.cfl_factor * 0.4 * (2.0 * P.radius / sqrt(maxVel));
            hn = fmin(hn, P.cfl_max);
            hn = fmax(hn, P.cfl_min);
            if (P.cfl_method == 2 && sc->prev_iters != 0) {
                double hh = hd;
                if (sc->prev_iters > 10) hh *= 0.9;
                else if (sc->prev_iters < 5) hh *= 1.1;
                hn = fmin(hh, hn);
            }
        }
        sc->dt_next = hn;
    }
}

// computeDensityAdv (TimeStepDFSPH.cpp:1190-1243) and the pressure-solve set-up
// (:264-309): advected density, warm-started kappa (USE_WARMSTART).
template <class T, int LPP>
__global__ void __launch_bounds__(kBlock) k_press_init(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info<LPP>(P);
    T accf = T(0);
    V3<T> vi = mk3<T>(0, 0, 0);
    if (q.act) {
        const v4_t<T> xi = ldv(B.x, q.i);
        vi = xyz<T>(ldv(B.v, q.i));
        struct XV {
            v4_t<T> x, v;
        };
        fluid_loop<LPP, kUnroll>(P, B, q.i, q.l, [&](uint32_t j) { return XV{ldv(B.x, j), ldv(B.v, j)}; },
                                 [&](uint32_t, const XV &d) {
                                     const V3<T> r = diff3<T>(xi, d.x);
                                     accf += grad_coef_d2(P.K, dot(r, r)) * dot(sub(vi, xyz<T>(d.v)), r);
                                 });
    }
    accf = gsum<LPP>(accf);
    if (!q.act || q.l != 0) return;
    const uint32_t i = q.i;
    const T h = (T)B.sc[q.s].dt_next;
    T accb = dot(vi, xyz<T>(ldv(B.bg, i)));
    if (P.vmove || P.bmove) accb -= (T)ldv(B.bv, i).w;   // moving boundaries: (v_i - v_b) . gradW
    const T dadv = B.density[i] / rho0_at(P, B, i) + h * (accf * P.V + accb);
    B.dadv[i] = dadv;
    const T invH2 = T(1) / (h * h);
    const T k = B.kappa[i];
    const T kn = dadv > T(1) ? T(0.5) * (k < T(0.00025) ? k : T(0.00025)) * invH2 : T(0);
    B.kappa[i] = kn;
    store_w(B.xk, i, kn);
}

// x += h_old v (TimeStepDFSPH.cpp:220-237) accumulated in FP64 (double-float
// compensated positions in FP32 mode), kappa *= h_new^2 (:365-383); the scene's
// last block advances its time (:248) and makes dt_next its next step size.
// (s, e) with s + e = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (x, lo) <- x + lo + (hh + hl) v in double-float arithmetic: the product hh v exactly (p + pe,
// FMA), x + p exactly (TwoSum), the small terms in FP32 and a final TwoSum; the new pair holds
// the sum to about 2^-47 of |x| (FP64 rounding of the same sum: 2^-53)
__device__ __forceinline__ void df_advance(float &x, float &lo, float hh, float hl, float v)
{
    const float p = __fmul_rn(hh, v);
    const float pe = __fmaf_rn(hh, v, -p);
    float s, e;
    two_sum(x, p, s, e);
    const float t = __fadd_rn(e, __fadd_rn(lo, __fadd_rn(pe, __fmul_rn(hl, v))));
    two_sum(s, t, x, lo);
}

template <class T>
__global__ void __launch_bounds__(kBlock) k_integrate(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    StepScalars *const sc = B.sc + q.s;
    // FP32: the step sizes as float pairs, split once per block (FP64 runs at a small fraction
    // of the FP32 rate on this part)
    __shared__ float hsplit[4];
    if (sizeof(T) == 4 && threadIdx.x == 0) {
        const double h = sc->dt, hn2 = sc->dt_next * sc->dt_next;
        hsplit[0] = (float)h;
        hsplit[1] = (float)(h - (double)hsplit[0]);
        hsplit[2] = (float)hn2;
        hsplit[3] = (float)(hn2 - (double)hsplit[2]);
    }
    __syncthreads();
    if (q.act) {
        const uint32_t i = q.i;
        v4_t<T> x = ldv(B.x, i);
        const v4_t<T> v = ldv(B.v, i);
        if constexpr (sizeof(T) == 4) {
            float4 lo = B.xlo[i];
            df_advance(x.x, lo.x, hsplit[0], hsplit[1], v.x);
            df_advance(x.y, lo.y, hsplit[0], hsplit[1], v.y);
            df_advance(x.z, lo.z, hsplit[0], hsplit[1], v.z);
            lo.w = 0.f;
            B.xlo[i] = lo;
            // kappa h_new^2 with h_new^2 as a float pair
            const float k = B.kappa[i];
            B.kappa[i] = __fmaf_rn(k, hsplit[2], __fmul_rn(k, hsplit[3]));
        } else {
            const double h = sc->dt, hn = sc->dt_next;
            x.x = x.x + h * v.x;
            x.y = x.y + h * v.y;
            x.z = x.z + h * v.z;
            B.kappa[i] = B.kappa[i] * (hn * hn);
        }
        stv(B.x, i, x);
    }
    const double h = sc->dt;
    const double hn = sc->dt_next;
    __shared__ bool amLast;
    __syncthreads();
    const ReduceSlot rs = scene_reduce(P, B, q);
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(rs.counter, 1u);
        amLast = (t == rs.count - 1);
    }
    __syncthreads();
    if (amLast && threadIdx.x == 0) {
        *rs.counter = 0;
        sc->time += h;
        sc->dt_used = h;
        sc->dt = hn;
        sc->prev_iters = sc->iters;
    }
}

// ==========================================================================
// forces of the fluid on dynamic boundary bodies
// ==========================================================================
// BoundaryModel::addForce (BoundaryModel.h:38-49) collects for each dynamic body the force
// F = sum f and the torque T = sum (x_b - c) x f over the forces f that the fluid exerts on
// its boundary particles.  One thread per boundary particle of a dynamic body gathers the
// forces of its fluid neighbours: it walks the same cell grid and applies the same distance
// predicate, pair_d2(x_i, x_b) < h^2, as the fluid-to-boundary lists, so its pairs are
// exactly the pairs of those lists.  Blocks never span two bodies, and the body's last block
// sums the block partials in block order: the sums are deterministic.
//   phase 0, before the kick (positions, densities and the divergence solve's kappa_v in
//   xk.w, v after the divergence solve, the viscosity solution in cg_x):
//     divergence solve's final pressure term  f = m kappa_v_i V_b gradW_ib
//         (TimeStepDFSPH.cpp:514 with computePressureAccel :1337-1344),
//     XSPH boundary term  f = m (c_b / h) (rho0 V_b / rho_i) W_ib v_i   (XSPH.cpp:183-203),
//     Weiler2018 boundary term  f = -(m / rho_i) d mub (rho0 V_b / rho_i) (v'_i . x_ib) /
//         (|x_ib|^2 + 0.01 h_s^2) gradW_ib   (Viscosity_Weiler2018.cpp:960-975);
//   phase 1, after the pressure solve's last iteration (kappa in xk.w):
//     pressure term  f = m kappa_i V_b gradW_ib   (TimeStepDFSPH.cpp:359).
// Boundary particles are static (v_b = 0).
template <class T, int PHASE>
__global__ void __launch_bounds__(kBlock) k_body_forces(DevParams<T> P, DevBufs<T> B, BodyDev D)
{
    count_launch(&B.gsc->launches);
    const uint4 bk = D.blk[blockIdx.x];
    const uint32_t body = bk.x;
    const uint32_t e = bk.y + threadIdx.x;
    DSum<6> mine;
#pragma unroll
    for (int k = 0; k < 6; k++) mine.v[k] = 0.0;
    if (e < bk.z) {
        const uint32_t j = B.binv[D.slot[e]];   // the body's particles in upload order
        const v4_t<T> xb = ldv(B.xb, j);
        const V3<T> vbj = P.bmove ? xyz<T>(ldv(B.vbs, j)) : mk3<T>(0, 0, 0);   // a moving body's particle
        const uint32_t s = B.bscene ? B.bscene[j] : 0u;
        const SceneDev<T> S = scene_get(P, s);
        const StepScalars *sc = B.sc + s;
        const T Vb = (T)xb.w;
        const bool press = PHASE == 1 || P.div_on;
        const bool xs = PHASE == 0 && P.xsph_b != T(0);
        // (fluid phases: per particle, below)
        const bool visc = PHASE == 0 && P.visc_on && P.mub != T(0) && (P.nphase > 1 || sc->cg_state != 2u);
        const T xs_c = xs ? P.xsph_b / (T)sc->dt * P.rho0 * Vb : T(0);
        const T vi_c = P.vd * P.mub * P.rho0 * Vb;
        const T eps2 = T(0.01) * P.h2;
        double f[3] = {0.0, 0.0, 0.0};
        int cx, cy, cz;
        cell_of(S, xb, cx, cy, cz);
        for (int dz = -1; dz <= 1; dz++) {
            const int z = cz + dz;
            if (z < 0 || z >= S.dimz) continue;
            for (int dy = -1; dy <= 1; dy++) {
                const int y = cy + dy;
                if (y < 0 || y >= S.dimy) continue;
                for (int dx = -1; dx <= 1; dx++) {
                    const int x = cx + dx;
                    if (x < 0 || x >= S.dimx) continue;
                    const uint32_t c = S.cell_off + local_cell(S, x, y, z);
                    const uint32_t st = B.cstart[c];
                    if (st == kEmpty) continue;
                    const uint32_t en = B.cend[c];
                    for (uint32_t i = st; i < en; i++) {
                        const v4_t<T> xk = ldv(B.xk, i);
                        T rx, ry, rz;
                        const T d2 = pair_d2(xk, xb, rx, ry, rz);
                        if (!(d2 < P.K.h2)) continue;
                        const V3<T> r = mk3<T>(rx, ry, rz);
                        const T gc = grad_coef_d2(P.K, d2);
                        V3<T> fi = mk3<T>(0, 0, 0);
                        // fluid phases: the neighbour's mass and rest density
                        const T mi = P.nphase > 1 ? P.V * B.r0[i] : P.mass;
                        if (press) {
                            const T kap = (T)xk.w;
                            if (fabs(kap) > P.eps) fi = scl(r, mi * kap * Vb * gc);
                        }
                        if (xs || visc) {
                            const T rhoi = B.density[i];
                            if (xs) {
                                T xsc = xs_c;
                                if (P.nphase > 1) {   // the particle's model's coefficient and rest density
                                    T xf, xb;
                                    phase_xsph(P, B.ph[i], xf, xb);
                                    xsc = xb / (T)sc->dt * B.r0[i] * Vb;
                                }
                                const T w = mi * xsc / rhoi * kernel_W(P.K, dev_sqrt(d2));
                                V3<T> dv = xyz<T>(ldv(B.v, i));
                                if (P.bmove) dv = sub(dv, vbj);
                                fi = add(fi, scl(dv, w));
                            }
                            if (visc && !(P.nphase > 1 && ((sc->cg_zero >> B.ph[i]) & 1u))) {
                                V3<T> nv = xyz<T>(ldv(B.cg_x, i));
                                if (P.bmove) nv = sub(nv, vbj);
                                // fluid phases: mub = nu_b rho0 and rho0 of the particle's phase
                                T vc = vi_c;
                                if (P.nphase > 1) {
                                    T nu, nub;
                                    phase_visc(P, B.ph[i], nu, nub);
                                    vc = P.vd * (nub * B.r0[i]) * B.r0[i] * Vb;
                                }
                                const T a = vc / rhoi * dot(nv, r) / (d2 + eps2) * gc;
                                fi = sub(fi, scl(r, mi / rhoi * a));
                            }
                        }
                        f[0] += (double)fi.x;
                        f[1] += (double)fi.y;
                        f[2] += (double)fi.z;
                    }
                }
            }
        }
        const double *cc = D.center + 3 * (size_t)body;
        const double px = (double)xb.x - cc[0], py = (double)xb.y - cc[1], pz = (double)xb.z - cc[2];
        mine.v[0] = f[0];
        mine.v[1] = f[1];
        mine.v[2] = f[2];
        mine.v[3] = py * f[2] - pz * f[1];
        mine.v[4] = pz * f[0] - px * f[2];
        mine.v[5] = px * f[1] - py * f[0];
    }
    const ReduceSlot rs{D.partials, D.counters + body, bk.w, D.body_nblk[body]};
    double *const acc = D.acc + 6 * (size_t)body;
    grid_sum_finalize<6>(mine, rs, [&](const DSum<6> &tot) {
#pragma unroll
        for (int k = 0; k < 6; k++) acc[k] += tot.v[k];
    });
}

// Forces of the fluid on dynamic volume-map bodies (Bender2019): the branches of the same places
// call addForce(x_j, f) with the particle's boundary point x_j of the body
// (TimeStepDFSPH.cpp:1355-1364 in computePressureAccel, XSPH.cpp:196-204).  Body by body (block
// uniform), each thread forms its particle's force and torque, the block sums them and writes its
// partial; the last block adds the blocks' partials in block order (deterministic).
template <class T, int PHASE>
__global__ void __launch_bounds__(kBlock) k_vmap_forces(DevParams<T> P, DevBufs<T> B, BodyDev D)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    const bool press = PHASE == 1 || P.div_on;
    const bool xs = PHASE == 0 && P.xsph_b != T(0);
    // partials per slot among the block's scene's maps (one scene: the slot is the body)
    const uint2 mr = scene_maps(P, q.s);
    for (uint32_t b = 0; b < P.vmap_max; b++) {   // block uniform
        DSum<6> mine;
#pragma unroll
        for (int k = 0; k < 6; k++) mine.v[k] = 0.0;
        const uint32_t body = b < mr.y ? (P.vmap_info ? P.vmap_info[mr.x + b].x : b) : 0u;
        if (q.act && b < mr.y && D.dynamic[body]) {
            const uint32_t i = q.i;
            const v4_t<T> xj = ldv(B.bx, b * P.np + i);
            const T Vj = (T)xj.w;
            if (Vj > T(0)) {
                const v4_t<T> xk = ldv(B.xk, i);
                const T kap = (T)xk.w;
                const V3<T> r = diff3<T>(xk, xj);
                const T d2 = dot(r, r);
                V3<T> f = mk3<T>(0, 0, 0);
                const T mi = P.nphase > 1 ? P.V * B.r0[i] : P.mass;   // fluid phases
                if (press && fabs(kap) > P.eps) f = scl(r, mi * kap * Vj * grad_coef_d2(P.K, d2));
                const VMapDev<T> &mp = P.vmaps[mr.x + b];
                if (xs) {
                    T xsb = P.xsph_b;
                    if (P.nphase > 1) {   // the particle's model's coefficient
                        T xf;
                        phase_xsph(P, B.ph[i], xf, xsb);
                    }
                    const T w = mi * xsb / (T)B.sc[q.s].dt * rho0_at(P, B, i) * Vj / B.density[i] *
                                kernel_W(P.K, dev_sqrt(d2));
                    V3<T> dv = xyz<T>(ldv(B.v, i));
                    if (P.vmove) dv = sub(dv, vmap_point_velocity<T>(mp, xyz<T>(xj)));
                    f = add(f, scl(dv, w));
                }
                const double *c = D.center + 3 * (size_t)body;
                const double px = (double)xj.x - c[0], py = (double)xj.y - c[1], pz = (double)xj.z - c[2];
                const double fx = (double)f.x, fy = (double)f.y, fz = (double)f.z;
                mine.v[0] = fx;
                mine.v[1] = fy;
                mine.v[2] = fz;
                mine.v[3] = py * fz - pz * fy;
                mine.v[4] = pz * fx - px * fz;
                mine.v[5] = px * fy - py * fx;
                // Weiler2018 applyForces at the four samples (Viscosity_Weiler2018.cpp:1031-1080)
                const bool zero = P.nphase > 1 ? ((B.sc[q.s].cg_zero >> B.ph[i]) & 1u) != 0u : B.sc[q.s].cg_state == 2u;
                if (PHASE == 0 && P.visc_on && P.mub != T(0) && !zero) {
                    const V3<T> nv = xyz<T>(ldv(B.cg_x, i));
                    const T rhoi = B.density[i], vol = T(0.25) * Vj, eps2 = T(0.01) * P.h2;
                    T mub = P.mub;
                    if (P.nphase > 1) {   // the particle's phase
                        T nu, nub;
                        phase_visc(P, B.ph[i], nu, nub);
                        mub = nub * B.r0[i];
                    }
                    vmap_samples<T>(xk, xj, P.K.h, [&](const V3<T> &xs4) {
                        const V3<T> r4 = sub(xyz<T>(xk), xs4);
                        const T r2 = dot(r4, r4);
                        V3<T> dv = nv;
                        if (P.vmove) dv = sub(dv, vmap_point_velocity<T>(mp, xs4));
                        const T a = P.vd * mub * vol * dot(dv, r4) / (r2 + eps2) * grad_coef_d2(P.K, r2);
                        const V3<T> g = scl(r4, -mi / rhoi * a);
                        const double gx = (double)g.x, gy = (double)g.y, gz = (double)g.z;
                        const double qx = (double)xs4.x - c[0], qy = (double)xs4.y - c[1], qz = (double)xs4.z - c[2];
                        mine.v[0] += gx;
                        mine.v[1] += gy;
                        mine.v[2] += gz;
                        mine.v[3] += qy * gz - qz * gy;
                        mine.v[4] += qz * gx - qx * gz;
                        mine.v[5] += qx * gy - qy * gx;
                    });
                }
            }
        }
        const DSum<6> bs = block_sum<6>(mine);
        if (threadIdx.x == 0)
#pragma unroll
            for (int k = 0; k < 6; k++) D.vpartials[((size_t)b * 6 + k) * gridDim.x + blockIdx.x] = bs.v[k];
    }
    __shared__ bool amLast;
    if (threadIdx.x == 0) {
        __threadfence();
        amLast = atomicAdd(D.counters, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    for (uint32_t m = 0; m < P.nvmaps; m++) {   // every map: its body, scene and slot
        uint32_t body = m, slot = m, g0 = 0u, g1 = gridDim.x;
        if (P.vmap_info) {   // a batch: the blocks of the map's scene
            const uint4 inf = P.vmap_info[m];
            const SceneDev<T> S = scene_get(P, inf.y);
            body = inf.x;
            slot = inf.z;
            g0 = S.pstart / kBlock;
            g1 = (S.pstart + S.n + kBlock - 1) / kBlock;
        }
        DSum<6> part;
#pragma unroll
        for (int k = 0; k < 6; k++) part.v[k] = 0.0;
        for (uint32_t g = g0 + threadIdx.x; g < g1; g += blockDim.x)
#pragma unroll
            for (int k = 0; k < 6; k++) part.v[k] += __ldcg(&D.vpartials[((size_t)slot * 6 + k) * gridDim.x + g]);
        const DSum<6> tot = block_sum<6>(part);
        if (threadIdx.x == 0)
#pragma unroll
            for (int k = 0; k < 6; k++) D.acc[6 * (size_t)body + k] += tot.v[k];
    }
    if (threadIdx.x == 0) *D.counters = 0u;
}

// ==========================================================================
// learned warm start
// ==========================================================================
// Network inputs (10, all dimensionless): the raw features f0..f4 of particle i, with f3
// replaced by the previous stored kappa of i relative to its cubic-spline-weighted
// neighbourhood mean, followed by the weighted means of f0..f4 over i and its fluid
// neighbours (sum_j W_ij f_j / sum_j W_ij, self weight W(0)).  Runs before the pressure
// solve overwrites kappa, so B.kappa still holds the previous step's stored value.
template <class T, int LPP>
__global__ void __launch_bounds__(kBlock) k_features(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info<LPP>(P);
    float m[5] = {0, 0, 0, 0, 0};
    float wsum = 0.0f, km = 0.0f;
    if (q.act) {
        const v4_t<T> xi = ldv(B.x, q.i);
        struct XF {
            v4_t<T> x;
            float4 a;
            float b, k;
        };
        fluid_loop<LPP, kUnroll>(P, B, q.i, q.l,
                                 [&](uint32_t j) {
                                     return XF{ldv(B.x, j), *reinterpret_cast<const float4 *>(B.feat + (size_t)j * 8),
                                               B.feat[(size_t)j * 8 + 4], (float)B.kappa[j]};
                                 },
                                 [&](uint32_t, const XF &d) {
                                     const V3<T> r = diff3<T>(xi, d.x);
                                     const float w = (float)kernel_W(P.K, dev_sqrt(dot(r, r)));
                                     m[0] += w * d.a.x; m[1] += w * d.a.y; m[2] += w * d.a.z; m[3] += w * d.a.w;
                                     m[4] += w * d.b;
                                     km += w * d.k;
                                     wsum += w;
                                 });
    }
#pragma unroll
    for (int k = 0; k < 5; k++) m[k] = gsum<LPP>(m[k]);
    wsum = gsum<LPP>(wsum);
    km = gsum<LPP>(km);
    if (!q.act || q.l != 0) return;
    const uint32_t i = q.i;
    const float4 f0 = *reinterpret_cast<const float4 *>(B.feat + (size_t)i * 8);
    const float f4 = B.feat[(size_t)i * 8 + 4];
    const float ki = (float)B.kappa[i];
    const float w0 = (float)P.K.w0;
    m[0] += w0 * f0.x; m[1] += w0 * f0.y; m[2] += w0 * f0.z; m[3] += w0 * f0.w; m[4] += w0 * f4;
    wsum += w0;
    km += w0 * ki;
    float *X = B.mlp_x + (size_t)i * 10;
    X[0] = f0.x; X[1] = f0.y; X[2] = f0.z; X[4] = f4;
    X[3] = km > 0.0f ? ki / km * wsum : 0.0f;   // kappa_i / (weighted mean of kappa)
    const float inv = 1.0f / wsum;
#pragma unroll
    for (int k = 0; k < 5; k++) X[5 + k] = m[k] * inv;
}

// Predicted warm start of one solver: the network's output o times the output scale is a
// multiplier on the previous step's stored kappa_v / kappa, in place of the classic factor
// 0.5 (TimeStepDFSPH.cpp:449-453 divergence, :293-296 pressure), with the classic clamps and
// masks.  Since the classic warm start is 0.5 min(stored, clamp) / h^k where the mask holds
// (and 0 elsewhere), the prediction is 2 m x classic; m is limited to [0, 4].
template <class T, bool DIV>
__global__ void __launch_bounds__(kBlock) k_ws_kappa(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    const uint32_t i = q.i;
    const float o = B.mlp_y[(size_t)i * 2 + (DIV ? 0 : 1)] * (DIV ? P.ws_scale_v : P.ws_scale_p);
    const float mult = fminf(fmaxf(o, 0.0f), 4.0f);   // NaN -> 0 (fmaxf returns the non-NaN operand)
    const T classic = DIV ? B.kappa_v[i] : B.kappa[i];
    B.kl[i] = T(2) * (T)mult * classic;
}

// Pressure accelerations of both candidate warm starts: classic (xk.w) into pa, predicted (kl)
// into pa2 (the computePressureAccel sum of TimeStepDFSPH.cpp:1299-1367 for each).
template <class T, int LPP>
__global__ void __launch_bounds__(kBlock) k_ws_accel2(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info<LPP>(P);
    V3<T> ac = mk3<T>(0, 0, 0), al = mk3<T>(0, 0, 0);
    T pc = T(0), pl = T(0);
    if (q.act) {
        const v4_t<T> xi = ldv(B.xk, q.i);
        pc = (T)xi.w;
        pl = B.kl[q.i];
        struct XK {
            v4_t<T> x;
            T kl;
        };
        fluid_loop<LPP, kUnroll>(P, B, q.i, q.l, [&](uint32_t j) { return XK{ldv(B.xk, j), B.kl[j]}; },
                                 [&](uint32_t, const XK &d) {
                                     const V3<T> r = diff3<T>(xi, d.x);
                                     const T c = grad_coef_d2(P.K, dot(r, r));
                                     const T sc_ = pc + (T)d.x.w, sl = pl + d.kl;
                                     if (fabs(sc_) > P.eps) ac = add(ac, scl(r, c * sc_));
                                     if (fabs(sl) > P.eps) al = add(al, scl(r, c * sl));
                                 });
    }
    ac = gsum3<LPP>(ac);
    al = gsum3<LPP>(al);
    if (!q.act || q.l != 0) return;
    const V3<T> gb = xyz<T>(ldv(B.bg, q.i));
    V3<T> a1 = scl(ac, -P.V), a2 = scl(al, -P.V);
    if (fabs(pc) > P.eps) a1 = sub(a1, scl(gb, pc));
    if (fabs(pl) > P.eps) a2 = sub(a2, scl(gb, pl));
    stv(B.pa, q.i, pack(a1, T(0)));
    stv(B.pa2, q.i, pack(a2, T(0)));
}

// One Jacobi iteration of the solver (TimeStepDFSPH.cpp:621-706 divergence, :544-619
// pressure) for both candidate warm starts at once: aij from the two pressure accelerations,
// the updated kappa of each candidate (classic into kappa_v / kappa and xk.w, predicted into
// kl) and, in the last of the `sweeps` gate iterations, both average errors.  The scene's
// last block then keeps the predicted warm start only if its error is lower, books the
// gate iterations of the chosen candidate and takes the loop decision, so the solver loop
// continues with iteration sweeps + 1.  With one sweep the errors compared are the
// candidates' initial residuals.
template <class T, bool DIV, bool LAST, int LPP>
__global__ void __launch_bounds__(kBlock) k_ws_sweep(DevParams<T> P, DevBufs<T> B, unsigned sweeps,
                                                      cudaGraphConditionalHandle handle, int use_handle)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info<LPP>(P);
    StepScalars *const sc = B.sc + q.s;
    DSum<2> mine;
    mine.v[0] = mine.v[1] = 0.0;
    T s1 = T(0), s2 = T(0);
    V3<T> a1 = mk3<T>(0, 0, 0), a2 = mk3<T>(0, 0, 0);
    if (q.act) {
        const v4_t<T> xi = ldv(B.x, q.i);
        a1 = xyz<T>(ldv(B.pa, q.i));
        a2 = xyz<T>(ldv(B.pa2, q.i));
        struct XA {
            v4_t<T> x, a, b;
        };
        fluid_loop<LPP, kUnroll>(P, B, q.i, q.l, [&](uint32_t j) { return XA{ldv(B.x, j), ldv(B.pa, j), ldv(B.pa2, j)}; },
                                 [&](uint32_t, const XA &d) {
                                     const V3<T> r = diff3<T>(xi, d.x);
                                     const T c = grad_coef_d2(P.K, dot(r, r));
                                     s1 += c * dot(sub(a1, xyz<T>(d.a)), r);
                                     s2 += c * dot(sub(a2, xyz<T>(d.b)), r);
                                 });
    }
    s1 = gsum<LPP>(s1);
    s2 = gsum<LPP>(s2);
    if (q.act && q.l == 0) {
        const uint32_t i = q.i;
        const V3<T> gb = xyz<T>(ldv(B.bg, i));
        T ap1 = s1 * P.V + dot(a1, gb), ap2 = s2 * P.V + dot(a2, gb);
        T si, fac;
        bool zero = false;
        if (DIV) {
            const T h = (T)sc->dt;
            ap1 *= h;
            ap2 *= h;
            si = -B.dadv[i];
            zero = B.nf[i] + B.nbn[i] < 20u;
            fac = B.factor[i] * (T(1) / h);
        } else {
            const T h = (T)sc->dt_next;
            ap1 *= h * h;
            ap2 *= h * h;
            si = T(1) - B.dadv[i];
            fac = B.factor[i] * (T(1) / (h * h));
        }
        T *kap = DIV ? B.kappa_v : B.kappa;
        T k1 = kap[i] - T(0.5) * (si - ap1) * fac;
        T k2 = B.kl[i] - T(0.5) * (si - ap2) * fac;
        k1 = k1 > T(0) ? k1 : T(0);
        k2 = k2 > T(0) ? k2 : T(0);
        kap[i] = k1;
        B.kl[i] = k2;
        store_w(B.xk, i, k1);
        if (LAST && !zero) {
            const T r1 = (si - ap1) < T(0) ? (si - ap1) : T(0);
            const T r2 = (si - ap2) < T(0) ? (si - ap2) : T(0);
            mine.v[0] = -(double)P.rho0 * (double)r1;
            mine.v[1] = -(double)P.rho0 * (double)r2;
        }
    }
    if (!LAST) return;   // uniform over the grid: no block collective follows
    const uint32_t n_s = q.end - q.begin;
    const DevParams<T> &PP = P;
    const DevBufs<T> &BB = B;
    grid_sum_finalize<2>(mine, scene_reduce<LPP>(P, B, q), [&](const DSum<2> &tot) {
        const int k = DIV ? 0 : 1;
        const double inv = n_s ? 1.0 / (double)n_s : 0.0;
        sc->ws_rc[k] = tot.v[0] * inv;
        sc->ws_rl[k] = tot.v[1] * inv;
        const bool learned = tot.v[1] < tot.v[0];
        if (learned) sc->ws_used |= (1u << k);
        else sc->ws_used &= ~(1u << k);
        solver_decide<T, DIV>(PP, sc, (learned ? tot.v[1] : tot.v[0]) * inv, sweeps);
        batch_decide(PP, BB, handle, use_handle, true);
    });
}

// kappa of the chosen candidate after the gate iterations into kappa_v / kappa and xk.w
template <class T, bool DIV>
__global__ void __launch_bounds__(kBlock) k_ws_apply(DevParams<T> P, DevBufs<T> B)
{
    count_launch(&B.gsc->launches);
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    T *kap = DIV ? B.kappa_v : B.kappa;
    T k = kap[q.i];
    if (B.sc[q.s].ws_used & (1u << (DIV ? 0 : 1))) {
        k = B.kl[q.i];
        kap[q.i] = k;
    }
    store_w(B.xk, q.i, k);
}

// ==========================================================================
// boundary set-up
// ==========================================================================
template <class T>
__global__ void __launch_bounds__(kBlock) k_boundary_keys(DevParams<T> P, const v4_t<T> *__restrict__ xb,
                                                           const uint32_t *__restrict__ bscene, uint32_t *keys,
                                                           uint32_t *vals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    const SceneDev<T> S = scene_get(P, bscene ? bscene[i] : 0u);
    int cx, cy, cz;
    cell_of(S, ldv(xb, i), cx, cy, cz);
    keys[i] = S.key_prefix | morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
    vals[i] = i;
}

template <class T>
__global__ void __launch_bounds__(kBlock) k_boundary_gather(DevParams<T> P, DevBufs<T> B, const v4_t<T> *__restrict__ xb_in,
                                                             const uint32_t *__restrict__ bscene_in,
                                                             const uint32_t *__restrict__ perm, uint32_t *cells)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.nb) return;
    const uint32_t src = perm[k];
    v4_t<T> x = ldv(xb_in, src);
    x.w = 0;
    stv(B.xb, k, x);
    B.bid[k] = src;
    if (B.binv) B.binv[src] = k;   // contexts keep the inverse map; the allocation-free path has none
    const uint32_t s = bscene_in ? bscene_in[src] : 0u;
    if (B.bscene) B.bscene[k] = s;
    const SceneDev<T> S = scene_get(P, s);
    int cx, cy, cz;
    cell_of(S, x, cx, cy, cz);
    cells[k] = S.cell_off + local_cell(S, cx, cy, cz);
}

// Moving boundary bodies, every step before the neighbour search (SimulatorBase::updateBoundaryParticles,
// SimulatorBase.cpp:1620-1645): particle u of body b at R_b x0_u + t_b, moving at
// w_b x (R_b x0_u) + v_b; its sort key; the squared speeds enter the step's CFL maximum as the
// reference adds those of moving bodies' particles (Simulation.cpp:442-458), per scene.
template <class T>
__global__ void __launch_bounds__(kBlock) k_boundary_move(DevParams<T> P, DevBufs<T> B, BoundaryMoveDev<T> M,
                                                           uint32_t *keys, uint32_t *vals)
{
    count_launch(&B.gsc->launches);
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    T sp = T(0);
    const uint32_t scene = (M.scene && u < P.nb) ? M.scene[u] : 0u;
    if (u < P.nb) {
        const v4_t<T> x0 = ldv(M.x0, u);
        const BodyMotionDev<T> &m = M.motion[M.body[u]];
        const V3<T> r = mk3<T>(m.R[0] * (T)x0.x + m.R[1] * (T)x0.y + m.R[2] * (T)x0.z,
                               m.R[3] * (T)x0.x + m.R[4] * (T)x0.y + m.R[5] * (T)x0.z,
                               m.R[6] * (T)x0.x + m.R[7] * (T)x0.y + m.R[8] * (T)x0.z);
        const V3<T> x = add(r, mk3<T>(m.t[0], m.t[1], m.t[2]));
        const V3<T> v = mk3<T>(m.w[1] * r.z - m.w[2] * r.y + m.v[0], m.w[2] * r.x - m.w[0] * r.z + m.v[1],
                               m.w[0] * r.y - m.w[1] * r.x + m.v[2]);
        const v4_t<T> xp = pack(x, M.V0[u]);
        stv(M.xtmp, u, xp);
        stv(M.vtmp, u, pack(v, T(0)));
        const SceneDev<T> S = scene_get(P, scene);
        int cx, cy, cz;
        cell_of(S, xp, cx, cy, cz);
        keys[u] = S.key_prefix | morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
        vals[u] = u;
        sp = dot(v, v);
    }
    // the scene's maximum, in the encoding of the kick's fluid maximum: one atomic per warp of one
    // scene (the scenes' particles are contiguous), one per lane otherwise
    auto publish = [&](T m, uint32_t s) {
        if (!(m > T(0))) return;
        StepScalars *sc = B.sc + s;
        if constexpr (sizeof(T) == 8) atomicMax(&sc->maxvel_bits64, (unsigned long long)__double_as_longlong((double)m));
        else atomicMax(&sc->maxvel_bits, __float_as_uint((float)m));
    };
    const uint32_t s0 = __shfl_sync(0xffffffffu, scene, 0);
    if (__all_sync(0xffffffffu, scene == s0)) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sp = fmax(sp, __shfl_xor_sync(0xffffffffu, sp, o));
        if ((threadIdx.x & 31u) == 0) publish(sp, s0);
    } else {
        publish(sp, scene);
    }
}

// ... sorted into the boundary grid: positions (w = V), velocities, slot maps, cells
template <class T>
__global__ void __launch_bounds__(kBlock) k_boundary_regather(DevParams<T> P, DevBufs<T> B, BoundaryMoveDev<T> M,
                                                               const uint32_t *__restrict__ perm, uint32_t *cells)
{
    count_launch(&B.gsc->launches);
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.nb) return;
    const uint32_t src = perm[k];
    const v4_t<T> x = ldv(M.xtmp, src);
    stv(B.xb, k, x);
    stv(B.vbs, k, ldv(M.vtmp, src));
    B.bid[k] = src;
    B.binv[src] = k;
    const uint32_t sn = M.scene ? M.scene[src] : 0u;
    if (B.bscene) B.bscene[k] = sn;
    const SceneDev<T> S = scene_get(P, sn);
    int cx, cy, cz;
    cell_of(S, x, cx, cy, cz);
    cells[k] = S.cell_off + local_cell(S, cx, cy, cz);
}

// BoundaryModel_Akinci2012::computeBoundaryVolume (BoundaryModel_Akinci2012.cpp:48-75):
// V_b = 1 / (W0 + sum over the boundary neighbours of the same scene of W), over the particles
// of every body together.  Simulation::updateBoundaryVolume (Simulation.cpp:700-746) activates
// the static bodies, then each dynamic or animated body, with set_active(i, true, true), and a
// point set activated so searches every other point set: each body's sum covers the boundary
// particles of all bodies.
template <class T>
__global__ void __launch_bounds__(kBlock) k_boundary_volume(DevParams<T> P, DevBufs<T> B)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    const SceneDev<T> S = scene_get(P, B.bscene ? B.bscene[i] : 0u);
    v4_t<T> xi = ldv(B.xb, i);
    int cx, cy, cz;
    cell_of(S, xi, cx, cy, cz);
    T delta = P.K.w0;
    for (int dz = -1; dz <= 1; dz++) {
        const int z = cz + dz;
        if (z < 0 || z >= S.dimz) continue;
        for (int dy = -1; dy <= 1; dy++) {
            const int y = cy + dy;
            if (y < 0 || y >= S.dimy) continue;
            for (int dx = -1; dx <= 1; dx++) {
                const int x = cx + dx;
                if (x < 0 || x >= S.dimx) continue;
                const uint32_t c = S.cell_off + local_cell(S, x, y, z);
                const uint32_t s = B.bcstart[c];
                if (s == kEmpty) continue;
                const uint32_t e = B.bcend[c];
                for (uint32_t j = s; j < e; j++) {
                    if (j == i) continue;
                    T ddx, ddy, ddz;
                    const T d2 = pair_d2(xi, ldv(B.xb, j), ddx, ddy, ddz);
                    if (d2 < P.K.h2) delta += kernel_W(P.K, dev_sqrt(d2));
                }
            }
        }
    }
    // stored by a second pass: the w lane of xb is read by other threads here
    B.bscratch[i] = T(1) / delta;
}

template <class T>
__global__ void __launch_bounds__(kBlock) k_boundary_volume_store(DevParams<T> P, DevBufs<T> B)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nb) return;
    v4_t<T> x = ldv(B.xb, i);
    x.w = B.bscratch[i];
    stv(B.xb, i, x);
}

// ==========================================================================
// host <-> device field transfer helpers
// ==========================================================================
// slot i of scene s takes upload entry u = ustart_s + (i - begin_s); its id is id[u] (or u)
template <class T>
__global__ void k_init_state(DevParams<T> P, DevBufs<T> B, const double *__restrict__ x, const double *__restrict__ v,
                             const uint32_t *__restrict__ id)
{
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    const uint32_t i = q.i;
    const uint32_t u = scene_get(P, q.s).ustart + (i - q.begin);
    v4_t<T> xx, vv, zz;
    xx.x = (T)x[3 * (size_t)u]; xx.y = (T)x[3 * (size_t)u + 1]; xx.z = (T)x[3 * (size_t)u + 2]; xx.w = 0;
    vv.x = (T)v[3 * (size_t)u]; vv.y = (T)v[3 * (size_t)u + 1]; vv.z = (T)v[3 * (size_t)u + 2]; vv.w = 0;
    zz.x = zz.y = zz.z = zz.w = 0;
    stv(B.x, i, xx);
    stv(B.v, i, vv);
    stv(B.vdiff, i, zz);
    if (B.xlo)
        B.xlo[i] = make_float4((float)(x[3 * (size_t)u] - (double)xx.x), (float)(x[3 * (size_t)u + 1] - (double)xx.y),
                               (float)(x[3 * (size_t)u + 2] - (double)xx.z), 0.f);
    B.kappa[i] = 0;
    B.kappa_v[i] = 0;
    B.id[i] = id ? id[u] : u;
}

template <class T>
__global__ void k_inverse_perm(DevParams<T> P, const uint32_t *__restrict__ id, uint32_t *__restrict__ inv)
{
    const SlotInfo q = slot_info(P);
    if (q.act && id[q.i] < P.nreal) inv[id[q.i]] = q.i;
}

template <class T> __device__ __forceinline__ void put(void *out, int dt, size_t idx, double v)
{
    if (dt == SPHGB_DTYPE_F32) static_cast<float *>(out)[idx] = (float)v;
    else if (dt == SPHGB_DTYPE_F64) static_cast<double *>(out)[idx] = v;
    else static_cast<uint32_t *>(out)[idx] = (uint32_t)v;
}
template <class T> __device__ __forceinline__ double get(const void *in, int dt, size_t idx)
{
    if (dt == SPHGB_DTYPE_F32) return (double)static_cast<const float *>(in)[idx];
    if (dt == SPHGB_DTYPE_F64) return static_cast<const double *>(in)[idx];
    return (double)static_cast<const uint32_t *>(in)[idx];
}

// boundary field of sorted boundary particle k, written at its upload index
template <class T>
__global__ void k_scatter_boundary(DevParams<T> P, DevBufs<T> B, int field, void *out, int odt)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.nb) return;
    const v4_t<T> x = ldv(B.xb, k);
    const uint32_t d = B.bid[k];
    if (field == SPHGB_FIELD_BOUNDARY_VOLUME) {
        put<T>(out, odt, d, (double)x.w);
    } else {
        put<T>(out, odt, 3 * (size_t)d, (double)x.x);
        put<T>(out, odt, 3 * (size_t)d + 1, (double)x.y);
        put<T>(out, odt, 3 * (size_t)d + 2, (double)x.z);
    }
}

// field value of the particle in slot k (scene s), written at its particle id d
template <class T>
__device__ __forceinline__ void emit_field(const DevParams<T> &P, const DevBufs<T> &B, int field, void *out, int odt,
                                           uint32_t k, uint32_t d, uint32_t s)
{
    const double hn = B.sc[s].dt_next;
    auto vec = [&](const v4_t<T> *arr, const float4 *lo) {
        const v4_t<T> a = ldv(arr, k);
        double ax = (double)a.x, ay = (double)a.y, az = (double)a.z;
        if (lo) { const float4 l = lo[k]; ax += l.x; ay += l.y; az += l.z; }
        put<T>(out, odt, 3 * (size_t)d, ax);
        put<T>(out, odt, 3 * (size_t)d + 1, ay);
        put<T>(out, odt, 3 * (size_t)d + 2, az);
    };
    switch (field) {
    case SPHGB_FIELD_POSITION: vec(B.x, B.xlo); break;
    case SPHGB_FIELD_VELOCITY: vec(B.v, nullptr); break;
    case SPHGB_FIELD_ACCELERATION: vec(B.a, nullptr); break;
    case SPHGB_FIELD_PRESSURE_ACCEL: vec(B.pa, nullptr); break;
    case SPHGB_FIELD_VDIFF: vec(B.vdiff, nullptr); break;
    case SPHGB_FIELD_DENSITY: put<T>(out, odt, d, (double)B.density[k]); break;
    case SPHGB_FIELD_FACTOR_RAW: put<T>(out, odt, d, (double)B.factor[k]); break;
    case SPHGB_FIELD_FACTOR: put<T>(out, odt, d, (double)B.factor[k] / (hn * hn)); break;
    case SPHGB_FIELD_DENSITY_ADV: put<T>(out, odt, d, (double)B.dadv[k]); break;
    case SPHGB_FIELD_PRESSURE_RHO2: put<T>(out, odt, d, (double)B.kappa[k]); break;
    case SPHGB_FIELD_PRESSURE_RHO2_V: put<T>(out, odt, d, (double)B.kappa_v[k]); break;
    case SPHGB_FIELD_PARTICLE_ID: put<T>(out, odt, d, (double)B.id[k]); break;
    case SPHGB_FIELD_NUM_FLUID_NEIGHBORS: put<T>(out, odt, d, (double)B.nf[k]); break;
    case SPHGB_FIELD_NUM_BOUNDARY_NEIGHBORS: put<T>(out, odt, d, (double)B.nbn[k]); break;
    case SPHGB_FIELD_FEATURES:
        if (B.mlp_x)
            for (int c = 0; c < 10; c++) put<T>(out, odt, 10 * (size_t)d + c, (double)B.mlp_x[(size_t)k * 10 + c]);
        break;
    case SPHGB_FIELD_POSITION_HI: vec(B.x, nullptr); break;
    case SPHGB_FIELD_STATE:       // every particle the device steps is Active (ParticleState 0)
    case SPHGB_FIELD_OBJECT_ID:   // the device keeps no object ids
        put<T>(out, odt, d, 0.0);
        break;
    case SPHGB_FIELD_POSITION_LO: {
        const float4 l = B.xlo ? B.xlo[k] : make_float4(0.f, 0.f, 0.f, 0.f);
        put<T>(out, odt, 3 * (size_t)d, (double)l.x);
        put<T>(out, odt, 3 * (size_t)d + 1, (double)l.y);
        put<T>(out, odt, 3 * (size_t)d + 2, (double)l.z);
        break;
    }
    default: break;
    }
}

// every slot's field value written at its particle id (a scattered write: device memory)
template <class T>
__global__ void k_scatter_field(DevParams<T> P, DevBufs<T> B, int field, void *out, int odt)
{
    const SlotInfo q = slot_info(P);
    if (!q.act) return;
    emit_field(P, B, field, out, odt, q.i, B.id[q.i], q.s);
}

// ... in particle-id order into host memory the device maps, several fields per launch: thread t
// of a block takes particle d0 + t from its slot inv[d] once; for each field it stages the value
// in shared memory, and the block writes its particles' values out as one contiguous range, with
// 16-byte stores where that range is 16-byte aligned (whole lines over the host link instead of
// strided 4-byte pieces)
template <class T>
__global__ void __launch_bounds__(kBlock) k_gather_fields(DevParams<T> P, DevBufs<T> B, FieldSet F, int odt,
                                                          const uint32_t *__restrict__ inv)
{
    __shared__ __align__(16) unsigned char buf[kBlock * kFieldSetMaxComps * 8];
    const uint32_t d0 = blockIdx.x * kBlock, d = d0 + threadIdx.x;
    uint32_t k = 0u, sc = 0u;
    if (d < P.nreal) {
        k = inv[d];
        sc = P.nscenes > 1 ? __ldg(P.blk + k / kBlock).x : 0u;
    }
    const size_t es = odt == SPHGB_DTYPE_F64 ? 8 : 4;
    const uint32_t cnt = min((uint32_t)kBlock, P.nreal - d0);   // every launched block holds a particle
    for (uint32_t f = 0; f < F.n; f++) {
        if (d < P.nreal) emit_field(P, B, F.field[f], buf, odt, k, threadIdx.x, sc);
        __syncthreads();
        const size_t bytes = (size_t)cnt * F.comps[f] * es;
        unsigned char *dst = static_cast<unsigned char *>(F.ptr[f]) + (size_t)d0 * F.comps[f] * es;
        size_t done = 0;
        if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
            const size_t nv = bytes / 16;
            for (size_t i = threadIdx.x; i < nv; i += kBlock)
                reinterpret_cast<float4 *>(dst)[i] = reinterpret_cast<const float4 *>(buf)[i];
            done = nv * 16;
        }
        for (size_t i = done / 4 + threadIdx.x; i < bytes / 4; i += kBlock)
            reinterpret_cast<uint32_t *>(dst)[i] = reinterpret_cast<const uint32_t *>(buf)[i];
        __syncthreads();   // the next field reuses the staging buffer
    }
}

// value d of an uploaded field (particle-id ordered input `in`) written to slot k
template <class T>
__device__ __forceinline__ void apply_field(const DevBufs<T> &B, int field, const void *in, int idt, uint32_t k,
                                            uint32_t d)
{
    auto vec = [&](v4_t<T> *arr, float4 *lo) {
        const double ax = get<T>(in, idt, 3 * (size_t)d), ay = get<T>(in, idt, 3 * (size_t)d + 1),
                     az = get<T>(in, idt, 3 * (size_t)d + 2);
        v4_t<T> a = ldv(arr, k);
        a.x = (T)ax; a.y = (T)ay; a.z = (T)az;
        stv(arr, k, a);
        if (lo) lo[k] = make_float4((float)(ax - (double)a.x), (float)(ay - (double)a.y), (float)(az - (double)a.z), 0.f);
    };
    switch (field) {
    case SPHGB_FIELD_POSITION: vec(B.x, B.xlo); break;
    case SPHGB_FIELD_VELOCITY: vec(B.v, nullptr); break;
    case SPHGB_FIELD_VDIFF: vec(B.vdiff, nullptr); break;
    case SPHGB_FIELD_PRESSURE_RHO2: B.kappa[k] = (T)get<T>(in, idt, d); break;
    case SPHGB_FIELD_PRESSURE_RHO2_V: B.kappa_v[k] = (T)get<T>(in, idt, d); break;
    case SPHGB_FIELD_POSITION_HI: {   // the stored high part; the low part is left as it is
        v4_t<T> a = ldv(B.x, k);
        a.x = (T)get<T>(in, idt, 3 * (size_t)d);
        a.y = (T)get<T>(in, idt, 3 * (size_t)d + 1);
        a.z = (T)get<T>(in, idt, 3 * (size_t)d + 2);
        stv(B.x, k, a);
        break;
    }
    case SPHGB_FIELD_POSITION_LO:
        if (B.xlo)
            B.xlo[k] = make_float4((float)get<T>(in, idt, 3 * (size_t)d), (float)get<T>(in, idt, 3 * (size_t)d + 1),
                                   (float)get<T>(in, idt, 3 * (size_t)d + 2), 0.f);
        break;
    default: break;
    }
}

// Uploaded fields in particle-id order, several per launch.  For each field the block reads its
// particles' values (one contiguous range of the input, which may be host memory the device
// maps) into shared memory, with 16-byte loads where the range is 16-byte aligned; thread t then
// writes particle d0 + t's values to its slot inv[d0 + t].
template <class T>
__global__ void __launch_bounds__(kBlock) k_upload_fields(DevParams<T> P, DevBufs<T> B, FieldSet F, int idt,
                                                          const uint32_t *__restrict__ inv)
{
    __shared__ __align__(16) unsigned char buf[kBlock * 3 * 8];   // uploadable fields: at most 3 components
    const uint32_t d0 = blockIdx.x * kBlock;
    const size_t es = idt == SPHGB_DTYPE_F64 ? 8 : 4;
    const uint32_t cnt = min((uint32_t)kBlock, P.nreal - d0);   // every launched block holds a particle
    const bool mine = d0 + threadIdx.x < P.nreal;
    const uint32_t k = mine ? inv[d0 + threadIdx.x] : 0u;
    for (uint32_t f = 0; f < F.n; f++) {
        const size_t bytes = (size_t)cnt * F.comps[f] * es;
        const unsigned char *src = static_cast<const unsigned char *>(F.ptr[f]) + (size_t)d0 * F.comps[f] * es;
        size_t done = 0;
        if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
            const size_t nv = bytes / 16;
            for (size_t i = threadIdx.x; i < nv; i += kBlock)
                reinterpret_cast<float4 *>(buf)[i] = reinterpret_cast<const float4 *>(src)[i];
            done = nv * 16;
        }
        for (size_t i = done / 4 + threadIdx.x; i < bytes / 4; i += kBlock)
            reinterpret_cast<uint32_t *>(buf)[i] = reinterpret_cast<const uint32_t *>(src)[i];
        __syncthreads();
        if (mine) apply_field(B, F.field[f], buf, idt, k, threadIdx.x);
        __syncthreads();   // the next field reuses the staging buffer
    }
}

// Big-endian copy of n words of `bytes` bytes each (4 or 8), in place (file formats such as
// legacy VTK store big-endian binary data)
__global__ void k_byteswap(void *data, size_t n, int bytes)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (bytes == 8) {
        unsigned long long *p = static_cast<unsigned long long *>(data) + k;
        const unsigned long long v = *p;
        const uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
        *p = ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | (unsigned long long)__byte_perm(hi, 0, 0x0123);
    } else {
        uint32_t *p = static_cast<uint32_t *>(data) + k;
        *p = __byte_perm(*p, 0, 0x0123);
    }
}

// Neighbour lists to particle ids, CSR (debug / oracle comparison path).  kind 0: fluid
// list in the layout of lpp_log2, kind 1: boundary list.
__global__ void k_lists_to_ids(const uint32_t *__restrict__ list, const uint32_t *__restrict__ cnt, uint32_t cap,
                               const uint32_t *__restrict__ id, const uint32_t *__restrict__ inv,
                               const uint32_t *__restrict__ bid, int kind, uint32_t lpp_log2,
                               const uint32_t *__restrict__ offsets, uint32_t *__restrict__ out, uint32_t n)
{
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;   // particle id
    if (d >= n) return;
    const uint32_t k = inv[d];
    const uint32_t c = min(cnt[k], cap);
    uint32_t *o = out + offsets[d];
    for (uint32_t m = 0; m < c; m++) {
        if (kind == 0) o[m] = id[list[fl_index(k, m, cap, lpp_log2)]];
        else o[m] = bid[list_ptr(list, k, cap)[m * 32u]];
    }
}

// Keeps the GPU busy for about `ns` nanoseconds without touching memory, so that
// the host can enqueue an event, a kernel and an event back to back behind it
// (per-kernel event timing without host-submission gaps).  Bounded: one sleep.
__global__ void k_delay(unsigned ns)
{
    if (threadIdx.x == 0) __nanosleep(ns);
}

}  // namespace

// ==========================================================================
// launchers: every particle kernel runs over all slots of all scenes; the neighbour
// passes with the context's lanes per particle (1 << P.lpp_log2)
// ==========================================================================
inline unsigned grid_lpp(uint32_t n, int lpp) { return (n + kBlock / lpp - 1) / (kBlock / lpp); }

#define LPP_DISPATCH(P, CALL)                                                                                      \
    do {                                                                                                           \
        switch ((P).lpp_log2) {                                                                                    \
        case 0: { constexpr int L = 1; CALL; } break;                                                              \
        case 1: { constexpr int L = 2; CALL; } break;                                                              \
        default: { constexpr int L = 4; CALL; } break;                                                             \
        }                                                                                                          \
    } while (0)

// dynamic shared memory of the staged solver passes (FP32, one lane per particle)
constexpr size_t kStageBytesPressure = kStageCap * sizeof(float4);
constexpr size_t kStageBytesJacobi = 3 * kStageCapJacobi * sizeof(float2);
template <class T> size_t stage_bytes(const DevParams<T> &P, int lpp, size_t bytes)
{
    return (sizeof(T) == 4 && lpp == 1 && P.staged) ? bytes : 0;
}

template <class T> void launch_keys(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np) k_keys<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B);
}
template <class T> void launch_gather(const DevParams<T> &P, const DevBufs<T> &B, const uint32_t *perm, cudaStream_t s)
{
    if (P.np) k_gather<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B, perm);
}
template <class T> void launch_cell_ranges(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np) k_cell_ranges<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B);
}
template <class T> void launch_vmap_boundary(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np && P.nvmaps) k_vmap_boundary<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B);
}
template <class T> void launch_stage_table(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np && P.staged) k_stage_table<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B);
}
template <class T> void launch_build(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np && P.staged) k_build<T, true><<<grid_for(P.np), kBlock, 0, s>>>(P, B);
    else if (P.np) k_build<T, false><<<grid_for(P.np), kBlock, 0, s>>>(P, B);
}
// The two solver passes with one lane per particle, unstaged, may run 128 or 512 threads per
// block (P.solver_nt, chosen by the autotuner; 512 for one scene only)
#define NT_DISPATCH(P, CALL)                                                                                       \
    do {                                                                                                           \
        if ((P).solver_nt == 128u) { constexpr int NT = 128; CALL; }                                               \
        else { constexpr int NT = 512; CALL; }                                                                     \
    } while (0)
template <class T> bool solver_nt_other(const DevParams<T> &P)
{
    return P.solver_nt != (uint32_t)kBlock && P.lpp_log2 == 0 && !P.staged &&
           (P.solver_nt == 128u || (P.solver_nt == 512u && P.nscenes == 1));
}

template <class T> void launch_pressure_accel(const DevParams<T> &P, const DevBufs<T> &B, bool div, int phase, cudaStream_t s,
                                              cudaGraphConditionalHandle h, bool use_handle)
{
    const unsigned limit = (div ? P.max_iter_v : P.max_iter) + 1;
    if (P.np && solver_nt_other(P)) {
        const int uh = use_handle ? 1 : 0;
        if (P.nphase > 1)
            NT_DISPATCH(P, (k_pressure_accel<T, 1, true, NT><<<(P.np + NT - 1) / NT, NT, 0, s>>>(P, B, limit, h, uh, phase)));
        else
            NT_DISPATCH(P, (k_pressure_accel<T, 1, false, NT><<<(P.np + NT - 1) / NT, NT, 0, s>>>(P, B, limit, h, uh, phase)));
    } else if (P.np)
    {
        if (P.nphase > 1)   // fluid phases: the rest-density ratio in the pressure term
            LPP_DISPATCH(P, (k_pressure_accel<T, L, true><<<grid_lpp(P.np, L), kBlock, 0, s>>>(
                                P, B, limit, h, use_handle ? 1 : 0, phase)));
        else
            LPP_DISPATCH(P, (k_pressure_accel<T, L><<<grid_lpp(P.np, L), kBlock, stage_bytes(P, L, kStageBytesPressure), s>>>(
                                P, B, limit, h, use_handle ? 1 : 0, phase)));
    }
}
template <class T>
void launch_jacobi(const DevParams<T> &P, const DevBufs<T> &B, bool div, int phase, cudaGraphConditionalHandle h,
                   bool use_handle, cudaStream_t s)
{
    if (!P.np) return;
    const int uh = use_handle ? 1 : 0;
    if (solver_nt_other(P)) {
        if (div) NT_DISPATCH(P, (k_jacobi<T, true, 1, NT><<<(P.np + NT - 1) / NT, NT, 0, s>>>(P, B, h, uh, phase)));
        else NT_DISPATCH(P, (k_jacobi<T, false, 1, NT><<<(P.np + NT - 1) / NT, NT, 0, s>>>(P, B, h, uh, phase)));
    } else if (div)
        LPP_DISPATCH(P, (k_jacobi<T, true, L><<<grid_lpp(P.np, L), kBlock, stage_bytes(P, L, kStageBytesJacobi), s>>>(
                            P, B, h, uh, phase)));
    else
        LPP_DISPATCH(P, (k_jacobi<T, false, L><<<grid_lpp(P.np, L), kBlock, stage_bytes(P, L, kStageBytesJacobi), s>>>(
                            P, B, h, uh, phase)));
}
template <class T> void launch_solver_finalize(const DevParams<T> &P, const DevBufs<T> &B, bool div, cudaStream_t s)
{
    if (!P.np) return;
    if (P.nphase > 1) {   // fluid phases: the rest-density ratio
        if (div) LPP_DISPATCH(P, (k_solver_finalize<T, true, L, true><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
        else LPP_DISPATCH(P, (k_solver_finalize<T, false, L, true><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
    } else {
        if (div) LPP_DISPATCH(P, (k_solver_finalize<T, true, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
        else LPP_DISPATCH(P, (k_solver_finalize<T, false, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
    }
}
template <class T> void launch_step_begin(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    k_step_begin<<<1, kBlock, 0, s>>>(B.sc, B.gsc, P.nscenes);
}
template <class T> void launch_loop_begin(const DevParams<T> &P, const DevBufs<T> &B, bool div, cudaStream_t s)
{
    k_loop_begin<<<1, kBlock, 0, s>>>(B.sc, B.gsc, P.nscenes, div ? 1 : 0, div ? P.max_iter_v : P.max_iter);
}
template <class T> void launch_xsph(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np) LPP_DISPATCH(P, (k_xsph<T, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, P.div_on)));
}
template <class T>
void launch_visc_setup(const DevParams<T> &P, const DevBufs<T> &B, cudaGraphConditionalHandle h, bool use_handle,
                       cudaStream_t s, int phase)
{
    if (!P.np) return;
    if (phase >= 0)
        LPP_DISPATCH(P, (k_visc_setup<T, L, true><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, h, use_handle ? 1 : 0, phase)));
    else
        LPP_DISPATCH(P, (k_visc_setup<T, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, h, use_handle ? 1 : 0, phase)));
}
template <class T>
void launch_xsph_visc_setup(const DevParams<T> &P, const DevBufs<T> &B, cudaGraphConditionalHandle h, bool use_handle,
                            cudaStream_t s)
{
    if (P.np)
        LPP_DISPATCH(P, (k_visc_setup<T, L, false, true><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, h, use_handle ? 1 : 0,
                                                                                             -1)));
}
template <class T> void launch_cg_matvec(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s,
                                         cudaGraphConditionalHandle h, bool use_handle, int phase)
{
    if (P.np)
        LPP_DISPATCH(P, (k_cg_matvec<T, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, h, use_handle ? 1 : 0, phase)));
}
template <class T>
void launch_cg_update(const DevParams<T> &P, const DevBufs<T> &B, cudaGraphConditionalHandle h, bool use_handle,
                      cudaStream_t s, int phase)
{
    if (P.np) k_cg_update<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B, h, use_handle ? 1 : 0, phase);
}
template <class T> void launch_cg_p(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s, int phase)
{
    if (P.np) k_cg_p<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B, phase);
}
template <class T> void launch_kick(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    k_kick<T><<<grid_for(P.np > 0 ? P.np : 1), kBlock, 0, s>>>(P, B);
}
template <class T> void launch_press_init(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np) LPP_DISPATCH(P, (k_press_init<T, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
}
template <class T> void launch_integrate(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    k_integrate<T><<<grid_for(P.np > 0 ? P.np : 1), kBlock, 0, s>>>(P, B);
}
template <class T> void launch_features(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (P.np) LPP_DISPATCH(P, (k_features<T, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
}
template <class T>
void launch_warmstart_select(const DevParams<T> &P, const DevBufs<T> &B, bool div, unsigned sweeps,
                             cudaGraphConditionalHandle h, bool use_handle, cudaStream_t s)
{
    if (!P.np || sweeps == 0) return;
    const unsigned g = grid_for(P.np);
    const int uh = use_handle ? 1 : 0;
    if (div) {
        k_ws_kappa<T, true><<<g, kBlock, 0, s>>>(P, B);
        for (unsigned k = 1; k <= sweeps; k++) {
            LPP_DISPATCH(P, (k_ws_accel2<T, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
            if (k < sweeps)
                LPP_DISPATCH(P, (k_ws_sweep<T, true, false, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, sweeps, h, uh)));
            else
                LPP_DISPATCH(P, (k_ws_sweep<T, true, true, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, sweeps, h, uh)));
        }
        k_ws_apply<T, true><<<g, kBlock, 0, s>>>(P, B);
    } else {
        k_ws_kappa<T, false><<<g, kBlock, 0, s>>>(P, B);
        for (unsigned k = 1; k <= sweeps; k++) {
            LPP_DISPATCH(P, (k_ws_accel2<T, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B)));
            if (k < sweeps)
                LPP_DISPATCH(P, (k_ws_sweep<T, false, false, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, sweeps, h, uh)));
            else
                LPP_DISPATCH(P, (k_ws_sweep<T, false, true, L><<<grid_lpp(P.np, L), kBlock, 0, s>>>(P, B, sweeps, h, uh)));
        }
        k_ws_apply<T, false><<<g, kBlock, 0, s>>>(P, B);
    }
}
template <class T>
void launch_body_forces(const DevParams<T> &P, const DevBufs<T> &B, const BodyDev &D, int phase, cudaStream_t s)
{
    if (!D.nblk) return;
    if (phase == 0) k_body_forces<T, 0><<<D.nblk, kBlock, 0, s>>>(P, B, D);
    else k_body_forces<T, 1><<<D.nblk, kBlock, 0, s>>>(P, B, D);
}
template <class T>
void launch_vmap_forces(const DevParams<T> &P, const DevBufs<T> &B, const BodyDev &D, int phase, cudaStream_t s)
{
    if (!P.np || !P.nvmaps || !D.nbodies || !D.vpartials) return;
    if (phase == 0) k_vmap_forces<T, 0><<<grid_for(P.np), kBlock, 0, s>>>(P, B, D);
    else k_vmap_forces<T, 1><<<grid_for(P.np), kBlock, 0, s>>>(P, B, D);
}
template <class T> void launch_boundary_keys(const DevParams<T> &P, const v4_t<T> *xb_in, const uint32_t *bscene_in,
                                             uint32_t *keys, uint32_t *vals, cudaStream_t s)
{
    if (P.nb) k_boundary_keys<T><<<grid_for(P.nb), kBlock, 0, s>>>(P, xb_in, bscene_in, keys, vals);
}
template <class T> void launch_boundary_gather(const DevParams<T> &P, const DevBufs<T> &B, const v4_t<T> *xb_in,
                                               const uint32_t *bscene_in, const uint32_t *perm, uint32_t *cells,
                                               cudaStream_t s)
{
    if (!P.nb) return;
    k_boundary_gather<T><<<grid_for(P.nb), kBlock, 0, s>>>(P, B, xb_in, bscene_in, perm, cells);
    k_cell_ranges_flat<<<grid_for(P.nb), kBlock, 0, s>>>(cells, B.bcstart, B.bcend, P.nb);
}
template <class T>
void launch_boundary_move(const DevParams<T> &P, const DevBufs<T> &B, const BoundaryMoveDev<T> &M, uint32_t *keys,
                          uint32_t *vals, cudaStream_t s)
{
    if (P.nb) k_boundary_move<T><<<grid_for(P.nb), kBlock, 0, s>>>(P, B, M, keys, vals);
}
template <class T>
void launch_boundary_regather(const DevParams<T> &P, const DevBufs<T> &B, const BoundaryMoveDev<T> &M,
                              const uint32_t *perm, uint32_t *cells, cudaStream_t s)
{
    if (!P.nb) return;
    k_boundary_regather<T><<<grid_for(P.nb), kBlock, 0, s>>>(P, B, M, perm, cells);
    k_cell_ranges_flat<<<grid_for(P.nb), kBlock, 0, s>>>(cells, B.bcstart, B.bcend, P.nb);
}
template <class T> void launch_boundary_volume(const DevParams<T> &P, const DevBufs<T> &B, cudaStream_t s)
{
    if (!P.nb) return;
    k_boundary_volume<T><<<grid_for(P.nb), kBlock, 0, s>>>(P, B);
    k_boundary_volume_store<T><<<grid_for(P.nb), kBlock, 0, s>>>(P, B);
}
template <class T> void launch_scatter_field(const DevParams<T> &P, const DevBufs<T> &B, int field, void *out,
                                             int odt, cudaStream_t s)
{
    if (field == SPHGB_FIELD_BOUNDARY_VOLUME || field == SPHGB_FIELD_BOUNDARY_POSITION) {
        if (P.nb) k_scatter_boundary<T><<<grid_for(P.nb), kBlock, 0, s>>>(P, B, field, out, odt);
    } else if (P.np) {
        k_scatter_field<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B, field, out, odt);
    }
}
template <class T> void launch_gather_fields(const DevParams<T> &P, const DevBufs<T> &B, const FieldSet &F, int odt,
                                             const uint32_t *inv, cudaStream_t s)
{
    if (P.nreal && F.n) k_gather_fields<T><<<grid_for(P.nreal), kBlock, 0, s>>>(P, B, F, odt, inv);
}
template <class T> void launch_upload_fields(const DevParams<T> &P, const DevBufs<T> &B, const FieldSet &F, int idt,
                                             const uint32_t *inv, cudaStream_t s)
{
    if (P.nreal && F.n) k_upload_fields<T><<<grid_for(P.nreal), kBlock, 0, s>>>(P, B, F, idt, inv);
}
template <class T> void launch_init_state(const DevParams<T> &P, const DevBufs<T> &B, const double *x, const double *v,
                                          const uint32_t *id, cudaStream_t s)
{
    if (P.np) k_init_state<T><<<grid_for(P.np), kBlock, 0, s>>>(P, B, x, v, id);
}
template <class T> void launch_inverse_perm(const DevParams<T> &P, const uint32_t *id, uint32_t *inv, cudaStream_t s)
{
    if (P.np) k_inverse_perm<T><<<grid_for(P.np), kBlock, 0, s>>>(P, id, inv);
}
void launch_delay(cudaStream_t s, unsigned ns) { k_delay<<<1, 32, 0, s>>>(ns); }
void launch_byteswap(void *data, size_t n, int bytes, cudaStream_t s)
{
    if (n) k_byteswap<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(data, n, bytes);
}

void launch_lists_to_ids(const uint32_t *list, const uint32_t *cnt, uint32_t cap, const uint32_t *id, const uint32_t *inv,
                         const uint32_t *bid, int kind, uint32_t lpp_log2, const uint32_t *offsets, uint32_t *out,
                         uint32_t n, cudaStream_t s)
{
    if (n) k_lists_to_ids<<<grid_for(n), kBlock, 0, s>>>(list, cnt, cap, id, inv, bid, kind, lpp_log2, offsets, out, n);
}

#define SPHGB_INSTANTIATE(T)                                                                                        \
    template void launch_keys<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                           \
    template void launch_gather<T>(const DevParams<T> &, const DevBufs<T> &, const uint32_t *, cudaStream_t);       \
    template void launch_cell_ranges<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                    \
    template void launch_build<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                          \
    template void launch_stage_table<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                    \
    template void launch_vmap_boundary<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                  \
    template void launch_pressure_accel<T>(const DevParams<T> &, const DevBufs<T> &, bool, int, cudaStream_t,       \
                                           cudaGraphConditionalHandle, bool);                                       \
    template void launch_jacobi<T>(const DevParams<T> &, const DevBufs<T> &, bool, int, cudaGraphConditionalHandle,  \
                                   bool, cudaStream_t);                                                             \
    template void launch_solver_finalize<T>(const DevParams<T> &, const DevBufs<T> &, bool, cudaStream_t);          \
    template void launch_loop_begin<T>(const DevParams<T> &, const DevBufs<T> &, bool, cudaStream_t);               \
    template void launch_step_begin<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                     \
    template void launch_features<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                       \
    template void launch_body_forces<T>(const DevParams<T> &, const DevBufs<T> &, const BodyDev &, int, cudaStream_t); \
    template void launch_vmap_forces<T>(const DevParams<T> &, const DevBufs<T> &, const BodyDev &, int, cudaStream_t); \
    template void launch_warmstart_select<T>(const DevParams<T> &, const DevBufs<T> &, bool, unsigned,              \
                                             cudaGraphConditionalHandle, bool, cudaStream_t);                       \
    template void launch_xsph<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                           \
    template void launch_visc_setup<T>(const DevParams<T> &, const DevBufs<T> &, cudaGraphConditionalHandle, bool,  \
                                       cudaStream_t, int);                                                          \
    template void launch_xsph_visc_setup<T>(const DevParams<T> &, const DevBufs<T> &, cudaGraphConditionalHandle,   \
                                            bool, cudaStream_t);                                                    \
    template void launch_cg_matvec<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t,                       \
                                      cudaGraphConditionalHandle, bool, int);                                       \
    template void launch_cg_update<T>(const DevParams<T> &, const DevBufs<T> &, cudaGraphConditionalHandle, bool,   \
                                      cudaStream_t, int);                                                           \
    template void launch_cg_p<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t, int);                      \
    template void launch_kick<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                           \
    template void launch_press_init<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                     \
    template void launch_integrate<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                      \
    template void launch_boundary_keys<T>(const DevParams<T> &, const v4_t<T> *, const uint32_t *, uint32_t *,      \
                                          uint32_t *, cudaStream_t);                                                \
    template void launch_boundary_gather<T>(const DevParams<T> &, const DevBufs<T> &, const v4_t<T> *,              \
                                            const uint32_t *, const uint32_t *, uint32_t *, cudaStream_t);          \
    template void launch_boundary_move<T>(const DevParams<T> &, const DevBufs<T> &, const BoundaryMoveDev<T> &,    \
                                          uint32_t *, uint32_t *, cudaStream_t);                                    \
    template void launch_boundary_regather<T>(const DevParams<T> &, const DevBufs<T> &, const BoundaryMoveDev<T> &, \
                                              const uint32_t *, uint32_t *, cudaStream_t);                          \
    template void launch_boundary_volume<T>(const DevParams<T> &, const DevBufs<T> &, cudaStream_t);                \
    template void launch_scatter_field<T>(const DevParams<T> &, const DevBufs<T> &, int, void *, int, cudaStream_t); \
    template void launch_gather_fields<T>(const DevParams<T> &, const DevBufs<T> &, const FieldSet &, int,          \
                                          const uint32_t *, cudaStream_t);                                          \
    template void launch_upload_fields<T>(const DevParams<T> &, const DevBufs<T> &, const FieldSet &, int,          \
                                          const uint32_t *, cudaStream_t);                                          \
    template void launch_init_state<T>(const DevParams<T> &, const DevBufs<T> &, const double *, const double *,    \
                                       const uint32_t *, cudaStream_t);                                             \
    template void launch_inverse_perm<T>(const DevParams<T> &, const uint32_t *, uint32_t *, cudaStream_t);

SPHGB_INSTANTIATE(float)
SPHGB_INSTANTIATE(double)

cudaError_t configure_staged_kernels()
{
    cudaError_t e = cudaFuncSetAttribute(k_jacobi<float, true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kStageBytesJacobi);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_jacobi<float, false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kStageBytesJacobi);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_pressure_accel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kStageBytesPressure);
    return e;
}

}  // namespace sphgb
