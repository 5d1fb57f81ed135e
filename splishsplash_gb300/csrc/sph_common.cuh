// Device-side building blocks shared by the sm_103a kernels: vector types, the
// cubic spline kernel, the neighbour predicate, deterministic FP64 reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sphgb {

constexpr int kBlock = 256;          // threads per block of every particle kernel
constexpr uint32_t kEmpty = 0xffffffffu;

// ---------------------------------------------------------------------------
// storage vector types: float4 for FP32, a 32-byte aligned double quad for FP64
// ---------------------------------------------------------------------------
struct alignas(32) dquad {
    double x, y, z, w;
};

template <class T> struct VecTraits;
template <> struct VecTraits<float> { using v4 = float4; };
template <> struct VecTraits<double> { using v4 = dquad; };
template <class T> using v4_t = typename VecTraits<T>::v4;

template <class T> struct V3 {
    T x, y, z;
};

template <class T> __device__ __forceinline__ V3<T> mk3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> __device__ __forceinline__ V3<T> add(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __device__ __forceinline__ V3<T> sub(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> __device__ __forceinline__ V3<T> scl(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ float4 ldv(const float4 *p, uint32_t i) { return p[i]; }
__device__ __forceinline__ dquad ldv(const dquad *p, uint32_t i)
{
    const double2 *q = reinterpret_cast<const double2 *>(p + i);
    double2 a = q[0], b = q[1];
    return dquad{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void stv(float4 *p, uint32_t i, float4 v) { p[i] = v; }
__device__ __forceinline__ void stv(dquad *p, uint32_t i, dquad v)
{
    double2 *q = reinterpret_cast<double2 *>(p + i);
    q[0] = make_double2(v.x, v.y);
    q[1] = make_double2(v.z, v.w);
}

// store only the w lane of element i
__device__ __forceinline__ void store_w(float4 *p, uint32_t i, float w) { reinterpret_cast<float *>(p + i)[3] = w; }
__device__ __forceinline__ void store_w(dquad *p, uint32_t i, double w) { p[i].w = w; }

template <class T> __device__ __forceinline__ V3<T> xyz(const v4_t<T> &v) { return V3<T>{(T)v.x, (T)v.y, (T)v.z}; }
template <class T> __device__ __forceinline__ v4_t<T> pack(V3<T> a, T w)
{
    v4_t<T> r;
    r.x = a.x; r.y = a.y; r.z = a.z; r.w = w;
    return r;
}

// ---------------------------------------------------------------------------
// neighbour predicate: |xi - xj|^2 < h^2 with separate round-to-nearest
// multiplies and adds, in the order ((dx*dx + dy*dy) + dz*dz).  The CPU oracle
// evaluates the identical expression, so neighbour sets are bit-exact.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pair_d2(const float4 &a, const float4 &b, float &dx, float &dy, float &dz)
{
    dx = __fsub_rn(a.x, b.x);
    dy = __fsub_rn(a.y, b.y);
    dz = __fsub_rn(a.z, b.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}
__device__ __forceinline__ double pair_d2(const dquad &a, const dquad &b, double &dx, double &dy, double &dz)
{
    dx = __dsub_rn(a.x, b.x);
    dy = __dsub_rn(a.y, b.y);
    dz = __dsub_rn(a.z, b.z);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// ---------------------------------------------------------------------------
// Cubic spline kernel (the analytic kernel of SPHKernels.h:16-91, evaluated in T)
// ---------------------------------------------------------------------------
template <class T> struct Kernel {
    T h;      // support radius
    T invh;   // 1/h
    T invh2;  // 1/h^2
    T k;      // 8 / (pi h^3)
    T l;      // 48 / (pi h^3)
    T w0;     // W(0)
    T h2;     // predicate bound: float(h*h) computed on the host in FP64
};

template <class T> __device__ __forceinline__ T kernel_W(const Kernel<T> &K, T rl)
{
    const T q = rl * K.invh;
    T res = T(0);
    if (q <= T(1)) {
        if (q <= T(0.5)) {
            const T q2 = q * q;
            res = K.k * (T(6) * q2 * q - T(6) * q2 + T(1));
        } else {
            const T t = T(1) - q;
            res = K.k * (T(2) * t * t * t);
        }
    }
    return res;
}

// scalar c such that gradW(r) = c * r
template <class T> __device__ __forceinline__ T kernel_gradW_coef(const Kernel<T> &K, T rl)
{
    const T q = rl * K.invh;
    T c = T(0);
    if (rl > T(1.0e-9) && q <= T(1)) {
        if (q <= T(0.5)) {
            c = K.l * K.invh2 * (T(3) * q - T(2));
        } else {
            const T f = T(1) - q;
            c = -K.l * f * f / (rl * K.h);
        }
    }
    return c;
}

__device__ __forceinline__ float dev_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dev_sqrt(double x) { return sqrt(x); }

// ---------------------------------------------------------------------------
// deterministic reductions: block partial sums in FP64, then the last block to
// finish sums the partials in a fixed order and runs a finalizer.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int NV> struct DSum {
    double v[NV];
};

// Sum NV doubles over the block; result valid in thread 0.
template <int NV> __device__ __forceinline__ DSum<NV> block_sum(DSum<NV> s)
{
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double v = warp_sum(s.v[k]);
        if (lane == 0) sh[k][warp] = v;
    }
    __syncthreads();
    DSum<NV> r;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double v = (warp == 0 && lane < nw) ? sh[k][lane] : 0.0;
        if (warp == 0) v = warp_sum(v);
        r.v[k] = v;
    }
    __syncthreads();
    return r;
}

// Reduction slot of one scene for the last-block pattern.  A scene owns the
// consecutive blocks [first, first + count) of the launch.
struct ReduceSlot {
    double *partials;    // NV x gridDim.x, indexed by block
    unsigned *counter;   // the scene's arrival counter: zero before the launch, reset by its last block
    unsigned first, count;
};

// Every block of the scene calls this once with its per-thread contributions
// (all threads of the block, no early return before it).  The scene's last block
// to arrive sums the scene's block partials in block order (deterministic) and
// calls fin(total) from its thread 0.
template <int NV, class Fin>
__device__ __forceinline__ void grid_sum_finalize(DSum<NV> mine, ReduceSlot slot, Fin fin)
{
    DSum<NV> b = block_sum<NV>(mine);
    __shared__ bool amLast;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) slot.partials[(size_t)k * gridDim.x + blockIdx.x] = b.v[k];
        __threadfence();
        const unsigned t = atomicAdd(slot.counter, 1u);
        amLast = (t == slot.count - 1);
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    DSum<NV> acc;
#pragma unroll
    for (int k = 0; k < NV; k++) acc.v[k] = 0.0;
    // U partials per thread in flight at a time, added in the same order as one by one (thread t
    // sums t, t + blockDim, t + 2 blockDim, ...), so the total does not depend on U
    constexpr unsigned U = NV <= 2 ? 8u : 4u;
    const double *src = slot.partials + slot.first;
    unsigned i = threadIdx.x;
    for (; i + (U - 1u) * blockDim.x < slot.count; i += U * blockDim.x) {
        double p[U][NV];
#pragma unroll
        for (unsigned u = 0; u < U; u++)
#pragma unroll
            for (int k = 0; k < NV; k++) p[u][k] = __ldcg(src + (size_t)k * gridDim.x + i + u * blockDim.x);
#pragma unroll
        for (unsigned u = 0; u < U; u++)
#pragma unroll
            for (int k = 0; k < NV; k++) acc.v[k] += p[u][k];
    }
    for (; i < slot.count; i += blockDim.x) {
#pragma unroll
        for (int k = 0; k < NV; k++) acc.v[k] += __ldcg(src + (size_t)k * gridDim.x + i);
    }
    DSum<NV> tot = block_sum<NV>(acc);
    if (threadIdx.x == 0) {
        *slot.counter = 0;
        fin(tot);
    }
}

// ---------------------------------------------------------------------------
// Morton code of 10-bit cell coordinates
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t spread10(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z)
{
    return spread10(x) | (spread10(y) << 1) | (spread10(z) << 2);
}

}  // namespace sphgb
