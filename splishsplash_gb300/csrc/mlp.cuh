// Warm-start network shared by the MLP library (mlp.cu) and the solver kernels:
// 10 inputs -> 64 (GELU) -> 64 (GELU) -> 2 outputs, BF16 weights and activations on
// the tensor cores (mma.sync m16n8k16, FP32 accumulation).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace sphgb {

constexpr int kMlpIn = 10;     // features
constexpr int kMlpInPad = 16;  // one k-step of the MMA
constexpr int kMlpH = 64;
constexpr int kMlpOut = 2;
constexpr int kMlpOutPad = 8;  // one n-tile

// FP32 master parameter layout (row-major, out x in):
//   W1[64][16] b1[64] W2[64][64] b2[64] W3[8][64] b3[8]
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpH * kMlpInPad;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpOutPad * kMlpH;
constexpr int kMlpParams = kOffB3 + kMlpOutPad;   // 5768

// Default output scales: network output x scale = the multiplier that the predicted warm
// start applies to the previous step's stored kappa_v (divergence) and kappa (pressure), in
// place of the classic factor 0.5.
constexpr float kMlpDefaultScaleV = 1.0f;
constexpr float kMlpDefaultScaleP = 1.0f;

// Device copy used by kernels: BF16 weights and FP32 biases, plus feature/output scales.
struct MlpDev {
    const __nv_bfloat16 *w;   // kMlpParams bf16 (biases unused in this copy)
    const float *p;           // kMlpParams fp32 (biases read from here)
    float out_scale[2];       // network output * scale = warm-start multiplier (divergence, pressure)
};

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x)
{
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
    return cdf + x * pdf;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);   // .x = lo (low 16 bits)
    return *reinterpret_cast<uint32_t *>(&v);
}

// D = A(16x16 bf16, row) * B(16x8 bf16, col) + C, FP32 accumulate
__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// B fragment for an n-tile of W (row-major [out][in]) at k-offset k0: B[k][n] = W[n0+n][k0+k].
// Lane (g = lane/4, t = lane%4) holds B[2t,2t+1][g] and B[2t+8,2t+9][g].
__device__ __forceinline__ void load_b(const __nv_bfloat16 *W, int ld, int n0, int k0, int lane, uint32_t b[2])
{
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16 *row = W + (size_t)(n0 + g) * ld + k0;
    b[0] = *reinterpret_cast<const uint32_t *>(row + 2 * t);
    b[1] = *reinterpret_cast<const uint32_t *>(row + 2 * t + 8);
}

// Forward pass of 16 samples held by one warp.  xin: this lane's A fragment of the padded
// 16x16 input tile.  Writes pre-activations (optional) and the 2 outputs of rows g and g+8
// (only lanes with t == 0 hold output columns 0 and 1).
// w: BF16 weights in shared or global memory, p: FP32 parameters (biases).
struct MlpFwdOut {
    float y[4];   // C fragment of the output tile: rows g/g+8, cols 2t/2t+1
};

template <bool STORE_Z>
__device__ __forceinline__ MlpFwdOut mlp_forward_warp(const __nv_bfloat16 *w, const float *p, const uint32_t xin[4],
                                                      int lane, float *z1 = nullptr, float *z2 = nullptr, int ldz = 0,
                                                      int valid = 16)
{
    const int g = lane >> 2, t = lane & 3;
    const bool r0 = g < valid, r1 = g + 8 < valid;   // rows of this lane that exist
    // layer 1: 16x16 * 16x64
    float h1[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const float b0 = p[kOffB1 + nt * 8 + 2 * t], b1 = p[kOffB1 + nt * 8 + 2 * t + 1];
        h1[nt][0] = b0; h1[nt][1] = b1; h1[nt][2] = b0; h1[nt][3] = b1;
        uint32_t b[2];
        load_b(w + kOffW1, kMlpInPad, nt * 8, 0, lane, b);
        mma_bf16_16816(h1[nt], xin, b);
        if (STORE_Z) {
            if (r0) { z1[(size_t)g * ldz + nt * 8 + 2 * t] = h1[nt][0]; z1[(size_t)g * ldz + nt * 8 + 2 * t + 1] = h1[nt][1]; }
            if (r1) {
                z1[(size_t)(g + 8) * ldz + nt * 8 + 2 * t] = h1[nt][2];
                z1[(size_t)(g + 8) * ldz + nt * 8 + 2 * t + 1] = h1[nt][3];
            }
        }
#pragma unroll
        for (int r = 0; r < 4; r++) h1[nt][r] = gelu(h1[nt][r]);
    }
    // C fragments of n-tiles 2kk and 2kk+1 form the A fragment of k-step kk
    uint32_t a2[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        a2[kk][0] = pack_bf16(h1[2 * kk][0], h1[2 * kk][1]);
        a2[kk][1] = pack_bf16(h1[2 * kk][2], h1[2 * kk][3]);
        a2[kk][2] = pack_bf16(h1[2 * kk + 1][0], h1[2 * kk + 1][1]);
        a2[kk][3] = pack_bf16(h1[2 * kk + 1][2], h1[2 * kk + 1][3]);
    }
    // layer 2: 16x64 * 64x64
    float h2[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const float b0 = p[kOffB2 + nt * 8 + 2 * t], b1 = p[kOffB2 + nt * 8 + 2 * t + 1];
        h2[nt][0] = b0; h2[nt][1] = b1; h2[nt][2] = b0; h2[nt][3] = b1;
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            uint32_t b[2];
            load_b(w + kOffW2, kMlpH, nt * 8, kk * 16, lane, b);
            mma_bf16_16816(h2[nt], a2[kk], b);
        }
        if (STORE_Z) {
            if (r0) { z2[(size_t)g * ldz + nt * 8 + 2 * t] = h2[nt][0]; z2[(size_t)g * ldz + nt * 8 + 2 * t + 1] = h2[nt][1]; }
            if (r1) {
                z2[(size_t)(g + 8) * ldz + nt * 8 + 2 * t] = h2[nt][2];
                z2[(size_t)(g + 8) * ldz + nt * 8 + 2 * t + 1] = h2[nt][3];
            }
        }
#pragma unroll
        for (int r = 0; r < 4; r++) h2[nt][r] = gelu(h2[nt][r]);
    }
    uint32_t a3[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        a3[kk][0] = pack_bf16(h2[2 * kk][0], h2[2 * kk][1]);
        a3[kk][1] = pack_bf16(h2[2 * kk][2], h2[2 * kk][3]);
        a3[kk][2] = pack_bf16(h2[2 * kk + 1][0], h2[2 * kk + 1][1]);
        a3[kk][3] = pack_bf16(h2[2 * kk + 1][2], h2[2 * kk + 1][3]);
    }
    // layer 3: 16x64 * 64x8 (2 used)
    MlpFwdOut o;
    const float c0 = p[kOffB3 + 2 * t], c1 = p[kOffB3 + 2 * t + 1];
    o.y[0] = c0; o.y[1] = c1; o.y[2] = c0; o.y[3] = c1;
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        uint32_t b[2];
        load_b(w + kOffW3, kMlpH, 0, kk * 16, lane, b);
        mma_bf16_16816(o.y, a3[kk], b);
    }
    return o;
}

// A fragment of a 16x16 input tile from row-major FP32 rows (ld floats, kMlpIn used).
// Lane (g, t) holds rows g, g+8 at columns 2t, 2t+1, 2t+8, 2t+9.
__device__ __forceinline__ void load_a_input(const float *rows, int ld, int nrows_valid, int lane, uint32_t a[4])
{
    const int g = lane >> 2, t = lane & 3;
    auto val = [&](int r, int c) -> float { return (r < nrows_valid && c < kMlpIn) ? rows[(size_t)r * ld + c] : 0.0f; };
    a[0] = pack_bf16(val(g, 2 * t), val(g, 2 * t + 1));
    a[1] = pack_bf16(val(g + 8, 2 * t), val(g + 8, 2 * t + 1));
    a[2] = pack_bf16(val(g, 2 * t + 8), val(g, 2 * t + 9));
    a[3] = pack_bf16(val(g + 8, 2 * t + 8), val(g + 8, 2 * t + 9));
}

}  // namespace sphgb
