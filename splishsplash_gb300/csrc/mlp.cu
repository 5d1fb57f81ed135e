// Warm-start network: hand-written training and inference kernels.
//
//   forward   : mma.sync m16n8k16 BF16 tensor-core tiles, FP32 accumulation (mlp.cuh)
//   backward  : FP32 on the CUDA cores against the BF16-rounded weights and
//               activations the forward pass used; per-block sums of the weight
//               gradients, one atomic add per weight and block
//   optimiser : Adam (FP32 master weights, BF16 copy refreshed after every step)
//
// Loss: mean over samples of sum_o mask_o (y_o - t_o)^2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/sphgb300.h"
#include "mlp.cuh"
#include "sph_ctx.h"

using namespace sphgb;

struct sphgb_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wbf = nullptr;
    float out_scale[2] = {kMlpDefaultScaleV, kMlpDefaultScaleP};
    uint64_t adam_step = 0;
    // training buffers
    uint32_t cap = 0;
    float *X = nullptr, *Y = nullptr, *M = nullptr;      // full data set on the device
    float *bx = nullptr, *by = nullptr, *bm = nullptr;   // minibatch
    float *z1 = nullptr, *z2 = nullptr, *yp = nullptr;
    uint32_t *perm = nullptr;
    float *loss = nullptr;
    uint32_t bcap = 0;
    std::string err;
};

namespace {

constexpr int kFwdThreads = 128;   // 4 warps x 16 samples
constexpr int kBwdThreads = 64;    // one sample per thread

__global__ void k_to_bf16(const float *__restrict__ p, __nv_bfloat16 *__restrict__ w, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = __float2bfloat16_rn(p[i]);
}

// Y[N][2] = net(X[N][kMlpIn]); optional pre-activations Z1, Z2 [N][64]
template <bool STORE_Z>
__global__ void __launch_bounds__(kFwdThreads) k_mlp_forward(const float *__restrict__ X, uint32_t n,
                                                              const __nv_bfloat16 *__restrict__ w,
                                                              const float *__restrict__ p, float *__restrict__ Y,
                                                              float *__restrict__ Z1, float *__restrict__ Z2)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t row0 = (blockIdx.x * (kFwdThreads / 32) + warp) * 16u;
    if (row0 >= n) return;
    const int valid = (int)min(16u, n - row0);
    uint32_t a[4];
    load_a_input(X + (size_t)row0 * kMlpIn, kMlpIn, valid, lane, a);
    MlpFwdOut o = mlp_forward_warp<STORE_Z>(w, p, a, lane, STORE_Z ? Z1 + (size_t)row0 * kMlpH : nullptr,
                                            STORE_Z ? Z2 + (size_t)row0 * kMlpH : nullptr, kMlpH, valid);
    const int g = lane >> 2, t = lane & 3;
    if (t == 0) {
        if (g < valid) { Y[(size_t)(row0 + g) * 2] = o.y[0]; Y[(size_t)(row0 + g) * 2 + 1] = o.y[1]; }
        if (g + 8 < valid) { Y[(size_t)(row0 + g + 8) * 2] = o.y[2]; Y[(size_t)(row0 + g + 8) * 2 + 1] = o.y[3]; }
    }
}

__device__ __forceinline__ float bfr(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Backward for 64 samples per block.  Gradients are accumulated into grad (FP32) and the
// sum of squared errors into loss[0].  inv_n scales the mean over the whole batch.
__global__ void __launch_bounds__(kBwdThreads) k_mlp_backward(const float *__restrict__ X, const float *__restrict__ Z1,
                                                               const float *__restrict__ Z2, const float *__restrict__ Yp,
                                                               const float *__restrict__ Yt, const float *__restrict__ Mk,
                                                               uint32_t n, float inv_n, const __nv_bfloat16 *__restrict__ w,
                                                               float *__restrict__ grad, float *__restrict__ loss)
{
    extern __shared__ float sm[];
    float *sX = sm;                                 // [64][16]
    float *sH1 = sX + kBwdThreads * kMlpInPad;      // [64][64]
    float *sH2 = sH1 + kBwdThreads * kMlpH;         // [64][64]
    float *sD1 = sH2 + kBwdThreads * kMlpH;         // [64][64]
    float *sD2 = sD1 + kBwdThreads * kMlpH;         // [64][64]
    float *sDY = sD2 + kBwdThreads * kMlpH;         // [64][2]
    const int t = threadIdx.x;
    const uint32_t s = blockIdx.x * kBwdThreads + t;
    const bool valid = s < n;
    float se = 0.0f;
    // per-sample part
    {
        float dy[2] = {0.0f, 0.0f};
        for (int i = 0; i < kMlpInPad; i++) sX[t * kMlpInPad + i] = (valid && i < kMlpIn) ? bfr(X[(size_t)s * kMlpIn + i]) : 0.0f;
        if (valid) {
            for (int o = 0; o < 2; o++) {
                const float mk = Mk ? Mk[(size_t)s * 2 + o] : 1.0f;
                const float d = Yp[(size_t)s * 2 + o] - Yt[(size_t)s * 2 + o];
                se += mk * d * d;
                dy[o] = 2.0f * mk * d * inv_n;
            }
        }
        sDY[t * 2] = dy[0];
        sDY[t * 2 + 1] = dy[1];
        float dz2[kMlpH];
        for (int k = 0; k < kMlpH; k++) {
            const float z = valid ? Z2[(size_t)s * kMlpH + k] : 0.0f;
            sH2[t * kMlpH + k] = valid ? bfr(gelu(z)) : 0.0f;
            const float dh = __bfloat162float(w[kOffW3 + k]) * dy[0] + __bfloat162float(w[kOffW3 + kMlpH + k]) * dy[1];
            dz2[k] = valid ? dh * gelu_grad(z) : 0.0f;
            sD2[t * kMlpH + k] = dz2[k];
        }
        for (int j = 0; j < kMlpH; j++) {
            const float z = valid ? Z1[(size_t)s * kMlpH + j] : 0.0f;
            sH1[t * kMlpH + j] = valid ? bfr(gelu(z)) : 0.0f;
            float dh = 0.0f;
            for (int k = 0; k < kMlpH; k++) dh += __bfloat162float(w[kOffW2 + k * kMlpH + j]) * dz2[k];
            sD1[t * kMlpH + j] = valid ? dh * gelu_grad(z) : 0.0f;
        }
    }
    __syncthreads();
    // block sums of the weight gradients: thread t owns row t of W1, W2 and column t of W3
    {
        float acc[kMlpH];
        for (int j = 0; j < kMlpH; j++) acc[j] = 0.0f;
        float db2 = 0.0f;
        for (int q = 0; q < kBwdThreads; q++) {
            const float d = sD2[q * kMlpH + t];
            db2 += d;
            for (int j = 0; j < kMlpH; j++) acc[j] += d * sH1[q * kMlpH + j];
        }
        for (int j = 0; j < kMlpH; j++) atomicAdd(&grad[kOffW2 + t * kMlpH + j], acc[j]);
        atomicAdd(&grad[kOffB2 + t], db2);
    }
    {
        float acc[kMlpIn];
        for (int i = 0; i < kMlpIn; i++) acc[i] = 0.0f;
        float db1 = 0.0f;
        for (int q = 0; q < kBwdThreads; q++) {
            const float d = sD1[q * kMlpH + t];
            db1 += d;
            for (int i = 0; i < kMlpIn; i++) acc[i] += d * sX[q * kMlpInPad + i];
        }
        for (int i = 0; i < kMlpIn; i++) atomicAdd(&grad[kOffW1 + t * kMlpInPad + i], acc[i]);
        atomicAdd(&grad[kOffB1 + t], db1);
    }
    {
        float a0 = 0.0f, a1 = 0.0f;
        for (int q = 0; q < kBwdThreads; q++) {
            const float h = sH2[q * kMlpH + t];
            a0 += sDY[q * 2] * h;
            a1 += sDY[q * 2 + 1] * h;
        }
        atomicAdd(&grad[kOffW3 + t], a0);
        atomicAdd(&grad[kOffW3 + kMlpH + t], a1);
        if (t < 2) {
            float db = 0.0f;
            for (int q = 0; q < kBwdThreads; q++) db += sDY[q * 2 + t];
            atomicAdd(&grad[kOffB3 + t], db);
        }
    }
    // squared error
    for (int o = 16; o > 0; o >>= 1) se += __shfl_down_sync(0xffffffffu, se, o);
    if ((t & 31) == 0) atomicAdd(loss, se);
}

__global__ void k_adam(float *__restrict__ p, float *__restrict__ g, float *__restrict__ m, float *__restrict__ v, int n,
                       float lr, float b1, float b2, float eps, float bc1, float bc2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // padded weight entries stay zero
    const bool pad = (i >= kOffW1 && i < kOffB1 && (i - kOffW1) % kMlpInPad >= kMlpIn) ||
                     (i >= kOffW3 && i < kOffB3 && (i - kOffW3) / kMlpH >= kMlpOut) || (i >= kOffB3 + kMlpOut);
    const float gi = pad ? 0.0f : g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    if (!pad) p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    g[i] = 0.0f;
}

__global__ void k_gather_rows(const float *__restrict__ src, const uint32_t *__restrict__ idx, float *__restrict__ dst,
                              uint32_t rows, int width)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= rows * (uint32_t)width) return;
    const uint32_t r = e / width, c = e % width;
    dst[e] = src[(size_t)idx[r] * width + c];
}

int merr(sphgb_mlp *m, const std::string &s)
{
    if (m) m->err = s;
    return SPHGB_ERR_CUDA;
}

#define MCK(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return merr(m, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t bwd_smem() { return sizeof(float) * (kBwdThreads * kMlpInPad + 4 * kBwdThreads * kMlpH + kBwdThreads * 2); }

int ensure_batch(sphgb_mlp *m, uint32_t b)
{
    if (m->bcap >= b) return SPHGB_OK;
    cudaFree(m->bx); cudaFree(m->by); cudaFree(m->bm); cudaFree(m->z1); cudaFree(m->z2); cudaFree(m->yp);
    MCK(cudaMalloc(&m->bx, (size_t)b * kMlpIn * 4));
    MCK(cudaMalloc(&m->by, (size_t)b * 2 * 4));
    MCK(cudaMalloc(&m->bm, (size_t)b * 2 * 4));
    MCK(cudaMalloc(&m->z1, (size_t)b * kMlpH * 4));
    MCK(cudaMalloc(&m->z2, (size_t)b * kMlpH * 4));
    MCK(cudaMalloc(&m->yp, (size_t)b * 2 * 4));
    m->bcap = b;
    return SPHGB_OK;
}

// forward + backward on device arrays (rows already gathered); accumulates grad and loss
int fwd_bwd(sphgb_mlp *m, const float *X, const float *Y, const float *Mk, uint32_t n, float inv_n)
{
    const unsigned fb = (n + 63) / 64;
    k_mlp_forward<true><<<fb, kFwdThreads, 0, m->stream>>>(X, n, m->wbf, m->params, m->yp, m->z1, m->z2);
    const unsigned bb = (n + kBwdThreads - 1) / kBwdThreads;
    k_mlp_backward<<<bb, kBwdThreads, bwd_smem(), m->stream>>>(X, m->z1, m->z2, m->yp, Y, Mk, n, inv_n, m->wbf,
                                                                m->grad, m->loss);
    MCK(cudaGetLastError());
    return SPHGB_OK;
}

int refresh_bf16(sphgb_mlp *m)
{
    k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, m->stream>>>(m->params, m->wbf, kMlpParams);
    MCK(cudaGetLastError());
    return SPHGB_OK;
}

}  // namespace

namespace sphgb {
// used by the solver: inference on device rows
void mlp_infer_device(const float *X, uint32_t n, const void *w, const float *p, float *Y, cudaStream_t s)
{
    if (n)
        k_mlp_forward<false><<<(n + 63) / 64, kFwdThreads, 0, s>>>(X, n, static_cast<const __nv_bfloat16 *>(w), p, Y,
                                                                   nullptr, nullptr);
}
// device buffers of a network, for copying into a solver context
void mlp_export(const sphgb_mlp *m, const float **params, const void **w, float scale[2], int *device)
{
    *params = m->params;
    *w = m->wbf;
    scale[0] = m->out_scale[0];
    scale[1] = m->out_scale[1];
    *device = m->device;
}
}  // namespace sphgb

extern "C" {

int sphgb_mlp_create(int device, uint32_t seed, sphgb_mlp **out)
{
    if (!out) return SPHGB_ERR_ARGUMENT;
    sphgb_mlp *m = new sphgb_mlp();
    m->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&m->params, kMlpParams * 4) != cudaSuccess || cudaMalloc(&m->grad, kMlpParams * 4) != cudaSuccess ||
        cudaMalloc(&m->m, kMlpParams * 4) != cudaSuccess || cudaMalloc(&m->v, kMlpParams * 4) != cudaSuccess ||
        cudaMalloc(&m->wbf, kMlpParams * 2) != cudaSuccess || cudaMalloc(&m->loss, 16) != cudaSuccess ||
        cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem()) != cudaSuccess) {
        cudaGetLastError();
        delete m;
        return SPHGB_ERR_CUDA;
    }
    // He-uniform initialisation of the used weights, zero biases and padding
    std::vector<float> p(kMlpParams, 0.0f);
    std::mt19937 rng(seed);
    auto fill = [&](int off, int rows, int cols, int used_rows, int used_cols, int fan_in) {
        std::uniform_real_distribution<float> U(-std::sqrt(6.0f / fan_in), std::sqrt(6.0f / fan_in));
        for (int r = 0; r < rows; r++)
            for (int c = 0; c < cols; c++) p[off + r * cols + c] = (r < used_rows && c < used_cols) ? U(rng) : 0.0f;
    };
    fill(kOffW1, kMlpH, kMlpInPad, kMlpH, kMlpIn, kMlpIn);
    fill(kOffW2, kMlpH, kMlpH, kMlpH, kMlpH, kMlpH);
    fill(kOffW3, kMlpOutPad, kMlpH, kMlpOut, kMlpH, kMlpH);
    if (cudaMemcpy(m->params, p.data(), kMlpParams * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->grad, 0, kMlpParams * 4) != cudaSuccess || cudaMemset(m->m, 0, kMlpParams * 4) != cudaSuccess ||
        cudaMemset(m->v, 0, kMlpParams * 4) != cudaSuccess || refresh_bf16(m) != SPHGB_OK ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) {
        delete m;
        return SPHGB_ERR_CUDA;
    }
    *out = m;
    return SPHGB_OK;
}

int sphgb_mlp_destroy(sphgb_mlp *m)
{
    if (!m) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(m->device);
    cudaStreamSynchronize(m->stream);
    for (void *q : {(void *)m->params, (void *)m->grad, (void *)m->m, (void *)m->v, (void *)m->wbf, (void *)m->loss,
                    (void *)m->X, (void *)m->Y, (void *)m->M, (void *)m->bx, (void *)m->by, (void *)m->bm, (void *)m->z1,
                    (void *)m->z2, (void *)m->yp, (void *)m->perm})
        if (q) cudaFree(q);
    cudaStreamDestroy(m->stream);
    delete m;
    return SPHGB_OK;
}

const char *sphgb_mlp_last_error(const sphgb_mlp *m) { return m ? m->err.c_str() : "null network"; }

int sphgb_mlp_num_params(void) { return kMlpParams; }

int sphgb_mlp_get_params(sphgb_mlp *m, float *out)
{
    if (!m || !out) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(m->device);
    MCK(cudaMemcpyAsync(out, m->params, kMlpParams * 4, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return SPHGB_OK;
}

int sphgb_mlp_set_params(sphgb_mlp *m, const float *in)
{
    if (!m || !in) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(m->device);
    MCK(cudaMemcpyAsync(m->params, in, kMlpParams * 4, cudaMemcpyHostToDevice, m->stream));
    int rc = refresh_bf16(m);
    if (rc) return rc;
    MCK(cudaStreamSynchronize(m->stream));
    return SPHGB_OK;
}

int sphgb_mlp_set_output_scale(sphgb_mlp *m, float scale_v, float scale_p)
{
    if (!m || !(scale_v > 0) || !(scale_p > 0)) return SPHGB_ERR_ARGUMENT;
    m->out_scale[0] = scale_v;
    m->out_scale[1] = scale_p;
    return SPHGB_OK;
}

int sphgb_mlp_get_output_scale(const sphgb_mlp *m, float *scale_v, float *scale_p)
{
    if (!m) return SPHGB_ERR_ARGUMENT;
    if (scale_v) *scale_v = m->out_scale[0];
    if (scale_p) *scale_p = m->out_scale[1];
    return SPHGB_OK;
}

int sphgb_mlp_forward(sphgb_mlp *m, const float *X, uint32_t n, float *Y)
{
    if (!m || (n && (!X || !Y))) return SPHGB_ERR_ARGUMENT;
    if (n == 0) return SPHGB_OK;
    cudaSetDevice(m->device);
    int rc = ensure_batch(m, n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(m->bx, X, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice, m->stream));
    k_mlp_forward<false><<<(n + 63) / 64, kFwdThreads, 0, m->stream>>>(m->bx, n, m->wbf, m->params, m->yp, nullptr, nullptr);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(Y, m->yp, (size_t)n * 2 * 4, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return SPHGB_OK;
}

int sphgb_mlp_loss_grad(sphgb_mlp *m, const float *X, const float *Y, const float *mask, uint32_t n, float *loss,
                        float *grad)
{
    if (!m || !X || !Y || n == 0) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(m->device);
    int rc = ensure_batch(m, n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(m->bx, X, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemcpyAsync(m->by, Y, (size_t)n * 2 * 4, cudaMemcpyHostToDevice, m->stream));
    if (mask) MCK(cudaMemcpyAsync(m->bm, mask, (size_t)n * 2 * 4, cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemsetAsync(m->grad, 0, kMlpParams * 4, m->stream));
    MCK(cudaMemsetAsync(m->loss, 0, 4, m->stream));
    if ((rc = fwd_bwd(m, m->bx, m->by, mask ? m->bm : nullptr, n, 1.0f / n))) return rc;
    if (grad) MCK(cudaMemcpyAsync(grad, m->grad, kMlpParams * 4, cudaMemcpyDeviceToHost, m->stream));
    float l = 0.f;
    MCK(cudaMemcpyAsync(&l, m->loss, 4, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaMemsetAsync(m->grad, 0, kMlpParams * 4, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (loss) *loss = l / n;
    return SPHGB_OK;
}

int sphgb_mlp_train(sphgb_mlp *m, const float *X, const float *Y, const float *mask, uint32_t n, uint32_t epochs,
                    uint32_t batch, float lr, uint32_t seed, float *epoch_loss)
{
    if (!m || !X || !Y || n == 0 || batch == 0 || !(lr > 0)) return SPHGB_ERR_ARGUMENT;
    cudaSetDevice(m->device);
    if (m->cap < n) {
        cudaFree(m->X); cudaFree(m->Y); cudaFree(m->M); cudaFree(m->perm);
        m->X = m->Y = m->M = nullptr;
        m->perm = nullptr;
        MCK(cudaMalloc(&m->X, (size_t)n * kMlpIn * 4));
        MCK(cudaMalloc(&m->Y, (size_t)n * 2 * 4));
        MCK(cudaMalloc(&m->M, (size_t)n * 2 * 4));
        MCK(cudaMalloc(&m->perm, (size_t)n * 4));
        m->cap = n;
    }
    int rc = ensure_batch(m, batch);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(m->X, X, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemcpyAsync(m->Y, Y, (size_t)n * 2 * 4, cudaMemcpyHostToDevice, m->stream));
    if (mask) MCK(cudaMemcpyAsync(m->M, mask, (size_t)n * 2 * 4, cudaMemcpyHostToDevice, m->stream));
    std::vector<uint32_t> perm(n);
    for (uint32_t i = 0; i < n; i++) perm[i] = i;
    std::mt19937 rng(seed);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (uint32_t ep = 0; ep < epochs; ep++) {
        std::shuffle(perm.begin(), perm.end(), rng);
        MCK(cudaMemcpyAsync(m->perm, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
        MCK(cudaMemsetAsync(m->loss, 0, 4, m->stream));
        MCK(cudaStreamSynchronize(m->stream));   // the host permutation buffer is reused next epoch
        for (uint32_t b0 = 0; b0 < n; b0 += batch) {
            const uint32_t nb = std::min(batch, n - b0);
            const uint32_t *idx = m->perm + b0;
            k_gather_rows<<<(nb * kMlpIn + 255) / 256, 256, 0, m->stream>>>(m->X, idx, m->bx, nb, kMlpIn);
            k_gather_rows<<<(nb * 2 + 255) / 256, 256, 0, m->stream>>>(m->Y, idx, m->by, nb, 2);
            if (mask) k_gather_rows<<<(nb * 2 + 255) / 256, 256, 0, m->stream>>>(m->M, idx, m->bm, nb, 2);
            if ((rc = fwd_bwd(m, m->bx, m->by, mask ? m->bm : nullptr, nb, 1.0f / nb))) return rc;
            m->adam_step++;
            const float bc1 = 1.0f - std::pow(b1, (float)m->adam_step), bc2 = 1.0f - std::pow(b2, (float)m->adam_step);
            k_adam<<<(kMlpParams + 255) / 256, 256, 0, m->stream>>>(m->params, m->grad, m->m, m->v, kMlpParams, lr, b1, b2,
                                                                  eps, bc1, bc2);
            if ((rc = refresh_bf16(m))) return rc;
        }
        if (epoch_loss) {
            float l = 0.f;
            MCK(cudaMemcpyAsync(&l, m->loss, 4, cudaMemcpyDeviceToHost, m->stream));
            MCK(cudaStreamSynchronize(m->stream));
            epoch_loss[ep] = l / n;
        }
    }
    MCK(cudaStreamSynchronize(m->stream));
    return SPHGB_OK;
}

}  // extern "C"
