// Akinci2012 boundary volumes without any device allocation.
//
// For callers that must not allocate device memory themselves or through this
// library: code that runs while a stream is being captured into a CUDA graph
// (cudaMalloc is not capturable), and hosts that own a fixed device-memory
// budget or pool and forbid allocations after start-up (real-time and embedded
// set-ups, plugins inside a larger renderer or solver).  The caller passes
// device pointers for the input positions and the output volumes; every scratch
// buffer lives in one file-scope __device__ array of fixed size that each GPU
// loading this library holds until the process exits.
//
// Same result as sphgb_upload_boundary + sphgb_download(SPHGB_FIELD_BOUNDARY_VOLUME)
// (BoundaryModel_Akinci2012::computeBoundaryVolume, BoundaryModel_Akinci2012.cpp:48-75):
// the same kernels run on the scratch array instead of context allocations.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/sphgb300.h"
#include "sph_ctx.h"

using namespace sphgb;

namespace {

constexpr uint32_t kMaxB = SPHGB_NOALLOC_MAX_BOUNDARY;
constexpr uint32_t kMaxCells = SPHGB_NOALLOC_MAX_CELLS;
constexpr uint32_t kMaxTiles = (kMaxB + kSortTile - 1) / kSortTile;

// byte offsets of the scratch sub-arrays (all multiples of 256)
constexpr size_t kOffXbIn = 0;
constexpr size_t kOffXb = kOffXbIn + (size_t)kMaxB * sizeof(float4);
constexpr size_t kOffVol = kOffXb + (size_t)kMaxB * sizeof(float4);
constexpr size_t kOffBid = kOffVol + (size_t)kMaxB * sizeof(float);
constexpr size_t kOffKeys = kOffBid + (size_t)kMaxB * 4;
constexpr size_t kOffVals = kOffKeys + (size_t)kMaxB * 4;
constexpr size_t kOffKeys2 = kOffVals + (size_t)kMaxB * 4;
constexpr size_t kOffVals2 = kOffKeys2 + (size_t)kMaxB * 4;
constexpr size_t kOffCells = kOffVals2 + (size_t)kMaxB * 4;
constexpr size_t kOffHist = kOffCells + (size_t)kMaxB * 4;
constexpr size_t kOffStart = kOffHist + (size_t)(kMaxTiles + 1) * 256 * 4;   // tile rows + digit totals
constexpr size_t kOffEnd = kOffStart + (size_t)kMaxCells * 4;
constexpr size_t kScratchBytes = kOffEnd + (size_t)kMaxCells * 4;
static_assert(kScratchBytes % 256 == 0, "scratch layout must stay 256-byte aligned");

// The scratch.  In host code this name is only a host-side stand-in for the
// symbol, never a device address: host code gets the address with
// cudaGetSymbolAddress (once per device, below) and passes that to kernels.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
unsigned char *g_ptr[kMaxDevices] = {};

__global__ void k_pack(const float *__restrict__ xb, float4 *__restrict__ out, uint32_t nb)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb) out[i] = make_float4(xb[3 * i], xb[3 * i + 1], xb[3 * i + 2], 0.0f);
}

__global__ void k_unsort_volume(const float4 *__restrict__ xb, const uint32_t *__restrict__ bid,
                                float *__restrict__ vol, uint32_t nb)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nb) vol[bid[k]] = xb[k].w;
}

// Address of the scratch array on the current device; the first call on a
// device looks it up (with that device current) and caches it.
int scratch_for_current_device(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SPHGB_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return SPHGB_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return SPHGB_ERR_CUDA;
        }
        g_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_ptr[dev];
    return SPHGB_OK;
}

}  // namespace

extern "C" int sphgb_boundary_volume_noalloc(const float *xb, uint32_t nb, double particle_radius,
                                             const double box_min[3], const double box_max[3], float *volume,
                                             void *stream)
{
    if (nb == 0) return SPHGB_OK;
    if (!xb || !volume || !box_min || !box_max || !(particle_radius > 0)) return SPHGB_ERR_ARGUMENT;
    if (nb > kMaxB) return SPHGB_ERR_CAPACITY;
    // the cell grid of the context path: cell 1.001 h, one cell of margin, clamped positions
    const double h = 4.0 * particle_radius;
    const double cell = h * 1.001;
    double org[3];
    int dim[3];
    size_t ncell = 1;
    int maxdim = 1;
    if (!std::isfinite(particle_radius)) return SPHGB_ERR_ARGUMENT;
    for (int d = 0; d < 3; d++) {
        if (!std::isfinite(box_min[d]) || !std::isfinite(box_max[d]) || !(box_max[d] >= box_min[d]))
            return SPHGB_ERR_ARGUMENT;
        org[d] = box_min[d] - cell;
        // the cell count in double first: an extent far beyond the grid never reaches the int
        const double cells = std::floor((box_max[d] - org[d]) / cell) + 2.0;
        if (!(cells <= 1024.0)) return SPHGB_ERR_GRID;
        dim[d] = (int)cells;
        maxdim = dim[d] > maxdim ? dim[d] : maxdim;
        ncell *= (size_t)dim[d];
    }
    if (ncell > kMaxCells) return SPHGB_ERR_GRID;
    int bits = 1;
    while ((1 << bits) < maxdim) bits++;

    unsigned char *base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    DevParams<float> P{};
    P.K.h = (float)h;
    P.K.invh = (float)(1.0 / h);
    P.K.invh2 = (float)(1.0 / (h * h));
    P.K.k = (float)(8.0 / (M_PI * h * h * h));
    P.K.l = (float)(48.0 / (M_PI * h * h * h));
    P.K.w0 = P.K.k;
    P.K.h2 = (float)(h * h);
    P.nscenes = 1;
    P.s0.ox = (float)org[0];
    P.s0.oy = (float)org[1];
    P.s0.oz = (float)org[2];
    P.s0.inv_cell = (float)(1.0 / cell);
    P.s0.dimx = dim[0];
    P.s0.dimy = dim[1];
    P.s0.dimz = dim[2];
    P.nb = nb;
    DevBufs<float> B{};
    float4 *xb_in = reinterpret_cast<float4 *>(base + kOffXbIn);
    B.xb = reinterpret_cast<float4 *>(base + kOffXb);
    B.bscratch = reinterpret_cast<float *>(base + kOffVol);
    B.bid = reinterpret_cast<uint32_t *>(base + kOffBid);
    B.bcstart = reinterpret_cast<uint32_t *>(base + kOffStart);
    B.bcend = reinterpret_cast<uint32_t *>(base + kOffEnd);
    uint32_t *keys = reinterpret_cast<uint32_t *>(base + kOffKeys);
    uint32_t *vals = reinterpret_cast<uint32_t *>(base + kOffVals);
    uint32_t *keys2 = reinterpret_cast<uint32_t *>(base + kOffKeys2);
    uint32_t *vals2 = reinterpret_cast<uint32_t *>(base + kOffVals2);
    uint32_t *cells = reinterpret_cast<uint32_t *>(base + kOffCells);
    uint32_t *hist = reinterpret_cast<uint32_t *>(base + kOffHist);

    // the scratch keeps the previous call's contents: empty cells must read as empty
    if (cudaMemsetAsync(B.bcstart, 0xff, ncell * 4, s) != cudaSuccess) return SPHGB_ERR_CUDA;
    const unsigned blocks = (nb + kBlock - 1) / kBlock;
    k_pack<<<blocks, kBlock, 0, s>>>(xb, xb_in, nb);
    launch_boundary_keys<float>(P, xb_in, nullptr, keys, vals, s);
    const uint32_t tiles = (nb + kSortTile - 1) / kSortTile;
    const bool sw = radix_sort_pairs(keys, vals, keys2, vals2, nb, 3 * bits, hist, tiles, s);
    launch_boundary_gather<float>(P, B, xb_in, nullptr, sw ? vals2 : vals, cells, s);
    launch_boundary_volume<float>(P, B, s);
    k_unsort_volume<<<blocks, kBlock, 0, s>>>(B.xb, B.bid, volume, nb);
    if (cudaGetLastError() != cudaSuccess) return SPHGB_ERR_CUDA;
    return SPHGB_OK;
}
