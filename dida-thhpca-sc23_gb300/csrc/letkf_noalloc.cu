// letkf_noalloc.cu -- the batched LETKF core for callers that cannot allocate
// device memory.
//
// Some host programs may not call cudaMalloc/cudaFree: a model that reserves
// the GPU's memory for its own pool at start-up and hands out only buffers it
// owns, or a caller that must not add the implicit device-wide
// synchronization that cudaMalloc and cudaFree bring.  For them
// letkf_gpu_core_batch_noalloc takes every input and output as device memory
// the caller owns, and keeps its own scratch (the per-problem observation
// counts, a status word and the kernel counters) in the file-scope array
// below instead of allocating it.
#include <mutex>

#include "letkf_internal.cuh"

bool lg_core_supports(int k);
cudaError_t lg_launch_core_batch_raw(int k, double inflation, int64_t nb, const int64_t *d_off,
                                     const int32_t *d_cnt, const double *d_hx, const float *d_rdi,
                                     const double *d_dep, const double *d_rloc, double *d_trans,
                                     double *d_w, unsigned long long *counters, unsigned *status,
                                     cudaStream_t stream);

namespace {

constexpr size_t kCountBytes = sizeof(int32_t) * LETKF_NOALLOC_MAX_PROBLEMS;
constexpr size_t kStatusBytes = 256;   // status word, then LG_CNT_N counters
static_assert(8 + sizeof(unsigned long long) * LG_CNT_N <= kStatusBytes, "status area");

// Every GPU that loads this library holds this array until the process exits.
// In host code the name is only a stand-in for the device address, which is
// taken with cudaGetSymbolAddress per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kCountBytes + kStatusBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch on device `dev` (current), looked up once.
int scratch_address(int dev, unsigned char **out)
{
    if (dev < 0 || dev >= kMaxDevices) return LETKF_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return LETKF_ERR_CUDA;
        g_scratch_addr[dev] = p;
    }
    *out = (unsigned char *)g_scratch_addr[dev];
    return LETKF_OK;
}

// counts[b] = offsets[b+1] - offsets[b]; flags offsets that do not start at 0,
// are negative, go backwards or give a problem more than 2^31-1 rows.  A
// flagged problem gets count 0 (no row of it is read), and the core launched
// after this kernel returns at once when anything was flagged.
__global__ void k_noalloc_counts(int64_t nb, const int64_t *__restrict__ offsets,
                                 int32_t *__restrict__ counts, unsigned *__restrict__ status)
{
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb;
         b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o0 = offsets[b], o1 = offsets[b + 1];
        const int64_t c = o1 - o0;
        const bool bad = o0 < 0 || o1 < 0 || c < 0 || c > 0x7fffffffLL || (b == 0 && o0 != 0);
        counts[b] = bad ? 0 : (int32_t)c;
        if (bad) atomicOr(status, LG_ST_BAD_OBS);
    }
}

}  // namespace

extern "C" int letkf_gpu_core_batch_noalloc(int ens, double inflation, int64_t nb,
                                            const int64_t *offsets, const double *hxens,
                                            const float *rdiaginv, const double *dep,
                                            const double *rloc, double *trans, double *w,
                                            void *stream)
{
    if (nb < 0 || nb > LETKF_NOALLOC_MAX_PROBLEMS) return LETKF_ERR_INVALID;
    if (!lg_core_supports(ens)) return LETKF_ERR_UNSUPPORTED;
    if (!(inflation > 0.0)) return LETKF_ERR_INVALID;
    if (nb == 0) return LETKF_OK;
    if (!offsets || !hxens || !rdiaginv || !dep || !rloc || !trans || !w) return LETKF_ERR_INVALID;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return LETKF_ERR_CUDA;
    unsigned char *base = nullptr;
    int rc = scratch_address(dev, &base);
    if (rc != LETKF_OK) return rc;
    int32_t *counts = (int32_t *)base;
    unsigned *status = (unsigned *)(base + kCountBytes);
    unsigned long long *counters = (unsigned long long *)(base + kCountBytes + 8);
    cudaStream_t s = (cudaStream_t)stream;
    // the scratch keeps the previous call's contents: clear status and counters
    if (cudaMemsetAsync(base + kCountBytes, 0, kStatusBytes, s) != cudaSuccess) return LETKF_ERR_CUDA;
    const int blocks = (int)std::min<int64_t>((nb + 255) / 256, 1024);
    lg_count_launch();
    k_noalloc_counts<<<blocks, 256, 0, s>>>(nb, offsets, counts, status);
    if (cudaGetLastError() != cudaSuccess) return LETKF_ERR_CUDA;
    if (lg_launch_core_batch_raw(ens, inflation, nb, offsets, counts, hxens, rdiaginv, dep, rloc,
                                 trans, w, counters, status, s) != cudaSuccess)
        return LETKF_ERR_CUDA;
    unsigned st = 0;
    if (cudaMemcpyAsync(&st, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return LETKF_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return LETKF_ERR_CUDA;
    if (st & LG_ST_BAD_OBS) return LETKF_ERR_INVALID;
    if (st & LG_ST_NOT_CONV) return LETKF_ERR_NOT_CONVERGED;
    return LETKF_OK;
}
