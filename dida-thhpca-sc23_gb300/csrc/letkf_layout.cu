// letkf_layout.cu -- the coupler's state layout transforms on the device.
//
// Reference: struct_atm2endnn / struct_endnn2atm and their mean-only forms
// (code/x86/TradDA/DA/EnDNN/src/data_trans.F90:1-70).  The model side holds a
// variable group as xb(ens, lon, lat, n) (Fortran order: members fastest, then
// longitude, latitude, the group's rows); the analysis side holds the whole
// state as xb2(ens_max, n_max, lat, lon), i.e. [col][row][member] with
// col = lat + nlat * lon.  atm2endnn writes the group into rows
// n_start..n_start+n-1 and members ens_start..ens_start+ens-1 of xb2;
// endnn2atm reads them back.  Both are copies of contiguous member vectors
// (one warp per vector, members across lanes); the mean-only forms move
// single values, one thread each, in the destination's order.
#include "letkf_internal.cuh"

namespace {

constexpr int kT = 256;

// vector v enumerates (nn, i, j) in xb2 order: v = nn + n * (i + nx * j)
__global__ void __launch_bounds__(kT)
k_atm2endnn(int ens, int n, int nx, int ny, int ens_max, int n_max, int es, int ns,
            const double *__restrict__ xb, double *__restrict__ xb2)
{
    const int lane = threadIdx.x & 31;
    const int64_t nv = (int64_t)n * nx * ny, warps = (int64_t)gridDim.x * (kT / 32);
    for (int64_t v = blockIdx.x * (int64_t)(kT / 32) + (threadIdx.x >> 5); v < nv; v += warps) {
        const int nn = (int)(v % n);
        const int64_t ij = v / n;
        const int i = (int)(ij % nx), j = (int)(ij / nx);
        const double *src = xb + (((int64_t)nn * nx + i) * ny + j) * ens;
        double *dst = xb2 + (((int64_t)j * nx + i) * n_max + ns + nn) * ens_max + es;
        for (int e = lane; e < ens; e += 32) dst[e] = src[e];
    }
}

// vector v enumerates (j, i, nn) in xb order: v = j + ny * (i + nx * nn)
__global__ void __launch_bounds__(kT)
k_endnn2atm(int ens, int n, int nx, int ny, int ens_max, int n_max, int es, int ns,
            const double *__restrict__ xb, double *__restrict__ xb2)
{
    const int lane = threadIdx.x & 31;
    const int64_t nv = (int64_t)n * nx * ny, warps = (int64_t)gridDim.x * (kT / 32);
    for (int64_t v = blockIdx.x * (int64_t)(kT / 32) + (threadIdx.x >> 5); v < nv; v += warps) {
        const int j = (int)(v % ny);
        const int64_t rest = v / ny;
        const int i = (int)(rest % nx), nn = (int)(rest / nx);
        const double *src = xb + (((int64_t)j * nx + i) * n_max + ns + nn) * ens_max + es;
        double *dst = xb2 + v * ens;
        for (int e = lane; e < ens; e += 32) dst[e] = src[e];
    }
}

__global__ void __launch_bounds__(kT)
k_atm2endnn_a(int n, int nx, int ny, int n_max, int ns, const double *__restrict__ axb, double *__restrict__ axb2)
{
    const int64_t total = (int64_t)n * nx * ny;
    for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        const int nn = (int)(t % n);
        const int64_t ij = t / n;
        const int i = (int)(ij % nx), j = (int)(ij / nx);
        axb2[((int64_t)j * nx + i) * n_max + ns + nn] = axb[((int64_t)nn * nx + i) * ny + j];
    }
}

__global__ void __launch_bounds__(kT)
k_endnn2atm_a(int n, int nx, int ny, int n_max, int ns, const double *__restrict__ axb, double *__restrict__ axb2)
{
    const int64_t total = (int64_t)n * nx * ny;
    for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        const int j = (int)(t % ny);
        const int64_t rest = t / ny;
        const int i = (int)(rest % nx), nn = (int)(rest / nx);
        axb2[t] = axb[((int64_t)j * nx + i) * n_max + ns + nn];
    }
}

unsigned blocks_for(int64_t work, int per_block)
{
    const int64_t b = (work + per_block - 1) / per_block;
    return (unsigned)(b < 1 ? 1 : (b < (1 << 20) ? b : (1 << 20)));
}

bool dims_ok(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start, int n_start)
{
    return ens >= 1 && n >= 1 && nx >= 1 && ny >= 1 && ens_start >= 1 && n_start >= 1 &&
           ens_start - 1 + ens <= ens_max && n_start - 1 + n <= n_max;
}

int finish(cudaError_t e) { return e == cudaSuccess ? LETKF_OK : LETKF_ERR_CUDA; }

}  // namespace

extern "C" {

int letkf_struct_atm2endnn(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start, int n_start,
                           const double *xb, double *xb2, void *stream)
{
    if (!xb || !xb2 || !dims_ok(ens, n, nx, ny, ens_max, n_max, ens_start, n_start)) return LETKF_ERR_INVALID;
    lg_count_launch();
    k_atm2endnn<<<blocks_for((int64_t)n * nx * ny, kT / 32), kT, 0, (cudaStream_t)stream>>>(
        ens, n, nx, ny, ens_max, n_max, ens_start - 1, n_start - 1, xb, xb2);
    return finish(cudaGetLastError());
}

int letkf_struct_endnn2atm(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start, int n_start,
                           const double *xb, double *xb2, void *stream)
{
    if (!xb || !xb2 || !dims_ok(ens, n, nx, ny, ens_max, n_max, ens_start, n_start)) return LETKF_ERR_INVALID;
    lg_count_launch();
    k_endnn2atm<<<blocks_for((int64_t)n * nx * ny, kT / 32), kT, 0, (cudaStream_t)stream>>>(
        ens, n, nx, ny, ens_max, n_max, ens_start - 1, n_start - 1, xb, xb2);
    return finish(cudaGetLastError());
}

int letkf_struct_atm2endnn_a(int n, int nx, int ny, int n_max, int n_start, const double *axb, double *axb2,
                             void *stream)
{
    if (!axb || !axb2 || !dims_ok(1, n, nx, ny, 1, n_max, 1, n_start)) return LETKF_ERR_INVALID;
    lg_count_launch();
    k_atm2endnn_a<<<blocks_for((int64_t)n * nx * ny, kT), kT, 0, (cudaStream_t)stream>>>(n, nx, ny, n_max,
                                                                                          n_start - 1, axb, axb2);
    return finish(cudaGetLastError());
}

int letkf_struct_endnn2atm_a(int n, int nx, int ny, int n_max, int n_start, const double *axb, double *axb2,
                             void *stream)
{
    if (!axb || !axb2 || !dims_ok(1, n, nx, ny, 1, n_max, 1, n_start)) return LETKF_ERR_INVALID;
    lg_count_launch();
    k_endnn2atm_a<<<blocks_for((int64_t)n * nx * ny, kT), kT, 0, (cudaStream_t)stream>>>(n, nx, ny, n_max,
                                                                                          n_start - 1, axb, axb2);
    return finish(cudaGetLastError());
}

}  // extern "C"
