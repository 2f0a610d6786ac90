// letkf_prep.cu -- observation operator H on all members, mean removal, and
// the lat-lon bucket grid of the observations.
//
// Reference: gen_obs_struct (code/x86/TradDA/DA/LETKF/src/letkf_obs.F90:16-182)
// with find_obs_grid (:187-243), ps2ph_3d_interp and obs_interpolation_3d_2
// (obs_make.F90:233-381).  One warp per 32 observations: the scalar terms of
// an observation on one lane, then for each observation the lanes stride over
// the members, so every state read is a contiguous run of the member-fastest
// state (coalesced), and the ensemble mean is a warp-shuffle reduction.  A
// run whose state is still being copied in runs the geometry pass (mode 1)
// first and the members pass (mode 2) after the copy.
#include "letkf_internal.cuh"

namespace {

// First 1-based index i (1..m) with (double)g[i-1] >= x, 0 if none.  g is
// ascending, so the binary search returns the linear scan's answer.
__device__ __forceinline__ int first_ge(const float *g, int m, double x)
{
    int lo = 0, hi = m;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((double)g[mid] >= x) hi = mid; else lo = mid + 1;
    }
    return (lo < m) ? lo + 1 : 0;
}

struct Corners {
    int64_t c11, c21, c12, c22;   // (lat tx-1, lon ty-1), (tx, ty-1), (tx-1, ty), (tx, ty)
    double t1, t2;
};

// Bilinear value of (xb + axb) for member e at row r (obs_make.F90:285-294);
// with axb NULL, xb holds the full members (a fused members run).
__device__ __forceinline__ double bilin(const double *__restrict__ xb, const double *__restrict__ axb,
                                        int n, int k, const Corners &q, int r, int e)
{
    const double a11 = axb ? axb[q.c11 * n + r] : 0.0, a21 = axb ? axb[q.c21 * n + r] : 0.0;
    const double a12 = axb ? axb[q.c12 * n + r] : 0.0, a22 = axb ? axb[q.c22 * n + r] : 0.0;
    const double v11 = xb[(q.c11 * n + r) * k + e] + a11;
    const double v21 = xb[(q.c21 * n + r) * k + e] + a21;
    const double v12 = xb[(q.c12 * n + r) * k + e] + a12;
    const double v22 = xb[(q.c22 * n + r) * k + e] + a22;
    const double r1 = v11 * q.t1 + v21 * (1.0 - q.t1);
    const double r2 = v12 * q.t1 + v22 * (1.0 - q.t1);
    return r1 * q.t2 + r2 * (1.0 - q.t2);
}

// The grid cell of a valid observation (find_obs_grid, letkf_obs.F90:199-241;
// the spacing is a float difference) and its state row: the level's row for
// level select (h_mode 1), else the variable's first row with psearch set for
// a 3-D variable (the pressure search of obs_interpolation_3d_2).
__device__ __forceinline__ void obs_stencil(const LgGrid &g, const LgParams &prm, double lat, double lon, int v,
                                            int lev, Corners &q, int &row, bool &psearch)
{
    const bool is3d = v >= g.nvar2d;
    const int tx = first_ge(g.glat, g.nlat + 1, lat);
    const int ty = first_ge(g.glon, g.nlon + 1, lon);
    double ax = 0.0, ay = 0.0;
    if (tx > 1) {
        const double dlat = (double)(g.glat[tx - 1] - g.glat[tx - 2]);
        ax = (dlat - lat + (double)g.glat[tx - 2]) / dlat;
    }
    if (ty > 1) {
        const double dlon = (double)(g.glon[ty - 1] - g.glon[ty - 2]);
        ay = (dlon - lon + (double)g.glon[ty - 2]) / dlon;
    }
    // rows beyond the poles clamp, columns wrap around the circle
    const int la0 = min(max(tx - 2, 0), g.nlat - 1), la1 = min(max(tx - 1, 0), g.nlat - 1);
    const int lo0 = ((ty - 2) % g.nlon + g.nlon) % g.nlon, lo1 = (ty - 1) % g.nlon;
    q.c11 = la0 + (int64_t)g.nlat * lo0;
    q.c21 = la1 + (int64_t)g.nlat * lo0;
    q.c12 = la0 + (int64_t)g.nlat * lo1;
    q.c22 = la1 + (int64_t)g.nlat * lo1;
    q.t1 = ax;
    q.t2 = ay;
    const int start = is3d ? g.nvar2d + (v - g.nvar2d) * g.nz : v;
    psearch = is3d && prm.h_mode == 0;
    row = (is3d && prm.h_mode == 1) ? start + lev - 1 : start;
}

// Validity of an observation as k_obs_prepare tests it, with its level.
__device__ __forceinline__ bool obs_valid(const LgGrid &g, const LgParams &prm, double lat, double lon, int v,
                                          const int32_t *olev, const double *oph, int64_t o, int &lev)
{
    const bool is3d = v >= g.nvar2d;
    lev = 1;
    bool ok = (lat >= -90.0 && lat <= 90.0 && lon >= 0.0 && lon <= 360.0 && v >= 0 && v < g.nvar2d + g.nvar3d);
    if (ok && is3d && prm.h_mode == 1) {
        lev = olev[o];
        ok = lev >= 1 && lev <= g.nz;
    }
    if (ok && is3d && prm.h_mode == 0) ok = oph[o] > 0.0;
    return ok;
}

// The state rows the observation operator reads, copied from the caller's
// host arrays (a device-accessible view: mapped page-locked memory, or
// pageable memory where the device shares the host's page tables) into the
// device state, so that H can run while the bulk copy of the state is still
// under way: the level's row of each observation's four stencil columns (with
// the pressure search, the surface-pressure row and every level of the
// variable), each (column, row) once per run (a bit in `mark` decides which
// lane claims it), k doubles of xb and one of axb.  A lane owns one
// (observation, corner) pair; the warp then copies the rows its lanes claimed,
// four at a time, so that many reads over the host link are in flight.  The
// host arrays hold column c at host column off + c % nlat + ld * (c / nlat).
__global__ void __launch_bounds__(256)
k_gather_rows(LgGrid g, LgParams prm, int64_t nobs, const double *__restrict__ olat,
              const double *__restrict__ olon, const double *__restrict__ oph, const int32_t *__restrict__ olev,
              const int32_t *__restrict__ ovar, const double *__restrict__ hxb, const double *__restrict__ haxb,
              int64_t ld, int64_t off, double *__restrict__ dxb, double *__restrict__ daxb,
              unsigned *__restrict__ mark, int vec2)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int k = g.k, n = g.n;
    const int64_t npairs = 4 * nobs;
    for (int64_t base = warp * 32; base < npairs; base += nwarps * 32) {
        // this lane's (observation, corner): its column, first row and rows
        const int64_t pr = base + lane;
        int64_t col = 0, hcol = 0;
        int row0 = 0, nrows = 0;
        if (pr < npairs) {
            const int64_t o = pr >> 2;
            const double lat = olat[o], lon = olon[o];
            const int v = ovar[o];
            int lev = 1;
            if (obs_valid(g, prm, lat, lon, v, olev, oph, o, lev)) {
                Corners q;
                bool psearch = false;
                obs_stencil(g, prm, lat, lon, v, lev, q, row0, psearch);
                const int corner = (int)(pr & 3);
                col = corner == 0 ? q.c11 : corner == 1 ? q.c21 : corner == 2 ? q.c12 : q.c22;
                hcol = off + col % g.nlat + ld * (col / g.nlat);
                nrows = psearch ? g.nz + 1 : 1;
            }
        }
        int maxr = nrows;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) maxr = max(maxr, __shfl_xor_sync(0xffffffffu, maxr, o));
        for (int ri = 0; ri < maxr; ri++) {
            const int r = ri == g.nz ? g.ps_row : row0 + ri;
            bool fresh = false;
            if (ri < nrows) {
                const int64_t bit = col * n + r;
                const unsigned m = 1u << (bit & 31);
                fresh = (atomicOr(mark + (bit >> 5), m) & m) == 0;
                if (fresh) daxb[bit] = haxb[hcol * n + r];
            }
            unsigned todo = __ballot_sync(0xffffffffu, fresh);
            while (todo) {
                // up to four claimed rows, copied by the whole warp
                int src[4];
                int cnt = 0;
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    src[t] = todo ? __ffs(todo) - 1 : -1;
                    if (todo) {
                        todo &= todo - 1;
                        cnt++;
                    }
                }
                const double *sp[4];
                double *dp[4];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int sl = src[t] < 0 ? 0 : src[t];
                    const long long c = __shfl_sync(0xffffffffu, (long long)col, sl);
                    const long long hc = __shfl_sync(0xffffffffu, (long long)hcol, sl);
                    const int rr = __shfl_sync(0xffffffffu, r, sl);
                    sp[t] = hxb + ((int64_t)hc * n + rr) * k;
                    dp[t] = dxb + ((int64_t)c * n + rr) * k;
                }
                if (vec2) {
                    for (int e = lane; e < k / 2; e += 32) {
                        double2 x[4];
#pragma unroll
                        for (int t = 0; t < 4; t++)
                            if (t < cnt) x[t] = reinterpret_cast<const double2 *>(sp[t])[e];
#pragma unroll
                        for (int t = 0; t < 4; t++)
                            if (t < cnt) reinterpret_cast<double2 *>(dp[t])[e] = x[t];
                    }
                } else {
                    for (int e = lane; e < k; e += 32) {
                        double x[4];
#pragma unroll
                        for (int t = 0; t < 4; t++)
                            if (t < cnt) x[t] = sp[t][e];
#pragma unroll
                        for (int t = 0; t < 4; t++)
                            if (t < cnt) dp[t][e] = x[t];
                    }
                }
            }
        }
    }
}

__device__ __forceinline__ double ph_interface(const LgGrid &g, int i, double ps)
{
    return g.hyai[i] * (g.p0 - g.ptop) + g.hybi[i] * (ps - g.ptop) + g.ptop;
}

__device__ __forceinline__ double ph_mid(const LgGrid &g, int i /* 0-based level */, double ps)
{
    return 0.5 * (ph_interface(g, i, ps) + ph_interface(g, i + 1, ps));
}

// One warp per group of 32 observations.  The per-observation scalar terms
// (validity, grid cell, weights, geometry, bucket; FP64 trig and divides) run
// one observation per lane, so a warp instruction serves 32 observations; the
// warp then sweeps the group one observation at a time with the lanes over the
// members, taking the cell from the owning lane by shuffles.  Arithmetic per
// observation is the same as in the one-warp-per-observation form.
__global__ void __launch_bounds__(256)
k_obs_prepare(LgGrid g, LgParams prm, const double *__restrict__ xb, const double *__restrict__ axb,
              int64_t nobs, const double *__restrict__ olat, const double *__restrict__ olon,
              const double *__restrict__ oph, const int32_t *__restrict__ olev,
              const int32_t *__restrict__ ovar, const double *__restrict__ oyo,
              const double *__restrict__ orinv, double *__restrict__ yb, double *__restrict__ dep,
              float *__restrict__ rinvf, double *__restrict__ os, double *__restrict__ oc,
              double *__restrict__ oyr, float4 *__restrict__ oxyz, int *__restrict__ obucket,
              float *__restrict__ ys32, float *__restrict__ oef, unsigned *__restrict__ ymax,
              int nblat, int nblon, double cell_lat, double cell_lon, unsigned *status, int mode)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int k = g.k, n = g.n;
    // the mean as sum * 2^-m when k is a power of two (exact, equal to sum / k)
    const bool kpow2 = (k & (k - 1)) == 0;
    const double invk = 1.0 / (double)k;
    float amax = 0.0f;       // the largest |ys32| and |oef| this lane wrote (mixed form)

    for (int64_t base = warp * 32; base < nobs; base += nwarps * 32) {
        // ---- per-observation terms, observation base + lane on this lane
        const int64_t o = base + lane;
        Corners q{0, 0, 0, 0, 0.0, 0.0};
        int row = 0;             // state row, or the variable's first level (pressure search)
        bool ok = false, psearch = false;
        double sr = 0.0, p_obs = 0.0;
        if (o < nobs) {
            const double lat = olat[o], lon = olon[o];
            const int v = ovar[o];
            int lev = 1;
            ok = obs_valid(g, prm, lat, lon, v, olev, oph, o, lev);
            if (!ok) {
                if (mode != 1) {
                    dep[o] = 0.0;
                    if (oef) oef[o] = 0.0f;
                }
                if (mode != 2) {
                    rinvf[o] = 0.0f;
                    obucket[o] = -1;
                    atomicOr(status, LG_ST_BAD_OBS);
                }
            } else {
                obs_stencil(g, prm, lat, lon, v, lev, q, row, psearch);
                if (psearch) p_obs = oph[o];
                const float rf = (float)orinv[o];
                // scaled perturbations for the tensor-core products: y sqrt(rdiaginv)
                sr = sqrt((double)rf);
            }
            if (ok && mode != 2) {
                rinvf[o] = (float)orinv[o];
                const double xr = lg_rad(lat), yr = lg_rad(lon);
                const double s = sin(xr), c = cos(xr);
                os[o] = s;
                oc[o] = c;
                oyr[o] = yr;
                oxyz[o] = make_float4((float)(c * cos(yr)), (float)(c * sin(yr)), (float)s,
                                      __int_as_float((int)o));
                int b = -1;
                if (fabs(lat) <= prm.obs_polar) {
                    int bl = (int)floor((lat + 90.0) / cell_lat);
                    int bn = (int)floor(lon / cell_lon);
                    bl = min(max(bl, 0), nblat - 1);
                    bn = min(max(bn, 0), nblon - 1);
                    b = bl * nblon + bn;
                }
                obucket[o] = b;
            }
        }
        const unsigned okmask = __ballot_sync(0xffffffffu, ok);
        const unsigned psmask = __ballot_sync(0xffffffffu, psearch);
        if (mode == 1) continue;

        // ---- members of each observation of the group, lanes over the members
        double mymean = 0.0;
        const int gn = (int)min((int64_t)32, nobs - base);
        for (int j = 0; j < gn; j++) {
            const int64_t oj = base + j;
            if (!((okmask >> j) & 1u)) {
                for (int e = lane; e < k; e += 32) {
                    yb[oj * k + e] = 0.0;
                    if (ys32) ys32[oj * k + e] = 0.0f;
                }
                continue;
            }
            Corners qj;
            qj.c11 = __shfl_sync(0xffffffffu, (long long)q.c11, j);
            qj.c21 = __shfl_sync(0xffffffffu, (long long)q.c21, j);
            qj.c12 = __shfl_sync(0xffffffffu, (long long)q.c12, j);
            qj.c22 = __shfl_sync(0xffffffffu, (long long)q.c22, j);
            qj.t1 = __shfl_sync(0xffffffffu, q.t1, j);
            qj.t2 = __shfl_sync(0xffffffffu, q.t2, j);
            const int rj = __shfl_sync(0xffffffffu, row, j);
            const bool psj = (psmask >> j) & 1u;
            const double pj = psj ? __shfl_sync(0xffffffffu, p_obs, j) : 0.0;
            double sum = 0.0;
            double yv[LG_MAX_ENS / 32];
#pragma unroll
            for (int i = 0; i < LG_MAX_ENS / 32; i++) {
                const int e = lane + 32 * i;
                double y = 0.0;
                if (e < k) {
                    if (!psj) {
                        y = bilin(xb, axb, n, k, qj, rj, e);
                    } else {
                        // member's pressure profile, level search, log-p interpolation
                        const double ps = bilin(xb, axb, n, k, qj, g.ps_row, e);
                        int jl = 1;
                        while (jl <= g.nz && pj > ph_mid(g, jl - 1, ps)) jl++;
                        const int pos = jl - 1;
                        if (pos >= 1 && pos < g.nz) {
                            const int tl = rj + pos - 1;
                            const double pa = ph_mid(g, pos, ps), pb = ph_mid(g, pos - 1, ps);
                            const double t3 = (log(pa) - log(pj)) / (log(pa) - log(pb));
                            const double r1 = bilin(xb, axb, n, k, qj, tl, e);
                            const double r3 = bilin(xb, axb, n, k, qj, tl + 1, e);
                            y = r1 * t3 + r3 * (1.0 - t3);
                        } else {
                            const int tl = (pos == 0) ? rj : rj + g.nz - 1;
                            y = bilin(xb, axb, n, k, qj, tl, e);
                        }
                    }
                    sum += y;
                }
                yv[i] = y;
            }
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, s);
            const double mean = kpow2 ? sum * invk : sum / (double)k;
            if (lane == j) mymean = mean;
#pragma unroll
            for (int i = 0; i < LG_MAX_ENS / 32; i++) {
                const int e = lane + 32 * i;
                if (e < k) yb[oj * k + e] = yv[i] - mean;
            }
            if (ys32) {
                const double srj = __shfl_sync(0xffffffffu, sr, j);
#pragma unroll
                for (int i = 0; i < LG_MAX_ENS / 32; i++) {
                    const int e = lane + 32 * i;
                    if (e < k) {
                        const float v = (float)((yv[i] - mean) * srj);
                        ys32[oj * k + e] = v;
                        amax = fmaxf(amax, fabsf(v));
                    }
                }
            }
        }

        // ---- departures, observation base + lane on this lane
        if (ok) {
            const double d = oyo[o] - mymean;
            dep[o] = d;
            // the mixed form's departure factor: e = sqrt(rloc) sqrt(rdiaginv) dep
            if (oef) {
                const float ef = sqrtf(rinvf[o]) * (float)d;
                oef[o] = ef;
                amax = fmaxf(amax, fabsf(ef));
            }
        }
    }
    // the run's largest magnitude of the A build's operands (float bits of a
    // non-negative value order as unsigned integers)
    if (ymax && mode != 1) {
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, s));
        if (lane == 0 && amax > 0.0f) atomicMax(ymax, __float_as_uint(amax));
    }
}

__global__ void k_bucket_count(int64_t nobs, const int *__restrict__ obucket, int *__restrict__ count)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < nobs;
         o += (int64_t)gridDim.x * blockDim.x) {
        const int b = obucket[o];
        if (b >= 0) atomicAdd(&count[b], 1);
    }
}

// Exclusive scan of n counts into out[0..n] with one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_exclusive(const int *__restrict__ in, int *__restrict__ out, int n)
{
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (n + 1023) / 1024;
    const int b = min(n, t * per), e = min(n, b + per);
    int s = 0;
    for (int i = b; i < e; i++) s += in[i];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        int v = (t >= off) ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;
    for (int i = b; i < e; i++) {
        out[i] = run;
        run += in[i];
    }
    if (t == 1023) out[n] = part[1023];
}

__global__ void k_bucket_fill(int64_t nobs, const int *__restrict__ obucket, const int *__restrict__ start,
                              int *__restrict__ cursor, const float4 *__restrict__ oxyz,
                              int *__restrict__ bidx, float4 *__restrict__ bxyz)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < nobs;
         o += (int64_t)gridDim.x * blockDim.x) {
        const int b = obucket[o];
        if (b < 0) continue;
        const int pos = start[b] + atomicAdd(&cursor[b], 1);
        bidx[pos] = (int)o;
        bxyz[pos] = oxyz[o];
    }
}

int grid_for(int64_t work, int threads, int cap)
{
    int64_t b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

}  // namespace

cudaError_t lg_launch_obs_prepare(letkf_ctx *ctx, const LgGrid &g, const double *xb,
                                  const double *axb, int64_t nobs, const double *olat,
                                  const double *olon, const double *oph, const int32_t *olev,
                                  const int32_t *ovar, const double *oyo, const double *orinv, int mode)
{
    const bool mixed = lg_is_mixed(ctx->params.precision);
    if (mixed && mode != 1) {
        const cudaError_t e = cudaMemsetAsync(ctx->d_ymax.p, 0, sizeof(unsigned), ctx->stream);
        if (e != cudaSuccess) return e;
    }
    if (nobs == 0) return cudaSuccess;
    const LgParams prm = lg_params(ctx);
    const int blocks = grid_for(nobs, 256, 152 * 64);
    lg_count_launch();
    k_obs_prepare<<<blocks, 256, 0, ctx->stream>>>(
        g, prm, xb, axb, nobs, olat, olon, oph, olev, ovar, oyo, orinv, ctx->d_yb.p, ctx->d_dep.p,
        ctx->d_rinvf.p, ctx->d_os.p, ctx->d_oc.p, ctx->d_oyr.p, ctx->d_oxyz.p, ctx->d_obucket.p,
        mixed ? ctx->d_ys32.p : nullptr, mixed ? ctx->d_oef.p : nullptr, mixed ? ctx->d_ymax.p : nullptr,
        ctx->nblat, ctx->nblon, ctx->cell_lat, ctx->cell_lon, ctx->d_status.p, mode);
    return cudaGetLastError();
}

cudaError_t lg_launch_gather_rows(letkf_ctx *ctx, cudaStream_t stream, const LgGrid &g, int64_t nobs,
                                  const double *olat, const double *olon, const double *oph,
                                  const int32_t *olev, const int32_t *ovar, const double *hxb,
                                  const double *haxb, double *dxb, double *daxb)
{
    if (nobs == 0) return cudaSuccess;
    const size_t words = ((size_t)ctx->ncol * ctx->n + 31) / 32;
    cudaError_t e = ctx->d_rowmark.reserve(words);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_rowmark.p, 0, words * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    const LgParams prm = lg_params(ctx);
    lg_count_launch();
    // two blocks per SM keep ~1 MB of reads in flight (enough for the host
    // link) and leave the SMs to the geometry and search running beside it
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    k_gather_rows<<<grid_for(nobs * 32, 256, 2 * (nsm > 0 ? nsm : 152)), 256, 0, stream>>>(
        g, prm, nobs, olat, olon, oph, olev, ovar, hxb, haxb, ctx->host_ld, ctx->host_off, dxb, daxb,
        ctx->d_rowmark.p, (g.k % 2 == 0 && (uintptr_t)hxb % 16 == 0 && (uintptr_t)dxb % 16 == 0) ? 1 : 0);
    return cudaGetLastError();
}

// Per-row and per-column geometry of the cube centres, with the same device
// functions as the per-obs terms (the exact distance test uses both).
__global__ void k_geo_tables(const float *__restrict__ glat, const float *__restrict__ glon, int nlat, int nlon,
                             double *__restrict__ row_s, double *__restrict__ row_c, double *__restrict__ col_yr,
                             double *__restrict__ col_cos, double *__restrict__ col_sin)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlat + nlon; i += gridDim.x * blockDim.x) {
        if (i < nlat) {
            const double xr = lg_rad((double)glat[i]);
            row_s[i] = sin(xr);
            row_c[i] = cos(xr);
        } else {
            const int j = i - nlat;
            const double yr = lg_rad((double)glon[j]);
            col_yr[j] = yr;
            col_cos[j] = cos(yr);
            col_sin[j] = sin(yr);
        }
    }
}

cudaError_t lg_launch_geo_tables(letkf_ctx *ctx)
{
    cudaError_t e;
    if ((e = ctx->d_row_s.reserve(ctx->nlat)) || (e = ctx->d_row_c.reserve(ctx->nlat)) ||
        (e = ctx->d_col_yr.reserve(ctx->nlon)) || (e = ctx->d_col_cos.reserve(ctx->nlon)) ||
        (e = ctx->d_col_sin.reserve(ctx->nlon)))
        return e;
    lg_count_launch();
    k_geo_tables<<<grid_for(ctx->nlat + ctx->nlon, 256, 1024), 256, 0, ctx->stream>>>(
        ctx->d_glat.p, ctx->d_glon.p, ctx->nlat, ctx->nlon, ctx->d_row_s.p, ctx->d_row_c.p, ctx->d_col_yr.p,
        ctx->d_col_cos.p, ctx->d_col_sin.p);
    return cudaGetLastError();
}

LgSearchGeo lg_search_geo(letkf_ctx *ctx)
{
    LgSearchGeo sg;
    sg.row_s = ctx->d_row_s.p;
    sg.row_c = ctx->d_row_c.p;
    sg.col_yr = ctx->d_col_yr.p;
    sg.col_cos = ctx->d_col_cos.p;
    sg.col_sin = ctx->d_col_sin.p;
    // the squared chord of two unit vectors rounded to float is within ~4e-6
    // relative of the true one for cut-off angles above 0.05 rad, so
    // candidates more than 2e-5 relative inside or outside the cut-off are
    // decided by the float test and only the band between (and every
    // candidate of a smaller cap) takes the reference's double formula
    const double theta = 2.0 * ctx->params.loc_dist_km / LG_EARTH_A;
    sg.theta = (float)theta;
    if (theta > 0.05) {
        const double a = 2.0 * std::sin(0.5 * theta * (1.0 - 2e-5));
        const double b = 2.0 * std::sin(0.5 * theta * (1.0 + 2e-5));
        sg.lo2 = (float)(a * a);
        sg.hi2 = (float)(b * b);
    } else {
        sg.lo2 = -1.0f;           // every candidate takes the double test
        sg.hi2 = 1.0e30f;
    }
    // antipode buckets reach at most two bucket sizes from the antipode
    const double ext = 2.0 * (ctx->cell_lat + ctx->cell_lon) * (M_PI / 180.0);
    sg.anti_far = (theta + ext + 0.01 < M_PI) ? 1 : 0;
    return sg;
}

void lg_launch_scan_exclusive(const int *in, int *out, int n, cudaStream_t stream)
{
    lg_count_launch();
    k_scan_exclusive<<<1, 1024, 0, stream>>>(in, out, n);
}

cudaError_t lg_launch_buckets(letkf_ctx *ctx, int64_t nobs)
{
    const int nb = ctx->nblat * ctx->nblon;
    cudaError_t e = cudaMemsetAsync(ctx->d_bcount.p, 0, sizeof(int) * nb, ctx->stream);
    if (e != cudaSuccess) return e;
    if (nobs > 0) {
        lg_count_launch();
        k_bucket_count<<<grid_for(nobs, 256, 152 * 16), 256, 0, ctx->stream>>>(nobs, ctx->d_obucket.p,
                                                                          ctx->d_bcount.p);
    }
    lg_count_launch();
    k_scan_exclusive<<<1, 1024, 0, ctx->stream>>>(ctx->d_bcount.p, ctx->d_bstart.p, nb);
    e = cudaMemsetAsync(ctx->d_bcount.p, 0, sizeof(int) * nb, ctx->stream);
    if (e != cudaSuccess) return e;
    if (nobs > 0) {
        lg_count_launch();
        k_bucket_fill<<<grid_for(nobs, 256, 152 * 16), 256, 0, ctx->stream>>>(
            nobs, ctx->d_obucket.p, ctx->d_bstart.p, ctx->d_bcount.p, ctx->d_oxyz.p, ctx->d_bidx.p,
            ctx->d_bxyz.p);
    }
    return cudaGetLastError();
}
