// letkf_ingest.cu -- observations built on the device from the obs store's
// raw buffers, in the flat canonical order the analysis scans.
//
// Reference: read_obs (code/x86/TradDA/DA/LETKF/src/read_obs_mod.F90:339-448)
// and read_obs_regular (:451-651).  The reference fills obs_list arrays
// dis_yo(nvar, nz, nobs), obs_rinv(nvar, nz, nobs), ph(nz, nobs), lat/lon(nobs)
// and gen_yb_dis scans them obs by obs, level by level, variable by variable
// (letkf_yb.F90:71-113); the flat entry (obs, level, var) is entry
// (obs * nz + level) * nvar + var here.  Arithmetic follows the reference's
// kinds: the buffers are real(4), so yo = val + randn * sigma and
// rinv = 1 / sigma^2 are single precision (stored as double), and the
// regular builder's corner average and cell centres are single precision.
//   records: per record lon, lat, lev and val[2 nvar + 1] = (value, sigma)
//       per variable, then pressure; nz = 1 for single-level types; for
//       profile types (ADPUPA, GPSRO) the records of a profile are levels
//       1..nz in order (a record with lev 1 starts a profile, :400-423);
//   regular: obs at the centres of an obs grid given by its cell edges, lon
//       outer and lat inner (:506-513); sigma per (var, level) (:527-536);
//       values and pressure the average of four corner fields (:595);
//       yo = value + randn / sqrt(rinv) with rinv in double (:605-627).
// Each entry point writes the context's observation buffers and returns a
// letkf_obs of device pointers into them for letkf_gpu_run (LETKF_DEVICE_PTRS).
#include <vector>

#include "letkf_internal.cuh"

namespace {

constexpr int kT = 256;

__global__ void __launch_bounds__(kT)
k_obs_records(int64_t nrec, int nvar, int nz, const float *__restrict__ lon, const float *__restrict__ lat,
              const float *__restrict__ lev, const float *__restrict__ val, const float *__restrict__ randn,
              const int32_t *__restrict__ var_of, double *olat, double *olon, double *oph, int32_t *olev,
              int32_t *ovar, double *oyo, double *orinv, unsigned *status)
{
    const int64_t total = nrec * nvar;
    const int nv = 2 * nvar + 1;
    for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        const int64_t r = t / nvar;
        const int n = (int)(t % nvar);
        const int64_t prof = r / nz;
        const int level = (int)(r % nz) + 1;
        if (nz > 1 && lev[r] != (float)level) atomicOr(status, LG_ST_BAD_OBS);   // complete profiles, in order
        const float v = val[r * nv + 2 * n], sg = val[r * nv + 2 * n + 1];
        const float z = randn ? randn[(int64_t)n * nrec + r] : 0.0f;
        const float yo = __fadd_rn(v, __fmul_rn(z, sg));
        const float ri = __fdiv_rn(1.0f, __fmul_rn(sg, sg));
        const int64_t e = (prof * nz + (level - 1)) * nvar + n;
        // lat/lon of a profile are those of its level-1 record
        const int64_t r1 = prof * nz;
        olat[e] = (double)lat[r1];
        olon[e] = (double)lon[r1];
        oph[e] = (double)val[r * nv + 2 * nvar];
        olev[e] = level;
        ovar[e] = var_of[n];
        oyo[e] = (double)yo;
        orinv[e] = (double)ri;
    }
}

// Fortran arrays: corner(nvar+1, nz, nlat_o, nlon_o), r(nvar, nz),
// randn(nvar, nz, nobs) with nobs = nlat_o * nlon_o, obs index = j + nlat_o * i.
__global__ void __launch_bounds__(kT)
k_obs_regular(int nlat_o, int nlon_o, int nz, int nvar, const float *__restrict__ latn,
              const float *__restrict__ lats, const float *__restrict__ lonw, const float *__restrict__ lone,
              const float *__restrict__ rr, const float *__restrict__ nw, const float *__restrict__ sw,
              const float *__restrict__ ne, const float *__restrict__ se, const float *__restrict__ randn,
              const int32_t *__restrict__ var_of, double *olat, double *olon, double *oph, int32_t *olev,
              int32_t *ovar, double *oyo, double *orinv)
{
    const int64_t nobs = (int64_t)nlat_o * nlon_o, total = nobs * nz * nvar;
    for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        const int n = (int)(t % nvar);
        const int64_t ok = t / nvar;
        const int k = (int)(ok % nz);
        const int64_t o = ok / nz;
        const int j = (int)(o % nlat_o), i = (int)(o / nlat_o);
        auto corner = [&](const float *f, int q) {
            return f[(int64_t)q + (int64_t)(nvar + 1) * (k + (int64_t)nz * (j + (int64_t)nlat_o * i))];
        };
        auto avg = [&](int q) {
            return __fdiv_rn(__fadd_rn(__fadd_rn(__fadd_rn(corner(nw, q), corner(sw, q)), corner(ne, q)),
                                       corner(se, q)),
                             4.0f);
        };
        const float sg = rr[n + (int64_t)nvar * k];
        const double rinv = (double)__fdiv_rn(1.0f, __fmul_rn(sg, sg));
        const double z = randn ? (double)randn[n + (int64_t)nvar * (k + (int64_t)nz * o)] : 0.0;
        olat[t] = (double)__fdiv_rn(__fadd_rn(latn[j], lats[j]), 2.0f);
        olon[t] = (double)__fdiv_rn(__fadd_rn(lonw[i], lone[i]), 2.0f);
        oph[t] = (double)avg(0);
        olev[t] = k + 1;
        ovar[t] = var_of[n];
        oyo[t] = __dadd_rn((double)avg(n + 1), __ddiv_rn(z, __dsqrt_rn(rinv)));
        orinv[t] = rinv;
    }
}

unsigned blocks_for(int64_t work)
{
    const int64_t b = (work + kT - 1) / kT;
    return (unsigned)(b < 1 ? 1 : (b < 65536 ? b : 65536));
}

// Device copies of the inputs (host inputs go through ctx->d_raw).
int stage_floats(letkf_ctx *ctx, bool host, const std::vector<std::pair<const float *, int64_t>> &in,
                 std::vector<const float *> &out)
{
    out.clear();
    if (!host) {
        for (auto &a : in) out.push_back(a.first);
        return LETKF_OK;
    }
    int64_t total = 0;
    for (auto &a : in) total += a.first ? a.second : 0;
    if (ctx->d_raw.reserve((size_t)std::max<int64_t>(total, 1)) != cudaSuccess)
        return lg_set_err(ctx, LETKF_ERR_CUDA, "obs staging");
    int64_t at = 0;
    for (auto &a : in) {
        if (!a.first) {
            out.push_back(nullptr);
            continue;
        }
        if (cudaMemcpyAsync(ctx->d_raw.p + at, a.first, sizeof(float) * a.second, cudaMemcpyHostToDevice,
                            ctx->stream) != cudaSuccess)
            return lg_set_err(ctx, LETKF_ERR_CUDA, "obs staging copy");
        out.push_back(ctx->d_raw.p + at);
        at += a.second;
    }
    return LETKF_OK;
}

int reserve_out(letkf_ctx *ctx, int64_t m, int nvar, const int32_t *var_of)
{
    const size_t n = (size_t)std::max<int64_t>(m, 1);
    if (ctx->d_plat.reserve(n) || ctx->d_plon.reserve(n) || ctx->d_pph.reserve(n) || ctx->d_pyo.reserve(n) ||
        ctx->d_prinv.reserve(n) || ctx->d_plev.reserve(n) || ctx->d_pvar.reserve(n) ||
        ctx->d_pvarof.reserve((size_t)nvar))
        return lg_set_err(ctx, LETKF_ERR_CUDA, "obs buffers");
    for (int v = 0; v < nvar; v++)
        if (var_of[v] < 0 || var_of[v] >= ctx->nvar2d + ctx->nvar3d)
            return lg_set_err(ctx, LETKF_ERR_INVALID, "var_of names no state variable");
    if (cudaMemcpyAsync(ctx->d_pvarof.p, var_of, sizeof(int32_t) * nvar, cudaMemcpyHostToDevice, ctx->stream))
        return lg_set_err(ctx, LETKF_ERR_CUDA, "var_of copy");
    return LETKF_OK;
}

void fill_view(letkf_ctx *ctx, int64_t m, letkf_obs *obs)
{
    obs->nobs = m;
    obs->lat = ctx->d_plat.p;
    obs->lon = ctx->d_plon.p;
    obs->ph = ctx->d_pph.p;
    obs->lev = ctx->d_plev.p;
    obs->var = ctx->d_pvar.p;
    obs->yo = ctx->d_pyo.p;
    obs->rinv = ctx->d_prinv.p;
}

}  // namespace

extern "C" {

int letkf_gpu_obs_from_records(letkf_ctx *ctx, int64_t nrec, int nvar, int nz, const float *lon,
                               const float *lat, const float *lev, const float *val, const float *randn,
                               const int32_t *var_of, letkf_obs *obs, int flags)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (!obs || !var_of || nrec < 0 || nvar < 1 || nz < 1 || (nrec > 0 && (!lon || !lat || !lev || !val)) ||
        nrec % nz != 0 || (flags != LETKF_HOST_PTRS && flags != LETKF_DEVICE_PTRS))
        return lg_set_err(ctx, LETKF_ERR_INVALID, "bad record buffers");
    if (nrec * nvar >= (int64_t)INT32_MAX) return lg_set_err(ctx, LETKF_ERR_INVALID, "too many observations");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return lg_set_err(ctx, LETKF_ERR_CUDA, "cudaSetDevice");
    int rc = reserve_out(ctx, nrec * nvar, nvar, var_of);
    if (rc) return rc;
    std::vector<const float *> d;
    rc = stage_floats(ctx, flags == LETKF_HOST_PTRS,
                      {{lon, nrec}, {lat, nrec}, {lev, nrec}, {val, nrec * (2 * nvar + 1)}, {randn, nrec * nvar}}, d);
    if (rc) return rc;
    rc = lg_reset_status(ctx);
    if (rc) return rc;
    if (nrec > 0) {
        lg_count_launch();
        k_obs_records<<<blocks_for(nrec * nvar), kT, 0, ctx->stream>>>(
            nrec, nvar, nz, d[0], d[1], d[2], d[3], d[4], ctx->d_pvarof.p, ctx->d_plat.p, ctx->d_plon.p,
            ctx->d_pph.p, ctx->d_plev.p, ctx->d_pvar.p, ctx->d_pyo.p, ctx->d_prinv.p, ctx->d_status.p);
        if (cudaGetLastError() != cudaSuccess) return lg_set_err(ctx, LETKF_ERR_CUDA, "k_obs_records");
    }
    unsigned st = 0;
    unsigned long long cnt[LG_CNT_N];
    rc = lg_read_status(ctx, st, cnt);
    if (rc) return rc;
    if (st & LG_ST_BAD_OBS)
        return lg_set_err(ctx, LETKF_ERR_INVALID, "profile records must hold levels 1..nz in order");
    fill_view(ctx, nrec * nvar, obs);
    return LETKF_OK;
}

int letkf_gpu_obs_regular(letkf_ctx *ctx, int nlat_o, int nlon_o, int nz, int nvar, const float *latn,
                          const float *lats, const float *lonw, const float *lone, const float *r,
                          const float *nw, const float *sw, const float *ne, const float *se, const float *randn,
                          const int32_t *var_of, letkf_obs *obs, int flags)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (!obs || !var_of || nlat_o < 1 || nlon_o < 1 || nz < 1 || nvar < 1 || !latn || !lats || !lonw ||
        !lone || !r || !nw || !sw || !ne || !se || (flags != LETKF_HOST_PTRS && flags != LETKF_DEVICE_PTRS))
        return lg_set_err(ctx, LETKF_ERR_INVALID, "bad regular-grid buffers");
    const int64_t nobs = (int64_t)nlat_o * nlon_o, m = nobs * nz * nvar;
    if (m >= (int64_t)INT32_MAX) return lg_set_err(ctx, LETKF_ERR_INVALID, "too many observations");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return lg_set_err(ctx, LETKF_ERR_CUDA, "cudaSetDevice");
    int rc = reserve_out(ctx, m, nvar, var_of);
    if (rc) return rc;
    const int64_t corner = (int64_t)(nvar + 1) * nz * nobs;
    std::vector<const float *> d;
    rc = stage_floats(ctx, flags == LETKF_HOST_PTRS,
                      {{latn, nlat_o}, {lats, nlat_o}, {lonw, nlon_o}, {lone, nlon_o}, {r, (int64_t)nvar * nz},
                       {nw, corner}, {sw, corner}, {ne, corner}, {se, corner}, {randn, m}}, d);
    if (rc) return rc;
    lg_count_launch();
    k_obs_regular<<<blocks_for(m), kT, 0, ctx->stream>>>(nlat_o, nlon_o, nz, nvar, d[0], d[1], d[2], d[3], d[4],
                                                         d[5], d[6], d[7], d[8], d[9], ctx->d_pvarof.p,
                                                         ctx->d_plat.p, ctx->d_plon.p, ctx->d_pph.p, ctx->d_plev.p,
                                                         ctx->d_pvar.p, ctx->d_pyo.p, ctx->d_prinv.p);
    if (cudaGetLastError() != cudaSuccess) return lg_set_err(ctx, LETKF_ERR_CUDA, "k_obs_regular");
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return lg_set_err(ctx, LETKF_ERR_CUDA, "obs build");
    fill_view(ctx, m, obs);
    return LETKF_OK;
}

}  // extern "C"
