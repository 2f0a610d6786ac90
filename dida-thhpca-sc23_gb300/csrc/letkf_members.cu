// letkf_members.cu -- the caller's conversion around letkf_run on the device.
//
// Reference: run_da_parallel (code/x86/TradDA/DA/EnDNN/src/module_da_parallel.F90:163-261)
// hands letkf_run the ensemble as mean and perturbations (dnn2letkf, :184-204)
// and turns the analysis back into full members with the relaxation-to-prior
// blend and the background and analysis spreads (letkf2dnn, :214-258).
// letkf_gpu_run_members runs the three steps on the GPU, so full members go in
// and full members and spreads come out without a host pass over the state.
// With one column per cube, no overlap and no vertical blocks (and k <= 64 in
// the mixed forms) the steps are fused into the analysis (LgParams::members):
// H reads the members as they are, and the update kernels form each row's
// mean and perturbations as they read the row and write the blended members
// and both spreads, so no pass over the state is added.  Otherwise:
//   k_members_split: per state row, the mean over members (sum / real(ens))
//       and the perturbations; a NaN member stops the run (the reference
//       prints and stops, :188-193);
//   the analysis of letkf_gpu_run on the split state;
//   k_members_blend: where |grid_lat| <= polar_lat,
//       xout = gamma1 (axb + xb) + gamma2 (axa + xa),
//       spread_b = sqrt(sum xb^2 / ens), spread_a = sqrt(sum (xout - axa)^2 / ens);
//       elsewhere the background passes through (xout = xb + axb) and both
//       spreads are the background's.
// One warp per state row: lanes over members, shuffle sums.
#include <cmath>

#include "letkf_internal.cuh"

namespace {

constexpr int kT = 256;

__global__ void __launch_bounds__(kT)
k_members_split(int64_t nrows, int k, const double *__restrict__ xin, double *__restrict__ xb,
                double *__restrict__ axb, unsigned *__restrict__ status)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (kT / 32);
    const double fk = (double)(float)k;    // real(ens)
    for (int64_t r = blockIdx.x * (int64_t)(kT / 32) + (threadIdx.x >> 5); r < nrows; r += warps) {
        const double *x = xin + r * k;
        double s = 0.0;
        bool bad = false;
        for (int e = lane; e < k; e += 32) {
            const double v = x[e];
            bad |= isnan(v);
            s += v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(status, LG_ST_BAD_STATE);
        const double m = s / fk;
        if (lane == 0) axb[r] = m;
        for (int e = lane; e < k; e += 32) xb[r * k + e] = x[e] - m;
    }
}

__global__ void __launch_bounds__(kT)
k_members_blend(int nlat, int n, int64_t nrows, int k, double gamma1, double gamma2, double polar,
                const float *__restrict__ glat, const double *__restrict__ xb, const double *__restrict__ axb,
                const double *xa, const double *__restrict__ axa, double *xout, double *__restrict__ spread_b,
                double *__restrict__ spread_a)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (kT / 32);
    const double fk = (double)(float)k;
    for (int64_t r = blockIdx.x * (int64_t)(kT / 32) + (threadIdx.x >> 5); r < nrows; r += warps) {
        const int64_t col = r / n;
        const double lat = (double)glat[col % nlat];
        const bool blend = fabs(lat) <= polar;
        const double ab = axb[r], aa = axa[r];
        double sb = 0.0, sa = 0.0;
        for (int e = lane; e < k; e += 32) {
            const double b = xb[r * k + e];
            // xout may be xa itself: each lane reads its member before writing it
            double o;
            if (blend) {
                o = __dadd_rn(__dmul_rn(gamma1, __dadd_rn(ab, b)), __dmul_rn(gamma2, __dadd_rn(aa, xa[r * k + e])));
                const double d = __dsub_rn(o, aa);
                sa = __dadd_rn(sa, __dmul_rn(d, d));
            } else {
                o = __dadd_rn(b, ab);
                sa = __dadd_rn(sa, __dmul_rn(b, b));
            }
            sb = __dadd_rn(sb, __dmul_rn(b, b));
            xout[r * k + e] = o;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sb += __shfl_xor_sync(0xffffffffu, sb, o);
            sa += __shfl_xor_sync(0xffffffffu, sa, o);
        }
        if (lane == 0) {
            spread_b[r] = sqrt(sb / fk);
            spread_a[r] = sqrt(sa / fk);
        }
    }
}

unsigned grid_for(int64_t nrows)
{
    const int64_t want = (nrows + kT / 32 - 1) / (kT / 32);
    return (unsigned)(want < (1 << 20) ? want : (1 << 20));
}

}  // namespace

extern "C" int letkf_gpu_run_members(letkf_ctx *ctx, const double *xb_in, const letkf_obs *obs,
                                     const letkf_blend *blend, double *xa_out, double *spread_b,
                                     double *spread_a, int flags)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (!xb_in || !xa_out || !spread_b || !spread_a || !blend)
        return lg_set_err(ctx, LETKF_ERR_INVALID, "NULL pointer");
    if (flags != LETKF_HOST_PTRS && flags != LETKF_DEVICE_PTRS) return lg_set_err(ctx, LETKF_ERR_INVALID, "bad flags");
    if (ctx->range0 != 0 || ctx->range1 != ctx->ncubes)
        return lg_set_err(ctx, LETKF_ERR_UNSUPPORTED, "the members entry point analyses every cube");
    int rc = lg_check_run(ctx, obs);
    if (rc) return rc;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return lg_set_err(ctx, LETKF_ERR_CUDA, "cudaSetDevice");
    const bool host = flags == LETKF_HOST_PTRS;
    const int k = ctx->k, n = ctx->n;
    const int64_t nrows = ctx->ncol * n;
    const size_t nstate = (size_t)nrows * k, nmean = (size_t)nrows;
    auto cu = [&](cudaError_t e) { return e == cudaSuccess ? LETKF_OK : lg_set_err(ctx, LETKF_ERR_CUDA, cudaGetErrorString(e)); };
#define LG_TRY(x)                     \
    do {                              \
        const int rc_ = cu(x);        \
        if (rc_) return rc_;          \
    } while (0)
    LG_TRY(cudaEventRecord(ctx->ev[0], ctx->stream));
    rc = lg_reset_status(ctx);
    if (rc) return rc;
    // The split and the blend fused into the analysis (H reads the members as
    // they are, the update forms each row's mean and perturbations as it reads
    // it and writes the blended members and both spreads): no state pass of
    // its own.  Kept as separate passes where the update is not one pass over
    // one column per cube (overlapped cubes, vertical blocks) and for the
    // mixed form's wide core (k = 96, 128).
    const bool fused = ctx->params.cube_n == 1 && ctx->params.overlap == 0 && !(ctx->params.vert_dist > 0.0) &&
                       !(lg_is_mixed(ctx->params.precision) && k > 64);
    if (fused) {
        LG_TRY(ctx->d_spb.reserve(nmean));
        LG_TRY(ctx->d_spa.reserve(nmean));
        const double *din = xb_in;
        double *dout = xa_out, *dsb = spread_b, *dsa = spread_a;
        if (host) {
            LG_TRY(ctx->d_xb.reserve(nstate));
            LG_TRY(ctx->d_xa.reserve(nstate));
            LG_TRY(cudaMemcpyAsync(ctx->d_xb.p, xb_in, sizeof(double) * nstate, cudaMemcpyHostToDevice, ctx->stream));
            din = ctx->d_xb.p;
            dout = ctx->d_xa.p;
            dsb = ctx->d_spb.p;
            dsa = ctx->d_spa.p;
        }
        ctx->members_on = true;
        ctx->members_g1 = blend->gamma1;
        ctx->members_g2 = blend->gamma2;
        ctx->members_polar = blend->polar_lat_deg;
        ctx->members_spb = dsb;
        ctx->members_spa = dsa;
        unsigned long long cnt[LG_CNT_N] = {};
        rc = lg_run_analysis(ctx, obs, host, din, nullptr, dout, nullptr, cnt);
        ctx->members_on = false;
        ctx->members_spb = ctx->members_spa = nullptr;
        if (rc) return rc;
        if (host) {
            LG_TRY(cudaMemcpyAsync(xa_out, dout, sizeof(double) * nstate, cudaMemcpyDeviceToHost, ctx->stream));
            LG_TRY(cudaMemcpyAsync(spread_b, dsb, sizeof(double) * nmean, cudaMemcpyDeviceToHost, ctx->stream));
            LG_TRY(cudaMemcpyAsync(spread_a, dsa, sizeof(double) * nmean, cudaMemcpyDeviceToHost, ctx->stream));
        }
        return lg_finish_run(ctx, obs, cnt);
    }
    LG_TRY(ctx->d_xb.reserve(nstate));
    LG_TRY(ctx->d_axb.reserve(nmean));
    LG_TRY(ctx->d_xa.reserve(nstate));
    LG_TRY(ctx->d_axa.reserve(nmean));
    const double *din = xb_in;
    if (host) {
        // the analysis perturbations are written to d_xa only after the split
        LG_TRY(cudaMemcpyAsync(ctx->d_xa.p, xb_in, sizeof(double) * nstate, cudaMemcpyHostToDevice, ctx->stream));
        din = ctx->d_xa.p;
    }
    lg_count_launch();
    k_members_split<<<grid_for(nrows), kT, 0, ctx->stream>>>(nrows, k, din, ctx->d_xb.p, ctx->d_axb.p,
                                                             ctx->d_status.p);
    LG_TRY(cudaGetLastError());
    unsigned long long cnt[LG_CNT_N] = {};
    unsigned st = 0;
    rc = lg_read_status(ctx, st, cnt);
    if (rc) return rc;
    if (st & LG_ST_BAD_STATE) return lg_set_err(ctx, LETKF_ERR_INVALID, "a background member is NaN");
    rc = lg_run_analysis(ctx, obs, host, ctx->d_xb.p, ctx->d_axb.p, ctx->d_xa.p, ctx->d_axa.p, cnt);
    if (rc) return rc;
    double *dout = xa_out, *dsb = spread_b, *dsa = spread_a;
    if (host) {
        LG_TRY(ctx->d_spb.reserve(nmean));
        LG_TRY(ctx->d_spa.reserve(nmean));
        dout = ctx->d_xa.p;          // blended in place
        dsb = ctx->d_spb.p;
        dsa = ctx->d_spa.p;
    }
    lg_count_launch();
    k_members_blend<<<grid_for(nrows), kT, 0, ctx->stream>>>(
        ctx->nlat, n, nrows, k, blend->gamma1, blend->gamma2, blend->polar_lat_deg, ctx->d_glat.p, ctx->d_xb.p,
        ctx->d_axb.p, ctx->d_xa.p, ctx->d_axa.p, dout, dsb, dsa);
    LG_TRY(cudaGetLastError());
    if (host) {
        LG_TRY(cudaMemcpyAsync(xa_out, dout, sizeof(double) * nstate, cudaMemcpyDeviceToHost, ctx->stream));
        LG_TRY(cudaMemcpyAsync(spread_b, dsb, sizeof(double) * nmean, cudaMemcpyDeviceToHost, ctx->stream));
        LG_TRY(cudaMemcpyAsync(spread_a, dsa, sizeof(double) * nmean, cudaMemcpyDeviceToHost, ctx->stream));
    }
#undef LG_TRY
    return lg_finish_run(ctx, obs, cnt);
}
