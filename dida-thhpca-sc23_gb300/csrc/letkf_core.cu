// letkf_core.cu -- FP64 per-cube LETKF core fused with the ensemble update.
//
// Reference: letkf_core (code/x86/TradDA/DA/LETKF/src/letkf_core.F90:14-233) and
// xb_2_xa (letkf_compute.F90:231-301), called per cube by
// letkf_compute_nooverlap (letkf_compute.F90:12-126).  One CTA per cube:
//
//   A' = (k-1)/rho I + Yhat Yhat^T,  Yhat = Y diag(sqrt(rdiaginv*rloc))
//        (lower-triangle 4x4 register tiles, obs rows staged in shared memory)
//   g  = Yhat (sqrt(rdiaginv*rloc) .* dep)
//   eigendecomposition of the SPD A' by one-sided (Hestenes) Jacobi on its
//        columns with a parallel round-robin pair ordering; for an SPD matrix
//        the converged columns are w_j = lambda_j v_j, so no separate
//        eigenvector matrix is kept
//   T  = sqrt(k-1) A'^(-1/2)   = sum_j sqrt((k-1)/lambda_j)/lambda_j^2 w_j w_j^T
//   wb = A'^(-1) g             = sum_j (w_j.g)/lambda_j^3 w_j
//   trans = T + wb 1^T         (letkf_core.F90:221-225)
//   xa = trans^T xb + axb, then the mean is recomputed and removed.
//
// The reference forms Pa and the k x p matrix Pa*Yhat^T (:129-195); the
// products here are the same quantities in O(k p + k^3) instead of O(k^2 p).
//
// Vertical localization (letkf_compute_nooverlap_vertical,
// letkf_compute.F90:358-526; gen_yb_dis_vertical and vertical_localization,
// letkf_yb.F90:137-243): per cube, every block of cube_nz levels solves its
// own problem with rloc = rloc_h * gc(|ln p_c - ln p_obs| / vert_dist), where
// ln p_c is the log of the block's centre-level pressure at the cube centre
// (ps2alnp, obs_make.F90:418-437, from the mean surface pressure), and
// updates only that block's rows (the 2-D variables with the last block).
// Overlapped cubes (letkf_compute and xb_add2_xa, letkf_compute.F90:128-228,
// 304-354): the core writes each cube's trans and k_overlap_update averages
// the updated columns over the cubes that cover them.
#include "letkf_internal.cuh"
#include "letkf_jacobi.cuh"

namespace {

constexpr int kT = LG_THREADS;

template <int K>
struct Cfg {
    static constexpr int KB = K / 4;
    static constexpr int NBLK = KB * (KB + 1) / 2;            // lower 4x4 blocks
    static constexpr int MB = (NBLK + kT - 1) / kT;            // blocks per thread
    static constexpr int NPAIR = K / 2;
    static constexpr int G = (NPAIR * 16 <= kT) ? 16 : (NPAIR * 8 <= kT) ? 8 : 4;  // threads per pair
    static constexpr int CH = (K <= 64) ? 64 : (K <= 96 ? 48 : 32);                // staged rows
    static constexpr int NO = (CH * K + kT - 1) / kT;          // update outputs per thread
    static constexpr size_t SMEM = sizeof(double) * (size_t)(K * K + CH * K + 5 * K + 2 * CH + K);
};

// Where the rows of a cube's local problem come from.
struct RowSrc {
    bool batch;
    // analysis run: global obs arrays + local lists
    const double *yb, *dep;
    const double *olnp;         // ln(ph) per obs (vertical localization) or null
    const float *rinvf;
    const int32_t *lidx;
    const double *lrloc;
    // batched core: packed per-problem rows
    const double *hx, *bdep, *brloc;
    const float *brdi;
};

// MEM: the fused members run (LgParams::members), a separate instantiation so
// the plain analysis keeps its registers.
template <int K, bool MEM = false>
__global__ void __launch_bounds__(kT)
k_core_fp64(LgGrid g, LgParams prm, RowSrc src, const int64_t *__restrict__ loff,
            const int32_t *__restrict__ lcnt, int64_t ncubes, const double *__restrict__ xb,
            const double *__restrict__ axb, double *__restrict__ xa, double *__restrict__ axa,
            double *__restrict__ trans_out, double *__restrict__ w_out,
            unsigned long long *__restrict__ counters, unsigned *__restrict__ status)
{
    using C = Cfg<K>;
    constexpr int MB = C::MB, CH = C::CH;
    extern __shared__ double sm[];
    double *W = sm;                    // K*K: A', Jacobi columns, then trans (row-major [i][e])
    double *S = W + K * K;             // CH*K staging
    double *gv = S + CH * K;           // K
    double *nrm = gv + K;              // K
    double *fco = nrm + K;             // K
    double *hco = fco + K;             // K
    double *wbar = hco + K;            // K
    double *sd = wbar + K;             // CH
    double *scl = sd + CH;             // CH
    double2 *rot = reinterpret_cast<double2 *>(scl + CH);   // K/2 rotations
    __shared__ int s_rot;

    const int tid = threadIdx.x;
    int bi[MB], bj[MB];
    bool bok[MB];
#pragma unroll
    for (int m = 0; m < MB; m++) {
        const int b = tid + m * kT;
        bok[m] = b < C::NBLK;
        lg_decode_block(bok[m] ? b : 0, bi[m], bj[m]);
    }

    // batched core: offsets flagged as bad by the counts pass before this
    // launch (same stream) stop every CTA before it reads a row
    if (src.batch && status && (*reinterpret_cast<volatile const unsigned *>(status) & LG_ST_BAD_OBS)) return;
    const bool vertical = !src.batch && src.olnp != nullptr;
    const int nvb = vertical ? (g.nz + prm.cube_nz - 1) / prm.cube_nz : 1;
    for (int64_t cube = prm.cube0 + blockIdx.x; cube < ncubes; cube += gridDim.x) {
        const int64_t off = loff[cube];
        const int p = lcnt[cube];
        const int bjc = (int)(cube % prm.nbj), bic = (int)(cube / prm.nbj);
        const int sj = bjc * prm.cube_step, ej = min(sj + prm.cube_n - 1, g.nlat - 1);
        const int si = bic * prm.cube_step, ei = min(si + prm.cube_n - 1, g.nlon - 1);
        for (int vb = 0; vb < nvb; vb++) {
        // vertical block vb: levels sk..ek, centre level ck; ln p of the
        // centre level at the cube centre from the mean surface pressure
        const int sk = vb * prm.cube_nz, ek = min(sk + prm.cube_nz - 1, g.nz - 1);
        double alnp = 0.0;
        if (vertical) {
            const int ck = ((sk + 1) + (ek + 1)) / 2 - 1;
            const int cj = ((sj + 1) + (ej + 1)) / 2 - 1, ci = ((si + 1) + (ei + 1)) / 2 - 1;
            const double ps = axb[(cj + (int64_t)g.nlat * ci) * g.n + g.ps_row];
            const double pt = g.ptop, dp = g.p0 - g.ptop;
            const double p_lo = g.hyai[ck] * dp + g.hybi[ck] * (ps - pt) + pt;
            const double p_hi = g.hyai[ck + 1] * dp + g.hybi[ck + 1] * (ps - pt) + pt;
            alnp = log(0.5 * (p_lo + p_hi));
        }

        // ---- A = Yhat Yhat^T (lower blocks), g = Yhat (s .* dep)
        double acc[MB][16];
#pragma unroll
        for (int m = 0; m < MB; m++)
#pragma unroll
            for (int i = 0; i < 16; i++) acc[m][i] = 0.0;
        double gacc = 0.0;
        for (int s0 = 0; s0 < p; s0 += CH) {
            const int cnt = min(CH, p - s0);
            if (tid < cnt) {
                const int64_t li = off + s0 + tid;
                double rdi, rl, d;
                if (src.batch) {
                    rdi = (double)src.brdi[li];
                    rl = src.brloc[li];
                    d = src.bdep[li];
                } else {
                    const int gi = src.lidx[li];
                    rdi = (double)src.rinvf[gi];
                    rl = src.lrloc[li];
                    d = src.dep[gi];
                    if (vertical) {
                        const double z = fabs(alnp - src.olnp[gi]) / prm.vert_dist;
                        rl = rl * (prm.gc_filter_vertical ? lg_schr2(z) : lg_schr(z));
                    }
                }
                const double sc = sqrt(rdi * rl);     // rrloc (letkf_core.F90:64-66)
                scl[tid] = sc;
                sd[tid] = sc * d;
            }
            __syncthreads();
            for (int idx = tid; idx < cnt * K; idx += kT) {
                const int o = idx / K, e = idx - o * K;
                const int64_t li = off + s0 + o;
                const double *row = src.batch ? src.hx + li * K : src.yb + (int64_t)src.lidx[li] * K;
                S[o * K + e] = row[e] * scl[o];
            }
            __syncthreads();
            if (tid < K)
                for (int o = 0; o < cnt; o++) gacc += S[o * K + tid] * sd[o];
            for (int o = 0; o < cnt; o++) {
                const double *ro = S + o * K;
#pragma unroll
                for (int m = 0; m < MB; m++) {
                    if (!bok[m]) continue;
                    const double2 a01 = *reinterpret_cast<const double2 *>(ro + 4 * bi[m]);
                    const double2 a23 = *reinterpret_cast<const double2 *>(ro + 4 * bi[m] + 2);
                    const double2 b01 = *reinterpret_cast<const double2 *>(ro + 4 * bj[m]);
                    const double2 b23 = *reinterpret_cast<const double2 *>(ro + 4 * bj[m] + 2);
                    const double a[4] = {a01.x, a01.y, a23.x, a23.y};
                    const double b[4] = {b01.x, b01.y, b23.x, b23.y};
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[m][i * 4 + j] += a[i] * b[j];
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int m = 0; m < MB; m++) {
            if (!bok[m]) continue;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = 4 * bi[m] + i, c = 4 * bj[m] + j;
                    W[c * K + r] = acc[m][i * 4 + j];
                    W[r * K + c] = acc[m][i * 4 + j];
                }
        }
        if (tid < K) gv[tid] = gacc;
        __syncthreads();
        if (tid < K) W[tid * K + tid] += (double)(K - 1) / prm.inflation;
        __syncthreads();

        // ---- eigendecomposition of A'
        const int sweeps = lg_jacobi<double, K, Cfg<K>::G>(W, nrm, rot, &s_rot, 1e-15, 40);
        if (tid == 0) {
            atomicMax(&counters[LG_CNT_MAXSWEEP], (unsigned long long)sweeps);
            atomicAdd(&counters[LG_CNT_SUMSWEEP], (unsigned long long)sweeps);
            if (sweeps > 40) {
                atomicAdd(&counters[LG_CNT_NOTCONV], 1ull);
                atomicOr(status, LG_ST_NOT_CONV);
            }
        }
        if (tid < K) {
            double s = 0.0, dot = 0.0;
            for (int r = 0; r < K; r++) {
                const double wv = W[tid * K + r];
                s += wv * wv;
                dot += wv * gv[r];
            }
            const double lam = sqrt(s);
            fco[tid] = sqrt((double)(K - 1) / lam) / (lam * lam);
            hco[tid] = dot / (lam * lam * lam);
        }
        __syncthreads();
        if (tid < K) {
            double s = 0.0;
            for (int j = 0; j < K; j++) s += hco[j] * W[j * K + tid];
            wbar[tid] = s;
        }
        // ---- T = sum_j f_j w_j w_j^T (lower blocks)
#pragma unroll
        for (int m = 0; m < MB; m++)
#pragma unroll
            for (int i = 0; i < 16; i++) acc[m][i] = 0.0;
        for (int j = 0; j < K; j++) {
            const double *wj = W + j * K;
            const double f = fco[j];
#pragma unroll
            for (int m = 0; m < MB; m++) {
                if (!bok[m]) continue;
                const double2 a01 = *reinterpret_cast<const double2 *>(wj + 4 * bi[m]);
                const double2 a23 = *reinterpret_cast<const double2 *>(wj + 4 * bi[m] + 2);
                const double2 b01 = *reinterpret_cast<const double2 *>(wj + 4 * bj[m]);
                const double2 b23 = *reinterpret_cast<const double2 *>(wj + 4 * bj[m] + 2);
                const double a[4] = {a01.x, a01.y, a23.x, a23.y};
                const double b[4] = {b01.x * f, b01.y * f, b23.x * f, b23.y * f};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) acc[m][i * 4 + jj] += a[i] * b[jj];
            }
        }
        __syncthreads();
        // trans(i, e) = T(i, e) + wbar(i), stored row-major Tr[i*K + e]
#pragma unroll
        for (int m = 0; m < MB; m++) {
            if (!bok[m]) continue;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = 4 * bi[m] + i, c = 4 * bj[m] + j;
                    const double v = acc[m][i * 4 + j];
                    W[r * K + c] = v + wbar[r];
                    W[c * K + r] = v + wbar[c];
                }
        }
        __syncthreads();
        if (trans_out) {
            for (int idx = tid; idx < K * K; idx += kT) {
                const int i = idx % K, j = idx / K;       // column-major (i, j)
                trans_out[cube * K * K + idx] = W[i * K + j];
            }
            if (tid < K) w_out[cube * K + tid] = wbar[tid];
        }
        if (xb == nullptr) {
            __syncthreads();
            continue;
        }

        // ---- xa = trans^T xb + axb for every column of the cube, then mean removal
        // (vertical blocks: the rows of the block's levels of each 3-D
        // variable, and the 2-D variables with the last block)
        const int n = g.n;
        const int nruns = vertical ? g.nvar2d + g.nvar3d : 1;
        for (int ii = si; ii <= ei; ii++)
            for (int jj = sj; jj <= ej; jj++) {
                const int64_t c = jj + (int64_t)g.nlat * ii;
                const double *xbc = xb + c * n * K;
                double *xac = xa + c * n * K;
                for (int run = 0; run < nruns; run++) {
                int rs = 0, re = n - 1;
                if (vertical) {
                    if (run < g.nvar2d) {
                        if (ek != g.nz - 1) continue;
                        rs = re = run;
                    } else {
                        rs = g.nvar2d + (run - g.nvar2d) * g.nz + sk;
                        re = g.nvar2d + (run - g.nvar2d) * g.nz + ek;
                    }
                }
                for (int r0 = rs; r0 <= re; r0 += CH) {
                    const int R = min(CH, re - r0 + 1);
                    for (int idx = tid; idx < R * K; idx += kT) S[idx] = xbc[(int64_t)r0 * K + idx];
                    __syncthreads();
                    if constexpr (MEM) {
                        // full members in: the row's mean (sum / real(ens),
                        // module_da_parallel.F90:194-199) into scl, the sum of
                        // squared perturbations into hco, perturbations into S
                        if (tid < R) {
                            const double fk = (double)(float)K;
                            double s = 0.0;
                            bool bad = false;
                            for (int e = 0; e < K; e++) {
                                s += S[tid * K + e];
                                bad |= isnan(S[tid * K + e]);
                            }
                            if (bad) atomicOr(status, LG_ST_BAD_STATE);
                            const double mb = s / fk;
                            double q2 = 0.0;
                            for (int e = 0; e < K; e++) {
                                const double d = S[tid * K + e] - mb;
                                q2 += d * d;
                            }
                            scl[tid] = mb;
                            hco[tid] = q2;
                        }
                        __syncthreads();
                        for (int idx = tid; idx < R * K; idx += kT) S[idx] -= scl[idx / K];
                        __syncthreads();
                    }
                    double out[C::NO];
#pragma unroll
                    for (int q = 0; q < C::NO; q++) {
                        const int idx = tid + q * kT;
                        out[q] = 0.0;
                        if (idx < R * K) {
                            const int rl = idx / K, e = idx - rl * K;
                            const double *xr = S + rl * K;
                            double a = 0.0;
#pragma unroll 8
                            for (int i = 0; i < K; i++) a += W[i * K + e] * xr[i];
                            out[q] = a + (MEM ? scl[rl] : axb[c * n + r0 + rl]);
                        }
                    }
                    __syncthreads();
#pragma unroll
                    for (int q = 0; q < C::NO; q++) {
                        const int idx = tid + q * kT;
                        if (idx < R * K) S[idx] = out[q];
                    }
                    __syncthreads();
                    if (tid < R) {
                        double m = 0.0;
                        for (int e = 0; e < K; e++) m += S[tid * K + e];
                        m = m / K;
                        sd[tid] = m;
                        if (!MEM) axa[c * n + r0 + tid] = m;
                    }
                    __syncthreads();
                    if constexpr (!MEM) {
                        for (int idx = tid; idx < R * K; idx += kT)
                            xac[(int64_t)r0 * K + idx] = S[idx] - sd[idx / K];
                    } else {
                        // letkf2dnn (module_da_parallel.F90:214-258): the
                        // blend, or the background where |lat| > polar, into
                        // the member array; S keeps what the analysis spread sums
                        const bool blend = fabs((double)g.glat[c % g.nlat]) <= prm.polar;
                        for (int idx = tid; idx < R * K; idx += kT) {
                            const int rl = idx / K;
                            const double mb = scl[rl], ma = sd[rl];
                            const double b = xbc[(int64_t)r0 * K + idx] - mb;
                            double o;
                            if (blend) {
                                o = prm.gamma1 * (mb + b) + prm.gamma2 * (ma + (S[idx] - ma));
                                S[idx] = o - ma;
                            } else {
                                o = b + mb;
                                S[idx] = b;
                            }
                            xac[(int64_t)r0 * K + idx] = o;
                        }
                        __syncthreads();
                        if (tid < R) {
                            const double fk = (double)(float)K;
                            double q2 = 0.0;
                            for (int e = 0; e < K; e++) q2 += S[tid * K + e] * S[tid * K + e];
                            prm.spb[c * n + r0 + tid] = sqrt(hco[tid] / fk);
                            prm.spa[c * n + r0 + tid] = sqrt(q2 / fk);
                        }
                    }
                    __syncthreads();
                }
                }
            }
        }
    }
}

// Overlapped cubes (xb_add2_xa, letkf_compute.F90:304-354, and the final
// division by the cover count, :206-226): per column, over the cubes that
// cover it in the reference's loop order (longitude start outer, latitude
// start inner): dist = axb + xb^T trans, xa += dist - mean(dist),
// axa += mean(dist); then xa and axa are divided by the number of cubes.
// One CTA per column; trans (with w, column-major) is staged in shared
// memory row-major with a padded stride; warps take rows, lanes members.
template <int K>
__global__ void __launch_bounds__(kT)
k_overlap_update(LgGrid g, LgParams prm, const double *__restrict__ trans, const double *__restrict__ xb,
                 const double *__restrict__ axb, double *__restrict__ xa, double *__restrict__ axa)
{
    extern __shared__ double Ts[];               // Ts[l * (K + 1) + e] = trans(l, e)
    constexpr int LDT = K + 1, PER = (K + 31) / 32;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = g.n, step = prm.cube_step, cn = prm.cube_n;
    const int64_t ncol = (int64_t)g.nlat * g.nlon;
    for (int64_t c = blockIdx.x; c < ncol; c += gridDim.x) {
        const int jj = (int)(c % g.nlat), ii = (int)(c / g.nlat);
        for (int idx = tid; idx < n * K; idx += kT) xa[c * n * K + idx] = 0.0;
        for (int r = tid; r < n; r += kT) axa[c * n + r] = 0.0;
        // cube starts i0 (j0) are multiples of step with i0 <= ii <= i0 + cube_n - 1
        const int i_lo = max(0, (ii - cn + 1 + step - 1) / step), i_hi = ii / step;
        const int j_lo = max(0, (jj - cn + 1 + step - 1) / step), j_hi = jj / step;
        int count = 0;
        for (int bi = i_lo; bi <= i_hi; bi++)
            for (int bj = j_lo; bj <= j_hi; bj++) {
                const int64_t cube = bj + (int64_t)prm.nbj * bi;
                __syncthreads();
                for (int idx = tid; idx < K * K; idx += kT) {
                    const int l = idx % K, e = idx / K;
                    Ts[l * LDT + e] = trans[cube * K * K + idx];
                }
                __syncthreads();
                for (int r = warp; r < n; r += kT / 32) {
                    const double *x = xb + (c * n + r) * K;
                    const double ab = axb[c * n + r];
                    double dist[PER];
                    double sum = 0.0;
#pragma unroll
                    for (int q = 0; q < PER; q++) {
                        const int e = lane + 32 * q;
                        double s = 0.0;
                        if (e < K)
                            for (int l = 0; l < K; l++) s += x[l] * Ts[l * LDT + e];
                        dist[q] = ab + s;
                        if (e < K) sum += dist[q];
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                    const double mean = sum / K;
#pragma unroll
                    for (int q = 0; q < PER; q++) {
                        const int e = lane + 32 * q;
                        if (e < K) xa[(c * n + r) * K + e] += dist[q] - mean;
                    }
                    if (lane == 0) axa[c * n + r] += mean;
                }
                count++;
            }
        __syncthreads();
        const double cnt = (double)count;
        for (int idx = tid; idx < n * K; idx += kT) xa[c * n * K + idx] = xa[c * n * K + idx] / cnt;
        for (int r = tid; r < n; r += kT) axa[c * n + r] = axa[c * n + r] / cnt;
        __syncthreads();
    }
}

template <int K>
cudaError_t launch_overlap(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb, double *xa,
                           double *axa)
{
    const size_t smem = sizeof(double) * (size_t)K * (K + 1);
    cudaError_t e = cudaFuncSetAttribute(k_overlap_update<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t ncol = (int64_t)g.nlat * g.nlon;
    const unsigned blocks = (unsigned)(ncol < (1 << 30) ? ncol : (1 << 30));
    lg_count_launch();
    k_overlap_update<K><<<blocks, kT, smem, ctx->stream>>>(g, lg_params(ctx), ctx->d_trans.p, xb, axb, xa, axa);
    return cudaGetLastError();
}

__global__ void k_obs_lnp(int64_t nobs, const double *__restrict__ oph, double *__restrict__ olnp)
{
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nobs; o += (int64_t)gridDim.x * blockDim.x)
        olnp[o] = log(oph[o]);
}

template <int K>
cudaError_t launch_k(letkf_ctx *ctx, const LgGrid &g, const RowSrc &src, const int64_t *loff,
                     const int32_t *lcnt, int64_t cube0, int64_t ncubes, const double *xb, const double *axb,
                     double *xa, double *axa, double *trans_out, double *w_out)
{
    const size_t smem = Cfg<K>::SMEM;
    LgParams prm = lg_params(ctx);
    prm.cube0 = cube0;
    auto kern = prm.members ? k_core_fp64<K, true> : k_core_fp64<K, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (ncubes <= cube0) return cudaSuccess;
    const int64_t nwin = ncubes - cube0;
    const unsigned blocks = (unsigned)(nwin < (1 << 30) ? nwin : (1 << 30));
    lg_count_launch();
    kern<<<blocks, kT, smem, ctx->stream>>>(g, prm, src, loff, lcnt, ncubes, xb, axb, xa, axa, trans_out, w_out,
                                            ctx->d_counters.p, ctx->d_status.p);
    return cudaGetLastError();
}

cudaError_t dispatch(letkf_ctx *ctx, const LgGrid &g, const RowSrc &src, const int64_t *loff,
                     const int32_t *lcnt, int64_t cube0, int64_t ncubes, const double *xb, const double *axb,
                     double *xa, double *axa, double *trans_out, double *w_out)
{
    switch (g.k) {
    case 32: return launch_k<32>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    case 48: return launch_k<48>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    case 64: return launch_k<64>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    case 96: return launch_k<96>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    case 128: return launch_k<128>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    case 4: return launch_k<4>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    case 8: return launch_k<8>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    case 16: return launch_k<16>(ctx, g, src, loff, lcnt, cube0, ncubes, xb, axb, xa, axa, trans_out, w_out);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool lg_core_supports(int k)
{
    return k == 4 || k == 8 || k == 16 || k == 32 || k == 48 || k == 64 || k == 96 || k == 128;
}

cudaError_t lg_launch_core_fp64(letkf_ctx *ctx, const LgGrid &g, const double *xb,
                                const double *axb, double *xa, double *axa, bool keep_trans)
{
    RowSrc src{};
    src.batch = false;
    src.yb = ctx->d_yb.p;
    src.dep = ctx->d_dep.p;
    src.rinvf = ctx->d_rinvf.p;
    src.lidx = ctx->d_lidx.p;
    src.lrloc = ctx->d_lrloc.p;
    src.olnp = (ctx->params.overlap == 0 && ctx->params.vert_dist > 0.0) ? ctx->d_olnp.p : nullptr;
    return dispatch(ctx, g, src, ctx->d_loff.p, ctx->d_lcnt.p, ctx->win0, ctx->win1, xb, axb, xa, axa,
                    keep_trans ? ctx->d_trans.p : nullptr, keep_trans ? ctx->d_w.p : nullptr);
}

cudaError_t lg_launch_overlap_update(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb,
                                     double *xa, double *axa)
{
    switch (g.k) {
    case 4: return launch_overlap<4>(ctx, g, xb, axb, xa, axa);
    case 8: return launch_overlap<8>(ctx, g, xb, axb, xa, axa);
    case 16: return launch_overlap<16>(ctx, g, xb, axb, xa, axa);
    case 32: return launch_overlap<32>(ctx, g, xb, axb, xa, axa);
    case 48: return launch_overlap<48>(ctx, g, xb, axb, xa, axa);
    case 64: return launch_overlap<64>(ctx, g, xb, axb, xa, axa);
    case 96: return launch_overlap<96>(ctx, g, xb, axb, xa, axa);
    case 128: return launch_overlap<128>(ctx, g, xb, axb, xa, axa);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t lg_launch_obs_lnp(letkf_ctx *ctx, int64_t nobs, const double *oph)
{
    if (nobs <= 0) return cudaSuccess;
    const int64_t want = (nobs + 255) / 256;
    const unsigned blocks = (unsigned)(want < 4096 ? want : 4096);
    lg_count_launch();
    k_obs_lnp<<<blocks, 256, 0, ctx->stream>>>(nobs, oph, ctx->d_olnp.p);
    return cudaGetLastError();
}

cudaError_t lg_launch_core_batch_fp64(letkf_ctx *ctx, int64_t nb, const int64_t *d_off,
                                      const double *d_hx, const float *d_rdi,
                                      const double *d_dep, const double *d_rloc,
                                      double *d_trans, double *d_w)
{
    RowSrc src{};
    src.batch = true;
    src.hx = d_hx;
    src.brdi = d_rdi;
    src.bdep = d_dep;
    src.brloc = d_rloc;
    LgGrid g = lg_grid(ctx);
    return dispatch(ctx, g, src, d_off, ctx->d_lcnt.p, 0, nb, nullptr, nullptr, nullptr, nullptr,
                    d_trans, d_w);
}

// Launch of the batched core with every buffer supplied by the caller
// (letkf_noalloc.cu): problem b uses rows d_off[b] .. d_off[b] + d_cnt[b] - 1.
namespace {
template <int K>
cudaError_t launch_raw(double inflation, int64_t nb, const int64_t *d_off, const int32_t *d_cnt,
                       const RowSrc &src, double *d_trans, double *d_w,
                       unsigned long long *counters, unsigned *status, cudaStream_t stream)
{
    const size_t smem = Cfg<K>::SMEM;
    cudaError_t e = cudaFuncSetAttribute(k_core_fp64<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    LgGrid g{};
    g.k = K;
    LgParams prm{};
    prm.inflation = inflation;
    prm.nbj = 1;
    prm.cube_n = 1;
    const unsigned blocks = (unsigned)(nb < (1 << 30) ? nb : (1 << 30));
    lg_count_launch();
    k_core_fp64<K><<<blocks, kT, smem, stream>>>(g, prm, src, d_off, d_cnt, nb, nullptr, nullptr,
                                                 nullptr, nullptr, d_trans, d_w, counters, status);
    return cudaGetLastError();
}
}  // namespace

cudaError_t lg_launch_core_batch_raw(int k, double inflation, int64_t nb, const int64_t *d_off,
                                     const int32_t *d_cnt, const double *d_hx, const float *d_rdi,
                                     const double *d_dep, const double *d_rloc, double *d_trans,
                                     double *d_w, unsigned long long *counters, unsigned *status,
                                     cudaStream_t stream)
{
    RowSrc src{};
    src.batch = true;
    src.hx = d_hx;
    src.brdi = d_rdi;
    src.bdep = d_dep;
    src.brloc = d_rloc;
    switch (k) {
    case 4: return launch_raw<4>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    case 8: return launch_raw<8>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    case 16: return launch_raw<16>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    case 32: return launch_raw<32>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    case 48: return launch_raw<48>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    case 64: return launch_raw<64>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    case 96: return launch_raw<96>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    case 128: return launch_raw<128>(inflation, nb, d_off, d_cnt, src, d_trans, d_w, counters, status, stream);
    default: return cudaErrorInvalidValue;
    }
}
