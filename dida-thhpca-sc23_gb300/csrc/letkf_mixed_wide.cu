// letkf_mixed_wide.cu -- mixed-precision per-cube LETKF core for k = 96 and 128.
//
// The same analysis and precision choices as k_core_mixed (letkf_mixed.cu;
// letkf_core, code/x86/TradDA/DA/LETKF/src/letkf_core.F90:14-233, and
// xb_2_xa, letkf_compute.F90:231-301) for ensembles whose stacked hi/lo rows
// (2k) do not fit one MMA's 128 rows.  Differences of layout:
//   * A: the tile holds Yhat_lo in rows 0..k-1 (zero to 127) and Yhat_hi
//     from row 128; two MMAs per K step, lo x hi and hi x hi (N = k),
//     accumulate into two TMEM ranges (columns 0 and 256 of a 512-column
//     allocation: one CTA per SM); g and the diagonal of A are summed on the
//     FP32 pipe by the conversion threads, as in the narrow core;
//   * A = 0.5 (S + S^T) with S = HH + 2 LH staged once (no FP64 copy of A':
//     the w-bar residual adds (k-1)/rho in FP64 to the FP32 A);
//   * the update's operands (xb rows and T, k members deep) are two
//     128-byte-swizzled tiles along the member axis.
// The FP32 Jacobi takes the hierarchical ordering over blocks of two columns
// (k = 128, lg_jacobi32b2) or three (k = 96, lg_jacobi32b3).
// Shared memory (k = 128): the previous cube's eigenvectors and X (64 KB),
// the Jacobi columns / S / T tiles (67 KB), A / T / xb tiles (65 KB); the
// A-build tiles and gather stages overlay the last two.
#include "letkf_internal.cuh"
#include "letkf_jacobi.cuh"
#include "letkf_mixed_util.cuh"
#include "letkf_umma.cuh"

#ifndef LG_MIXED_JACOBI_TOL
#define LG_MIXED_JACOBI_TOL 2e-6f
#endif
// chunks summed by the tensor cores in the scratch accumulators before the
// FP32 round-to-nearest addition to the running sums (as in letkf_mixed.cu)
#ifndef LG_ACC_FLUSH
#define LG_ACC_FLUSH 16
#endif

namespace {

constexpr int kTW = 256;

// Optional per-phase cycle counts of CTA 0 (built with -DLG_PHASE_CLOCKS).
#ifdef LG_PHASE_CLOCKS
#define LGW_PHASE(i)                                                 \
    do {                                                             \
        if (tid == 0) {                                              \
            const long long now_ = clock64();                        \
            ph_cyc[i] += now_ - ph_last;                             \
            ph_last = now_;                                          \
        }                                                            \
    } while (0)
#else
#define LGW_PHASE(i) \
    do {             \
    } while (0)
#endif

constexpr size_t r1024(size_t b) { return (b + 1023) & ~(size_t)1023; }
constexpr size_t zmax(size_t a, size_t b) { return a > b ? a : b; }

template <int K>
struct WCfg {
    static constexpr int KB = K / 4;
    static constexpr int NLOW = KB * (KB + 1) / 2;
    static constexpr int ML = (NLOW + kTW - 1) / kTW;
    static constexpr int NFULL = KB * KB;
    static constexpr int MF = (NFULL + kTW - 1) / kTW;
    static constexpr int G = 4;                          // K/2 pairs x 4 lanes <= 256 threads
    static constexpr int CH = 64;                        // observations per MMA tile
    static constexpr uint32_t TMEM_COLS = 512;
    static constexpr uint32_t HI_COL = 256;              // first TMEM column of the hi accumulator
    static constexpr uint32_t ACC1 = 128;                // scratch accumulators after the running ones
    static constexpr int NB = K;                         // A-build N: Yhat_hi
    static constexpr int TROWS = (128 + NB > 256) ? 128 + NB : 256;
    static constexpr int TILE = TROWS * 128;
    // Jacobi column stride and moving-buffer stride: K + 16 puts the two slots
    // of a quarter-warp on disjoint bank halves (hierarchical ordering)
    static constexpr int LDW = ((K & (K - 1)) == 0) ? K + 16 : K + 4;
    static constexpr int JEXTRA = 2 * K;                 // moving-column norms and ids after W
    static constexpr int LDS = K + 1;                    // S staging row stride
    static constexpr size_t STAGE = (size_t)CH * K * sizeof(float);
    static constexpr size_t TBSUB = (size_t)K * 128;     // one T tile along members (K rows)
    static constexpr size_t RV = r1024((size_t)K * K * sizeof(float));
    static constexpr size_t RA = r1024(zmax(zmax((size_t)K * LDW + JEXTRA, (size_t)K * LDS) * sizeof(float), 4 * TBSUB));
    static constexpr size_t RB = r1024(zmax(zmax((size_t)K * K * sizeof(float), 65536),
                                            2 * TILE + 2 * STAGE > RA ? 2 * TILE + 2 * STAGE - RA : 0));
    static constexpr size_t VEC = sizeof(double) * (4 * K + 128) + sizeof(float) * (2 * K) +
                                  3 * CH * (sizeof(int) + 2 * sizeof(float));
    static constexpr size_t SMEM = 1024 + RV + RA + RB + VEC + 256;
    static_assert(K > 64 && K <= 128 && K % 32 == 0, "wide form: k = 96 or 128");
    static_assert(TILE % 1024 == 0 && STAGE % 1024 == 0 && TBSUB % 1024 == 0, "1024-byte aligned tiles");
    static_assert(SMEM <= 227 * 1024, "shared memory");
    static_assert(16 * K * sizeof(float) <= STAGE, "g and diagonal task sums pass through a gather stage");
    static_assert(K <= (int)ACC1 && HI_COL + ACC1 + K <= TMEM_COLS, "A-build accumulators must fit the TMEM allocation");
};

template <int K>
__global__ void __launch_bounds__(kTW, 1)
k_core_mixed_wide(LgGrid g, LgParams prm, const float *__restrict__ ys32, const int32_t *__restrict__ lidx,
                  const float2 *__restrict__ lmeta, const int *__restrict__ queue, int nchunks, int chunk,
                  const int64_t *__restrict__ loff, const int32_t *__restrict__ lcnt, int64_t ncubes,
                  const double *__restrict__ xb, const double *__restrict__ axb, double *__restrict__ xa,
                  double *__restrict__ axa, double *__restrict__ trans_out, double *__restrict__ w_out,
                  unsigned long long *__restrict__ counters, unsigned *__restrict__ status,
                  const unsigned *__restrict__ ymax)
{
    using C = WCfg<K>;
    constexpr int CH = C::CH;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *area = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *RV = area, *RA = area + C::RV, *RB = RA + C::RA;
    double *gv = reinterpret_cast<double *>(RB + C::RB);
    double *wbar = gv + K;
    double *misc = wbar + K;       // 2K
    double *inc = misc + 2 * K;    // 128
    float *nrm32 = reinterpret_cast<float *>(inc + 128);           // K
    int *mg = reinterpret_cast<int *>(nrm32 + 2 * K);               // 3 x CH obs indices
    float *msq = reinterpret_cast<float *>(mg + 3 * CH);            // 3 x CH sqrt(rloc)
    float *me = msq + 3 * CH;                                       // 3 x CH e
    float *stage0 = reinterpret_cast<float *>(RA + 2 * C::TILE);
    float *stage1 = stage0 + CH * K;
    float *Vprev = reinterpret_cast<float *>(RV);                   // previous cube's X by rows
    __shared__ uint64_t mbar[3];
    __shared__ uint32_t s_tmem;
    __shared__ int s_rot, s_ok, s_chunk;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) lg_tmem_alloc(lg_smem_u32(&s_tmem), C::TMEM_COLS);
    if (tid == 0)
        for (int b = 0; b < 3; b++) lg_mbar_init(&mbar[b], 1);
    lg_tc_fence_before();
    __syncthreads();
    lg_tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t idesc_u = lg_idesc_bf16(128, K);         // update: xb (hi/lo) x T
    const uint32_t idesc_a = lg_idesc_f16(128, C::NB);      // A build
    // the A build's operands times 2^E (FP16 range), its products times 2^-2E
    const int ye = lg_f16_scale_exp(*ymax);
    const float ysc = lg_pow2f(ye), yunsc = lg_pow2f(-2 * ye);
    uint32_t ncommit[3] = {0u, 0u, 0u};
    bool pending[3] = {false, false, false};
    bool failed = false;

    // Bounded wait for the last commit on barrier b; one that runs out leaves
    // the commit pending for the drain (at most one commit per barrier is
    // outstanding, so the phase parity names it).
    auto wait_bar = [&](int b, uint32_t limit) -> bool {
        if (!pending[b]) return true;
        if (tid == 0) s_ok = lg_mbar_wait(&mbar[b], (ncommit[b] - 1u) & 1u, limit) ? 1 : 0;
        __syncthreads();
        const int ok = s_ok;
        __syncthreads();
        if (ok) pending[b] = false;
        return ok != 0;
    };

#ifdef LG_PHASE_CLOCKS
    long long ph_cyc[7] = {0, 0, 0, 0, 0, 0, 0};
    long long ph_last = clock64();
#endif
    for (;;) {
    if (tid == 0) {
        const unsigned long long q = atomicAdd(&counters[LG_CNT_QUEUE], 1ull);
        s_chunk = q < (unsigned long long)nchunks ? queue[q] : -1;
    }
    __syncthreads();
    const int ck = s_chunk;
    __syncthreads();
    if (ck < 0) break;
    // chunks are aligned to multiples of `chunk` in cube numbering; the
    // first and last chunk of a window may be partial
    const int64_t chunk_at = prm.cube0 / chunk * chunk + (int64_t)ck * chunk;
    const int cube_begin = (int)max(chunk_at, prm.cube0);
    const int cube_end = (int)min(ncubes, chunk_at + chunk);
    bool have_prev = false;
    for (int cube = cube_begin; cube < cube_end; cube++) {
        if (cube % LG_WARM_RUN == 0) have_prev = false;
        const int64_t off = loff[cube];
        const int p = lcnt[cube];
        LGW_PHASE(6);

        // ---------------- phase 1: A on the tensor cores, g and diag(A) -------------
        // rows K..127 and 128+K..TROWS-1 of both tiles stay zero
        for (int t = tid; t < 2 * C::TROWS * 8; t += kTW) {
            const int b = t / (C::TROWS * 8), rest = t % (C::TROWS * 8);
            const int r = rest / 8, c = rest % 8;
            if ((r >= K && r < 128) || r >= 128 + K)
                *reinterpret_cast<uint4 *>(RA + b * C::TILE + lg_sw128_offset(r, c)) = make_uint4(0, 0, 0, 0);
        }
        const int nch = (p + CH - 1) / CH;
        // the FP32-pipe sums of this thread's conversion tasks (t = tid + i kTW:
        // column t % K, observations 8 (t / K) .. + 7 of every chunk)
        constexpr int NTASK = (K * 8 + kTW - 1) / kTW;
        float acc_g[NTASK], acc_d[NTASK];
#pragma unroll
        for (int i = 0; i < NTASK; i++) acc_g[i] = acc_d[i] = 0.0f;
        auto load_meta = [&](int x, int &gi, float2 &mf) {      // tid < CH
            const int o = x * CH + tid;
            if (x < nch && o < p) {
                gi = lidx[off + o];
                mf = lmeta[off + o];
            } else {
                gi = -1;
                mf = make_float2(0.0f, 0.0f);
            }
        };
        auto put_meta = [&](int x, int gi, float2 mf) {
            const int r = (x % 3) * CH + tid;
            mg[r] = gi;
            msq[r] = mf.x * ysc;
            me[r] = mf.y * ysc;
        };
        auto issue_rows = [&](int x) {
            float *st = (x & 1) ? stage1 : stage0;
            const int *gs = mg + (x % 3) * CH;
            constexpr int PPR = K / 4;
            for (int q = tid; q < CH * PPR; q += kTW) {
                const int o = q / PPR, part = q % PPR;
                const int gi = gs[o];
                if (gi >= 0) cp_async16(lg_smem_u32(st + o * K + part * 4), ys32 + (int64_t)gi * K + part * 4);
            }
            cp_async_commit();
        };
        int pf_g = -1;
        float2 pf_m = make_float2(0.0f, 0.0f);
        if (nch > 0) {
            if (tid < CH) {
                int g0, g1;
                float2 m0, m1;
                load_meta(0, g0, m0);
                load_meta(1, g1, m1);
                load_meta(2, pf_g, pf_m);
                put_meta(0, g0, m0);
                put_meta(1, g1, m1);
            }
            __syncthreads();
            issue_rows(0);
            issue_rows(1);
        }
        for (int ch = 0; ch < nch; ch++) {
            const int b = ch & 1;
            const float *st = b ? stage1 : stage0;
            const float *sq = msq + (ch % 3) * CH, *ev = me + (ch % 3) * CH;
            cp_async_wait<1>();
            __syncthreads();
            unsigned char *tile = RA + b * C::TILE;
            if (!wait_bar(b, prm.spin_limit)) {
                failed = true;
                break;
            }
            const int cnt = min(CH, p - ch * CH);
#pragma unroll
            for (int i = 0; i < NTASK; i++) {
                const int t = tid + i * kTW;
                if (t < K * 8) {
                    const int m = t % K, c = t / K;
                    float v[8];
                    uint4 hi, lo;
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const int o = 8 * c + j;
                        v[j] = (o < cnt) ? st[o * K + m] * sq[o] : 0.0f;
                    }
                    split8_f16(v, hi, lo);
                    *reinterpret_cast<uint4 *>(tile + lg_sw128_offset(128 + m, c)) = hi;
                    *reinterpret_cast<uint4 *>(tile + lg_sw128_offset(m, c)) = lo;
                    // g and the diagonal (e is zero past the list's end)
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        acc_g[i] = fmaf(v[j], ev[8 * c + j], acc_g[i]);
                        acc_d[i] = fmaf(v[j], v[j], acc_d[i]);
                    }
                }
            }
            lg_fence_async_smem();
            __syncthreads();
            if (ch > 0 && ch % LG_ACC_FLUSH == 0) {
                // the last group's sums into the running ones in FP32 round to
                // nearest (the first group's copied) before this chunk's
                // products restart the scratch accumulators; chunk ch - 2's
                // products were waited for above
                if (!wait_bar(b ^ 1, prm.spin_limit)) {
                    failed = true;
                    break;
                }
                lg_tc_fence_after();
                if (warp < 4) {
                    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
                    for (int h = 0; h < 2; h++) {
                        const uint32_t base = tl + (h ? C::HI_COL : 0u);
#pragma unroll 1
                        for (int c0 = 0; c0 < K; c0 += 16) {
                            float v[16], u[16];
                            lg_tmem_ld16x2(base + C::ACC1 + (uint32_t)c0, base + (uint32_t)c0, v, u);
                            if (ch > LG_ACC_FLUSH) {
#pragma unroll
                                for (int j = 0; j < 16; j++) v[j] = u[j] + v[j];
                            }
                            lg_tmem_st16(base + (uint32_t)c0, v);
                        }
                    }
                }
                lg_tc_fence_before();
                __syncthreads();
            }
            if (tid == 0) {
                lg_tc_fence_after();
                const uint64_t dlo = lg_desc_sw128(lg_smem_u32(tile));
                const uint64_t dhi = lg_desc_sw128(lg_smem_u32(tile + 128 * 128));   // Yhat_hi, e: A_hi and B
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint32_t acc = (ch % LG_ACC_FLUSH != 0 || kk > 0) ? 1u : 0u;
                    lg_umma_bf16(tmem + C::ACC1, dlo + 2 * kk, dhi + 2 * kk, idesc_a, acc);
                    lg_umma_bf16(tmem + C::HI_COL + C::ACC1, dhi + 2 * kk, dhi + 2 * kk, idesc_a, acc);
                }
                lg_umma_commit(&mbar[b]);
            }
            ncommit[b]++;
            pending[b] = true;
            if (tid < CH) {
                put_meta(ch + 2, pf_g, pf_m);
                load_meta(ch + 3, pf_g, pf_m);
            }
            __syncthreads();
            issue_rows(ch + 2);
        }
        cp_async_wait<0>();
        if (failed) break;
        // the task sums through the first gather stage (no copy in flight, its
        // rows read before the last chunk's barrier): [g | diag][task]
#pragma unroll
        for (int i = 0; i < NTASK; i++) {
            const int t = tid + i * kTW;
            if (t < K * 8) {
                stage0[t] = acc_g[i];
                stage0[K * 8 + t] = acc_d[i];
            }
        }
        if (!wait_bar(0, prm.spin_limit) || !wait_bar(1, prm.spin_limit)) {
            failed = true;
            break;
        }
        lg_tc_fence_after();
        __syncthreads();
        // g and diag(A) over the 8 observation groups in a fixed order, times
        // 2^-2E, in misc (before S, which overlaps the stage, is written)
        if (tid < K) {
            double sg = 0.0, sd = 0.0;
#pragma unroll
            for (int c = 0; c < 8; c++) {
                sg += (double)stage0[c * K + tid];
                sd += (double)stage0[K * 8 + c * K + tid];
            }
            misc[tid] = sg * (double)yunsc;
            misc[K + tid] = sd * (double)yunsc;
        }
        __syncthreads();
        LGW_PHASE(0);

        // ---------------- phase 2: A = 0.5 (S + S^T), S = HH + 2 LH; g -------------------
        float *S = reinterpret_cast<float *>(RA);
        float *A32 = reinterpret_cast<float *>(RB);               // A (without (k-1)/rho I)
        float *W32 = reinterpret_cast<float *>(RA);
        if (warp < 4) {
            const int row = warp * 32 + lane;
            const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
            for (int c0 = 0; c0 < K; c0 += 16) {
                float lo[16], hi[16];
                if (p > 0) {
                    // the last group's sums, plus the running ones before it
                    float u[16];
                    lg_tmem_ld16x2(tl + C::ACC1 + (uint32_t)c0, tl + (uint32_t)c0, lo, u);
                    if (nch > LG_ACC_FLUSH) {
#pragma unroll
                        for (int j = 0; j < 16; j++) lo[j] = u[j] + lo[j];
                    }
                    lg_tmem_ld16x2(tl + C::HI_COL + C::ACC1 + (uint32_t)c0, tl + C::HI_COL + (uint32_t)c0, hi, u);
                    if (nch > LG_ACC_FLUSH) {
#pragma unroll
                        for (int j = 0; j < 16; j++) hi[j] = u[j] + hi[j];
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; j++) lo[j] = hi[j] = 0.0f;
                }
                if (row < K) {
#pragma unroll
                    for (int j = 0; j < 16; j++) S[row * C::LDS + c0 + j] = fmaf(2.0f, lo[j], hi[j]);
                }
            }
            if (row < K) gv[row] = misc[row];
        }
        lg_tc_fence_before();
        __syncthreads();
        for (int idx = tid; idx < K * K; idx += kTW) {
            const int i = idx / K, j = idx % K;
            A32[idx] = i == j ? (float)misc[K + i] : 0.5f * (S[i * C::LDS + j] + S[j * C::LDS + i]) * yunsc;
        }
        __syncthreads();                                          // S is dead
        const double cdiag = (double)(K - 1) / prm.inflation;
        const float cdiagf = (float)cdiag;
        if (!have_prev) {
            // cold start: the Jacobi works on A' itself (symmetric: column j = row j)
            for (int idx = tid; idx < K * K; idx += kTW) {
                const int j = idx / K, i = idx % K;
                W32[j * C::LDW + i] = A32[idx] + (i == j ? cdiagf : 0.0f);
            }
        } else {
            // warm start: W = A' Vprev = A Vprev + (k-1)/rho Vprev
            for (int m = 0; m < C::MF; m++) {
                const int b = tid + m * kTW;
                if (b >= C::NFULL) continue;
                const int bi = b / C::KB, bj = b % C::KB;
                float acc[16];
#pragma unroll
                for (int i = 0; i < 16; i++) acc[i] = 0.0f;
                for (int l = 0; l < K; l++) {
                    const float4 av = *reinterpret_cast<const float4 *>(A32 + l * K + 4 * bi);
                    const float4 vv = *reinterpret_cast<const float4 *>(Vprev + l * K + 4 * bj);
                    const float x[4] = {av.x, av.y, av.z, av.w};
                    const float y[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int jj = 0; jj < 4; jj++) acc[i * 4 + jj] = fmaf(x[i], y[jj], acc[i * 4 + jj]);
                }
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int jj = 0; jj < 4; jj++)
                        W32[(4 * bj + jj) * C::LDW + 4 * bi + i] =
                            fmaf(cdiagf, Vprev[(4 * bi + i) * K + 4 * bj + jj], acc[i * 4 + jj]);
            }
        }
        __syncthreads();
        LGW_PHASE(1);

        // ---------------- phase 3: FP32 Jacobi -> X (columns of W32) --------------------
        int sw;
        if constexpr (K == 128)
            sw = lg_jacobi32b2<K, C::LDW, C::LDW>(W32, W32 + K * C::LDW, &s_rot, LG_MIXED_JACOBI_TOL, 24);
        else
            sw = lg_jacobi32b3<K, C::LDW, C::LDW>(W32, W32 + K * C::LDW, &s_rot, LG_MIXED_JACOBI_TOL, 24);
        if (tid == 0) {
            atomicMax(&counters[LG_CNT_MAXSWEEP], (unsigned long long)sw);
            atomicAdd(&counters[LG_CNT_SUMSWEEP], (unsigned long long)sw);
            if (sw > 24) atomicAdd(&counters[LG_CNT_NOTCONV], 1ull);
        }
        LGW_PHASE(2);
        float *ilam32 = reinterpret_cast<float *>(misc);
        float *hc32 = ilam32 + K, *r32 = hc32 + 2 * K;
        for (int j = warp; j < K; j += kTW / 32) {
            float s = 0.0f;
            for (int r = lane; r < K; r += 32) s = fmaf(W32[j * C::LDW + r], W32[j * C::LDW + r], s);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) {
                const float lamf = sqrtf(s);
                nrm32[j] = 1.0f / lamf;
                ilam32[j] = 1.0f / lamf;
                hc32[j] = sqrtf((float)(K - 1) / lamf);
            }
        }
        __syncthreads();
        if (warp == 0) {
            float lo = 3.0e38f, hi = 0.0f;
            for (int j = lane; j < K; j += 32) {
                lo = fminf(lo, ilam32[j]);
                hi = fmaxf(hi, ilam32[j]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            if (lane == 0 && hi > 1.0e4f * lo) atomicAdd(&counters[LG_CNT_ILLCOND], 1ull);
        }

        // ---------------- phase 4: X, wbar with one refinement step ------------------------
        float *X32 = reinterpret_cast<float *>(RV);               // X32[j*K + r]; Vprev is consumed
        for (int idx = tid; idx < K * K; idx += kTW) X32[idx] = W32[(idx / K) * C::LDW + idx % K] * nrm32[idx / K];
        __syncthreads();
        if (tid < K) {
            nrm32[tid] = hc32[tid];                                // f for T
            r32[tid] = (float)gv[tid];
        }
        __syncthreads();
        for (int it = 0; it < 2; it++) {
            for (int j = warp; j < K; j += kTW / 32) {
                float d = 0.0f;
                for (int l = lane; l < K; l += 32) d = fmaf(X32[j * K + l], r32[l], d);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
                if (lane == 0) hc32[j] = d * ilam32[j];
            }
            __syncthreads();
            if (tid < K) {
                float a0 = 0.0f, a1 = 0.0f;
                for (int j = 0; j < K; j += 2) {
                    a0 = fmaf(X32[j * K + tid], hc32[j], a0);
                    a1 = fmaf(X32[(j + 1) * K + tid], hc32[j + 1], a1);
                }
                wbar[tid] = (it == 0 ? 0.0 : wbar[tid]) + (double)(a0 + a1);
            }
            __syncthreads();
            if (it == 0) {
                // residual g - A' wbar in FP64: A' = A (FP32 values) + (k-1)/rho I
                for (int i = warp; i < K; i += kTW / 32) {
                    double d = 0.0;
                    for (int l = lane; l < K; l += 32) d += (double)A32[i * K + l] * wbar[l];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
                    if (lane == 0) r32[i] = (float)(gv[i] - (d + cdiag * wbar[i]));
                }
                __syncthreads();
            }
        }

        LGW_PHASE(3);

        // ---------------- phase 5: T in FP32 ------------------------------------------------
        {
            const int bjc = (int)(cube % prm.nbj), bic = (int)(cube / prm.nbj);
            const int sj = bjc * prm.cube_n, ej = min(sj + prm.cube_n - 1, g.nlat - 1);
            const int si = bic * prm.cube_n, ei = min(si + prm.cube_n - 1, g.nlon - 1);
            const int64_t lines = ((int64_t)g.n * K * (int64_t)sizeof(double) + 127) / 128;
            for (int ii = si; ii <= ei; ii++)
                for (int jj = sj; jj <= ej; jj++) {
                    const int64_t col = jj + (int64_t)g.nlat * ii;
                    const char *base = reinterpret_cast<const char *>(xb + col * g.n * K);
                    for (int64_t l = tid; l < lines; l += kTW)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(base + l * 128));
                }
        }
        float *T32 = reinterpret_cast<float *>(RB);               // A is dead
        {
            float tacc[C::ML][16];
            int tbi[C::ML], tbj[C::ML];
            bool tok[C::ML];
#pragma unroll
            for (int m = 0; m < C::ML; m++) {
                const int b = tid + m * kTW;
                tok[m] = b < C::NLOW;
                lg_decode_block(tok[m] ? b : 0, tbi[m], tbj[m]);
#pragma unroll
                for (int i = 0; i < 16; i++) tacc[m][i] = 0.0f;
                if (!tok[m]) continue;
                for (int j = 0; j < K; j++) {
                    const float f = nrm32[j];
                    const float4 av = *reinterpret_cast<const float4 *>(X32 + j * K + 4 * tbi[m]);
                    const float4 bv = *reinterpret_cast<const float4 *>(X32 + j * K + 4 * tbj[m]);
                    const float a[4] = {av.x, av.y, av.z, av.w};
                    const float bq[4] = {bv.x * f, bv.y * f, bv.z * f, bv.w * f};
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int jj = 0; jj < 4; jj++) tacc[m][i * 4 + jj] = fmaf(a[i], bq[jj], tacc[m][i * 4 + jj]);
                }
            }
#pragma unroll
            for (int m = 0; m < C::ML; m++) {
                if (!tok[m]) continue;
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) {
                        const int r = 4 * tbi[m] + i, c = 4 * tbj[m] + jj;
                        T32[r * K + c] = tacc[m][i * 4 + jj];
                        T32[c * K + r] = tacc[m][i * 4 + jj];
                    }
            }
        }
        // X by rows for the next cube's warm start, in place through registers
        {
            constexpr int PER = (K * K + kTW - 1) / kTW;
            float xv[PER];
            __syncthreads();
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const int idx = tid + q * kTW;                     // idx = r*K + j
                xv[q] = (idx < K * K) ? X32[(idx % K) * K + idx / K] : 0.0f;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const int idx = tid + q * kTW;
                if (idx < K * K) Vprev[idx] = xv[q];
            }
        }
        __syncthreads();
        if (trans_out) {
            for (int idx = tid; idx < K * K; idx += kTW) {
                const int i = idx % K, j = idx / K;
                trans_out[(int64_t)cube * K * K + idx] = (double)T32[i * K + j] + wbar[i];
            }
            if (tid < K) w_out[(int64_t)cube * K + tid] = wbar[tid];
            __syncthreads();
        }
        // the member mean of xb^T T is sqrt(rho) xbar (T 1 = sqrt(rho) 1): the
        // FP64 increment takes it, xb^T (wbar + sqrt(rho)/k 1), not the tensor
        // products (as in the narrow core)
        if (tid < K) wbar[tid] += sqrt(prm.inflation) / (double)K;
        __syncthreads();

        LGW_PHASE(4);

        // ---------------- phase 6: xa = xb^T (T + wbar 1^T) -------------------------------
        // T tiles (B operand, N = K rows) along members: hi tiles 0, 1 then lo tiles 0, 1
        unsigned char *tb = RA;
        for (int t = tid; t < K * (K / 8); t += kTW) {
            const int e = t / (K / 8), cg = t % (K / 8), s = cg / 8, c = cg % 8;
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = T32[e * K + 8 * cg + j];
            uint4 hi, lo;
            split8(v, hi, lo);
            *reinterpret_cast<uint4 *>(tb + s * C::TBSUB + lg_sw128_offset(e, c)) = hi;
            *reinterpret_cast<uint4 *>(tb + (2 + s) * C::TBSUB + lg_sw128_offset(e, c)) = lo;
        }
        __syncthreads();                                           // T32 is dead: RB takes xb tiles
        unsigned char *xt = RB;                                    // hi tiles 0, 1 then lo tiles 0, 1
        const int n = g.n;
        const int bjc = (int)(cube % prm.nbj), bic = (int)(cube / prm.nbj);
        const int sj = bjc * prm.cube_n, ej = min(sj + prm.cube_n - 1, g.nlat - 1);
        const int si = bic * prm.cube_n, ei = min(si + prm.cube_n - 1, g.nlon - 1);
        for (int ii = si; ii <= ei && !failed; ii++)
            for (int jj = sj; jj <= ej && !failed; jj++) {
                const int64_t col = jj + (int64_t)g.nlat * ii;
                const double *xbc = xb + col * n * K;
                double *xac = xa + col * n * K;
                for (int r0 = 0; r0 < n; r0 += 128) {
                    const int R = min(128, n - r0);
                    for (int t = tid; t < 128 * (K / 8); t += kTW) {
                        const int r = t / (K / 8), cg = t % (K / 8), s = cg / 8, c = cg % 8;
                        float v[8];
                        if (r < R) {
                            const double2 *src =
                                reinterpret_cast<const double2 *>(xbc + (int64_t)(r0 + r) * K + 8 * cg);
#pragma unroll
                            for (int j = 0; j < 4; j++) {
                                const double2 q = src[j];
                                v[2 * j] = (float)q.x;
                                v[2 * j + 1] = (float)q.y;
                            }
                        } else {
#pragma unroll
                            for (int j = 0; j < 8; j++) v[j] = 0.0f;
                        }
                        uint4 hi, lo;
                        split8(v, hi, lo);
                        *reinterpret_cast<uint4 *>(xt + s * 16384 + lg_sw128_offset(r, c)) = hi;
                        *reinterpret_cast<uint4 *>(xt + (2 + s) * 16384 + lg_sw128_offset(r, c)) = lo;
                    }
                    for (int r = warp; r < R; r += kTW / 32) {
                        const double *src = xbc + (int64_t)(r0 + r) * K;
                        double s = 0.0;
                        for (int i = lane; i < K; i += 32) s += src[i] * wbar[i];
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                        if (lane == 0) inc[r] = s;
                    }
                    lg_fence_async_smem();
                    __syncthreads();
                    if (tid == 0) {
                        lg_tc_fence_after();
#pragma unroll
                        for (int kk = 0; kk < K / 16; kk++) {
                            const int s = kk / 4, k4 = kk % 4;
                            const uint64_t dh = lg_desc_sw128(lg_smem_u32(xt + s * 16384)) + 2 * k4;
                            const uint64_t dl = lg_desc_sw128(lg_smem_u32(xt + (2 + s) * 16384)) + 2 * k4;
                            const uint64_t th = lg_desc_sw128(lg_smem_u32(tb + s * C::TBSUB)) + 2 * k4;
                            const uint64_t tl = lg_desc_sw128(lg_smem_u32(tb + (2 + s) * C::TBSUB)) + 2 * k4;
                            lg_umma_bf16(tmem, dh, th, idesc_u, kk > 0 ? 1u : 0u);
                            lg_umma_bf16(tmem, dh, tl, idesc_u, 1u);
                            lg_umma_bf16(tmem, dl, th, idesc_u, 1u);
                        }
                        lg_umma_commit(&mbar[2]);
                    }
                    ncommit[2]++;
                    pending[2] = true;
                    if (!wait_bar(2, prm.spin_limit)) {
                        failed = true;
                        break;
                    }
                    lg_tc_fence_after();
                    if (warp < 4) {
                        const int r = warp * 32 + lane;
                        const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
                        // member mean and perturbations in FP32 (the products are
                        // FP32 sums of BF16 hi/lo terms), written as FP64 with the
                        // conversion on the integer pipe
                        float part[8];
#pragma unroll
                        for (int q = 0; q < 8; q++) part[q] = 0.0f;
                        for (int c0 = 0; c0 < K; c0 += 16) {
                            float v[16];
                            lg_tmem_ld16(tl + (uint32_t)c0, v);
#pragma unroll
                            for (int e = 0; e < 16; e++) part[e & 7] += v[e];
                        }
                        const float meanf =
                            (((part[0] + part[1]) + (part[2] + part[3])) + ((part[4] + part[5]) + (part[6] + part[7]))) /
                            (float)K;
                        if (r < R) {
                            const int64_t row = col * n + r0 + r;
                            axa[row] = axb[row] + inc[r];
                        }
                        double *dst = xac + (int64_t)(r0 + r) * K;
                        for (int c0 = 0; c0 < K; c0 += 16) {
                            float v[16];
                            lg_tmem_ld16(tl + (uint32_t)c0, v);
                            if (r < R) {
#pragma unroll
                                for (int e = 0; e < 16; e += 2)
                                    *reinterpret_cast<double2 *>(dst + c0 + e) =
                                        make_double2(lg_f2d_bits(v[e] - meanf), lg_f2d_bits(v[e + 1] - meanf));
                            }
                        }
                    }
                    lg_tc_fence_before();
                    __syncthreads();
                }
            }
        if (failed) break;
        have_prev = true;
        LGW_PHASE(5);
    }
    if (failed) break;
    }
#ifdef LG_PHASE_CLOCKS
    if (blockIdx.x == 0 && tid == 0)
        printf("wide phase cycles cta0: A-build %lld, A'-form %lld, jacobi32 %lld, X/wbar %lld, T %lld, "
               "update %lld, loop %lld\n",
               ph_cyc[0], ph_cyc[1], ph_cyc[2], ph_cyc[3], ph_cyc[4], ph_cyc[5], ph_cyc[6]);
#endif
    if (failed && tid == 0) atomicOr(status, LG_ST_TIMEOUT);
    cp_async_wait<0>();
    // every committed MMA finishes before the TMEM is freed (at the normal
    // limit, whatever limit the run's waits had)
    bool drained = true;
    for (int b = 0; b < 3; b++) drained = wait_bar(b, LG_MBAR_SPIN_LIMIT) && drained;
    if (!drained && tid == 0) atomicOr(status, LG_ST_TIMEOUT);
    lg_tc_fence_before();
    __syncthreads();
    lg_tc_fence_after();
    if (warp == 0) lg_tmem_dealloc(tmem, C::TMEM_COLS);
}

template <int K>
cudaError_t launch_wide(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb, double *xa,
                        double *axa, double *trans_out, double *w_out)
{
    const size_t smem = WCfg<K>::SMEM;
    cudaError_t e = cudaFuncSetAttribute(k_core_mixed_wide<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    if (ctx->win1 <= ctx->win0) return cudaSuccess;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int chunk = 0, nchunks = 0;
    e = lg_build_chunk_queue(ctx, chunk, nchunks);
    if (e != cudaSuccess) return e;
    // persistent grid, one CTA per SM (it holds all 512 TMEM columns)
    const unsigned blocks = (unsigned)(nchunks < nsm ? nchunks : nsm);
    lg_count_launch();
    k_core_mixed_wide<K><<<blocks, kTW, smem, ctx->stream>>>(
        g, lg_params(ctx), ctx->d_ys32.p, ctx->d_lidx.p, ctx->d_lmeta.p, ctx->d_queue.p, nchunks, chunk,
        ctx->d_loff.p, ctx->d_lcnt.p, ctx->win1, xb, axb, xa, axa, trans_out, w_out, ctx->d_counters.p,
        ctx->d_status.p, ctx->d_ymax.p);
    return cudaGetLastError();
}

}  // namespace

cudaError_t lg_launch_core_mixed_wide(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb,
                                      double *xa, double *axa, double *trans_out, double *w_out)
{
    switch (g.k) {
    case 96: return launch_wide<96>(ctx, g, xb, axb, xa, axa, trans_out, w_out);
    case 128: return launch_wide<128>(ctx, g, xb, axb, xa, axa, trans_out, w_out);
    default: return cudaErrorInvalidValue;
    }
}
