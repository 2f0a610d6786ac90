// letkf_mixed.cu -- mixed-precision per-cube LETKF core (precision 1).
//
// Same analysis as letkf_core.cu (letkf_core, code/x86/TradDA/DA/LETKF/src/
// letkf_core.F90:14-233, and xb_2_xa, letkf_compute.F90:231-301), with the two
// dense products on the Blackwell tensor cores and the conditioning-sensitive
// steps in FP64:
//
//   1. A = Yhat Yhat^T on tcgen05 (FP16 operands, FP32 accumulation in TMEM).
//      Yhat = Y sqrt(rdiaginv rloc), times a power of two that fits FP16's
//      range, is split per element into hi + lo FP16 parts; one MMA stream
//      multiplies the stacked [Yhat_lo; Yhat_hi] (M = 128 rows) by Yhat_hi
//      (N = k), so A = HH + LH + LH^T recovers the hi*lo cross terms.  The
//      observation rows are gathered, scaled and split into 128-byte-swizzled
//      K-major tiles by all threads while the previous tile's MMAs run (two
//      tiles, mbarrier-tracked).  g = Yhat e with e = sqrt(rdiaginv rloc) dep
//      and the diagonal of A are summed on the FP32 pipe by the same threads
//      (round to nearest: the tensor-core sums drift with the number of
//      observations, which those terms would pass to the analysis).
//   2. A' = A + (k-1)/rho I in FP64.
//   3. FP32 one-sided Jacobi of A' (warm-started from the neighbouring
//      cube's eigenvectors inside aligned runs of cubes, so that results do
//      not depend on the schedule) gives the eigenpairs: lambda_j = |w_j|,
//      x_j = w_j/lambda_j.
//   4. wbar = X diag(1/lambda) X^T g in FP32, then one step of iterative
//      refinement: wbar += X diag(1/lambda) X^T (g - A' wbar) with the
//      residual in FP64 against the FP64 A'.  A' has condition numbers below
//      ~1e3 at these sizes, so one step takes wbar from ~1e-7 to ~1e-13
//      relative; wbar is accumulated in FP64.
//   5. T = X diag(sqrt((k-1)/lambda)) X^T in FP32: it only feeds the BF16
//      hi/lo update, and FP32 eigenpairs give it to ~1e-7 relative.
//   6. xa = xb^T T on tcgen05 (hi/lo BF16 of both operands, three products in
//      one accumulator); the mean increment xb^T wbar is FP64.
//
// k = 32 and 48 run all steps in one persistent launch (k_core_mixed<k, 0>;
// warm-start runs of LG_WARM_RUN cubes).
// k = 64 runs them in three launches per block of cubes: the A and g build
// (k_core_mixed<64, 1>), steps 3-5 one warp per cube (k_eig_warp<64>, runs of
// 8 cubes warm-started inside a run, taken from a queue) and step 6
// (k_core_mixed<64, 3>), with A and g, then T and wbar, in HBM between them.
// LETKF_PREC_MIXED_F64EIG adds a fourth launch between the eigensolve and
// the update (k_eig_refine<64>): the FP32 eigenpairs refined in FP64, then
// T and wbar in FP64.
#include <cuda_bf16.h>

#include "letkf_internal.cuh"
#include "letkf_jacobi.cuh"
#include "letkf_mixed_util.cuh"
#include "letkf_umma.cuh"

// Chunks of observations (64 each) whose products the tensor cores sum in a
// scratch accumulator before its sums are added to the running ones in FP32
// round-to-nearest (the tensor cores' own sums drift by about 1e-8 of the sum
// per observation).
#ifndef LG_ACC_FLUSH
#define LG_ACC_FLUSH 16
#endif

// Column-cosine tolerance of the FP32 Jacobi.  It bounds the eigenvectors'
// orthogonality error, which reaches T (BF16 hi/lo in the update, ~1e-5
// relative) scaled by about one half.
#ifndef LG_MIXED_JACOBI_TOL
#define LG_MIXED_JACOBI_TOL 2e-6f
#endif

namespace {

constexpr int kT = 256;

// Optional per-phase cycle counts of CTA 0 (built with -DLG_PHASE_CLOCKS).
#ifdef LG_PHASE_CLOCKS
#define LG_PHASE(i)                                                  \
    do {                                                             \
        if (tid == 0) {                                              \
            const long long now_ = clock64();                        \
            ph_cyc[i] += now_ - ph_last;                             \
            ph_last = now_;                                          \
        }                                                            \
    } while (0)
#else
#define LG_PHASE(i) \
    do {            \
    } while (0)
#endif

template <int K>
struct MCfg {
    static constexpr int KB = K / 4;
    static constexpr int NLOW = KB * (KB + 1) / 2;     // lower 4x4 blocks
    static constexpr int ML = (NLOW + kT - 1) / kT;
    static constexpr int NFULL = KB * KB;              // all 4x4 blocks
    static constexpr int MF = (NFULL + kT - 1) / kT;
    static constexpr int G = (K / 2 * 16 <= kT) ? 16 : (K / 2 * 8 <= kT) ? 8 : 4;
    static constexpr int CH = 64;                      // observations per MMA tile (K of the MMA)
    static constexpr uint32_t TMEM_COLS = 128;         // A build: N = K columns, twice
    static constexpr uint32_t ACC1 = 64;               // the A build's scratch accumulator
    // A-build tile rows: Yhat_lo (K), Yhat_hi (K), zeros to the M = 128 rows
    // of the A operand
    static constexpr int TROWS = (2 * K > 128) ? 2 * K : 128;
    static constexpr int TILE = TROWS * 128;
    static constexpr int LDW = K + 4;                  // padded column stride of the FP32 Jacobi
    static constexpr size_t AREA = 64 * 1024;          // tiles / FP32 scratch / P, R, Xhat
    static constexpr size_t B1 = sizeof(double) * K * K;
    // per-chunk observation index and factors, a ring of 3 chunks
    static constexpr size_t VEC = sizeof(double) * (4 * K + 128) + sizeof(float) * (2 * K) +
                                  3 * CH * (sizeof(int) + 2 * sizeof(float));
    static constexpr size_t SMEM = 1024 + AREA + B1 + VEC + 256;
    // the A-build launch (ST 1) holds only the two tiles (then Dhh, Dlh) and
    // the two gather stages: three CTAs per SM
    static constexpr size_t AREA1 = ((2 * (size_t)TILE > 2 * (size_t)K * (K + 1) * sizeof(float)
                                          ? 2 * (size_t)TILE
                                          : 2 * (size_t)K * (K + 1) * sizeof(float)) + 1023) & ~(size_t)1023;
    static constexpr size_t SMEM1 = 1024 + AREA1 + B1 + VEC;
    // the update launch without the members (ST 3): the xb and T tiles (48 KB),
    // the epilogue's exchange rows, and the mean-increment partials in place of
    // B1 (T is read from its slot in global memory): three CTAs per SM
    static constexpr size_t AREA3 = 53 * 1024;
    static constexpr size_t B13 = sizeof(double) * 128 * (K / 8);
    static constexpr size_t SMEM3 = 1024 + AREA3 + B13 + VEC;
    static_assert(49152 + 128 * 9 * sizeof(float) <= AREA3, "update tiles and exchange rows");
    static_assert(2 * (size_t)K * (K + 1) * sizeof(float) <= AREA1, "Dhh and Dlh must fit over the tiles");
    static_assert(AREA1 % 1024 == 0, "1024-byte aligned tiles");
    // gathered FP32 observation rows of one chunk; two stages: the first in B1
    // (free while A is built), the second after it in B1 or after the tiles
    static constexpr size_t STAGE = (size_t)CH * K * sizeof(float);
    static constexpr bool STAGE1_IN_B1 = 2 * STAGE <= B1;
    static_assert(2 * K <= 128, "stacked hi/lo rows must fit M = 128");
    static_assert(K % 16 == 0, "N must be a multiple of 16");
    static_assert(2 * TILE <= 49152, "A-build tiles must not reach the warm-start vectors");
    static_assert(K <= (int)ACC1 && ACC1 + K <= TMEM_COLS, "A-build accumulators must fit the TMEM allocation");
    // the conversion threads' partial sums of g and diag(A), [2][8][K] floats,
    // pass through the first gather stage after the last chunk
    static_assert(16 * K * sizeof(float) <= STAGE, "g and diagonal partials");
    static_assert(STAGE <= B1 && (STAGE1_IN_B1 || 2 * TILE + STAGE <= 49152), "gather stages must fit");
};

// The end of a fused members run for one state row (letkf2dnn,
// module_da_parallel.F90:214-258), from the update's FP32 products v (member
// mean meanf), the row's background mean mb and the FP64 mean increment
// (with the member mean of xb^T T, sqrt(rho) xbar, in it):
// axa = mb + incr; where |grid_lat| <= polar the members are
// gamma1 (axb + xb) + gamma2 (axa + xa), taken as the FP64 row constant
// gamma1 mb + gamma2 axa plus the FP32 perturbation part gamma1 xb + gamma2
// xa (xb from the row's BF16 hi/lo tile, 2^-17 of xb), else the background
// members themselves; spread_b = sqrt(sum xb^2 / ens) from the staging's
// partial sums, spread_a = sqrt(sum (member - axa)^2 / ens).
template <int K>
__device__ __forceinline__ void members_epilogue(const LgParams &prm, const LgGrid &g, int64_t col, int r,
                                                 const double *xin_row, const unsigned char *t_hi,
                                                 const unsigned char *t_lo, double mb, double incr, float meanf,
                                                 const float *v, const float *sqp, double *dst, int64_t row)
{
    const float fk = (float)K;
    float sb = 0.0f;
#pragma unroll
    for (int c = 0; c < K / 8; c++) sb += sqp[c * 128 + r];
    const double ma = mb + incr;
    const bool blend = fabs((double)g.glat[col % g.nlat]) <= prm.polar;
    if (!blend) {
        for (int e = 0; e < K; e += 2)
            *reinterpret_cast<double2 *>(dst + e) = *reinterpret_cast<const double2 *>(xin_row + e);
        prm.spb[row] = sqrt((double)(sb / fk));
        prm.spa[row] = sqrt((double)(sb / fk));
        return;
    }
    const double cst = prm.gamma1 * mb + prm.gamma2 * ma;
    const float df = (float)(cst - ma), g1 = (float)prm.gamma1, g2 = (float)prm.gamma2;
    float sa = 0.0f;
#pragma unroll
    for (int c = 0; c < K / 8; c++) {
        const uint4 h = *reinterpret_cast<const uint4 *>(t_hi + lg_sw128_offset(r, c));
        const uint4 l = *reinterpret_cast<const uint4 *>(t_lo + lg_sw128_offset(r, c));
        const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            // BF16 pairs: element 2q in the low half, 2q + 1 in the high half
            const float b0 = __uint_as_float(hw[q] << 16) + __uint_as_float(lw[q] << 16);
            const float b1 = __uint_as_float(hw[q] & 0xffff0000u) + __uint_as_float(lw[q] & 0xffff0000u);
            const int e = 8 * c + 2 * q;
            const float d0 = fmaf(g1, b0, g2 * (v[e] - meanf)), d1 = fmaf(g1, b1, g2 * (v[e + 1] - meanf));
            sa = fmaf(df + d0, df + d0, fmaf(df + d1, df + d1, sa));
            *reinterpret_cast<double2 *>(dst + e) = make_double2(cst + lg_f2d_bits(d0), cst + lg_f2d_bits(d1));
        }
    }
    prm.spb[row] = sqrt((double)(sb / fk));
    prm.spa[row] = sqrt((double)(sa / fk));
}

// ST selects the stages a launch runs: 0 all of them; 1 the A build only
// (A without the diagonal shift and g to mA, mgv); 3 the update only, from T
// (FP32, row-major, in the slot of X) and wbar (FP64, in the slot of g),
// written by the eigensolve launch (k_eig_warp) or by the FP64 refinement
// (k_eig_refine).  The intermediates are indexed by cube - prm.cube0.
// MEM: the fused members run (LgParams::members; stages 0 and 3), a separate
// instantiation so the plain update keeps its registers.
template <int K, int ST, bool MEM = false>
__global__ void __launch_bounds__(kT, (ST == 1 || (ST == 3 && !MEM)) ? 3 : 2)
k_core_mixed(LgGrid g, LgParams prm, const float *__restrict__ ys32, const int32_t *__restrict__ lidx,
             const float2 *__restrict__ lmeta, const int *__restrict__ queue, int nchunks, int chunk,
             const int64_t *__restrict__ loff, const int32_t *__restrict__ lcnt, int64_t ncubes,
             const double *__restrict__ xb, const double *__restrict__ axb, double *__restrict__ xa,
             double *__restrict__ axa, double *__restrict__ trans_out, double *__restrict__ w_out,
             unsigned long long *__restrict__ counters, unsigned *__restrict__ status,
             float *__restrict__ mA, double *__restrict__ mgv, const float *__restrict__ mX,
             const unsigned *__restrict__ ymax)
{
    using C = MCfg<K>;
    constexpr int CH = C::CH;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *area = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr bool U3 = ST == 3 && !MEM;      // the compact update layout (MCfg::SMEM3)
    double *B1 = reinterpret_cast<double *>(area + (ST == 1 ? C::AREA1 : U3 ? C::AREA3 : C::AREA));
    double *gv = B1 + (U3 ? 128 * (K / 8) : K * K);
    double *wbar = gv + K;
    double *misc = wbar + K;       // 2K
    double *inc = misc + 2 * K;    // 128
    float *nrm32 = reinterpret_cast<float *>(inc + 128);           // K
    float2 *rot32 = reinterpret_cast<float2 *>(nrm32 + K);          // K/2
    int *mg = reinterpret_cast<int *>(rot32 + K / 2);               // 3 x CH obs indices
    float *msq = reinterpret_cast<float *>(mg + 3 * CH);            // 3 x CH sqrt(rloc)
    float *me = msq + 3 * CH;                                       // 3 x CH e
    float *stage0 = reinterpret_cast<float *>(B1);
    float *stage1 = C::STAGE1_IN_B1 ? stage0 + CH * K : reinterpret_cast<float *>(area + 2 * C::TILE);
    __shared__ uint64_t mbar[3];
    __shared__ uint32_t s_tmem;
    __shared__ int s_rot, s_ok, s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) lg_tmem_alloc(lg_smem_u32(&s_tmem), C::TMEM_COLS);
    if (tid == 0) {
        s_fail = 0;
        lg_mbar_init(&mbar[0], 1);
        lg_mbar_init(&mbar[1], 1);
        lg_mbar_init(&mbar[2], 1);
    }
    lg_tc_fence_before();
    __syncthreads();
    lg_tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t idesc = lg_idesc_bf16(128, K);           // update: xb (hi/lo) x T
    const uint32_t idesc_a = lg_idesc_f16(128, K);          // A build: Yhat products
    // the A build's operands times 2^E (FP16 range), its products times 2^-2E
    float ysc = 1.0f, yunsc = 1.0f;
    if (ST == 0 || ST == 1) {
        const int ye = lg_f16_scale_exp(*ymax);
        ysc = lg_pow2f(ye);
        yunsc = lg_pow2f(-2 * ye);
    }
    uint32_t ncommit[3] = {0u, 0u, 0u};
    bool pending[3] = {false, false, false};
    bool failed = false;

    // Wait (thread 0 polls, at most `limit` times) for the last commit on
    // barrier b.  A wait that runs out leaves the commit pending: the drain
    // before the TMEM is freed waits for it again.  Each barrier has at most one
    // commit outstanding (a tile is waited for before it is refilled), so its
    // phase parity names that commit.
    auto wait_bar = [&](int b, uint32_t limit) -> bool {
        if (!pending[b]) return true;
        if (tid == 0) s_ok = lg_mbar_wait(&mbar[b], (ncommit[b] - 1u) & 1u, limit) ? 1 : 0;
        __syncthreads();
        const int ok = s_ok;
        __syncthreads();
        if (ok) pending[b] = false;
        return ok != 0;
    };

    // 4x4 block ownership
    int lbi[C::ML], lbj[C::ML];
    bool lok[C::ML];
#pragma unroll
    for (int m = 0; m < C::ML; m++) {
        const int b = tid + m * kT;
        lok[m] = b < C::NLOW;
        lg_decode_block(lok[m] ? b : 0, lbi[m], lbj[m]);
    }
    // A-build conversion task of this thread: columns tm, tm + 1 of the
    // observations 8 tc .. 8 tc + 7 of a chunk (tile offsets fixed for the
    // whole launch)
    const bool has_task = tid < 4 * K;
    const int tm = 2 * (tid % (K / 2)), tc = tid / (K / 2);
    const uint32_t o_h0 = lg_sw128_offset(K + tm, tc), o_l0 = lg_sw128_offset(tm, tc);
    const uint32_t o_h1 = lg_sw128_offset(K + tm + 1, tc), o_l1 = lg_sw128_offset(tm + 1, tc);
    int fbi[C::MF], fbj[C::MF];
    bool fok[C::MF];
#pragma unroll
    for (int m = 0; m < C::MF; m++) {
        const int b = tid + m * kT;
        fok[m] = b < C::NFULL;
        fbi[m] = (fok[m] ? b : 0) / C::KB;
        fbj[m] = (fok[m] ? b : 0) % C::KB;
    }

#ifdef LG_PHASE_CLOCKS
    long long ph_cyc[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    long long ph_last = clock64();
#endif
    // 128-byte lines of the background state of cube cb's columns into L2
    auto prefetch_state = [&](int64_t cb) {
        const int bjc = (int)(cb % prm.nbj), bic = (int)(cb / prm.nbj);
        const int sj = bjc * prm.cube_n, ej = min(sj + prm.cube_n - 1, g.nlat - 1);
        const int si = bic * prm.cube_n, ei = min(si + prm.cube_n - 1, g.nlon - 1);
        const int64_t lines = ((int64_t)g.n * K * (int64_t)sizeof(double) + 127) / 128;
        for (int ii = si; ii <= ei; ii++)
            for (int jj = sj; jj <= ej; jj++) {
                const int64_t col = jj + (int64_t)g.nlat * ii;
                const char *base = reinterpret_cast<const char *>(xb + col * g.n * K);
                for (int64_t l = tid; l < lines; l += kT) asm volatile("prefetch.global.L2 [%0];" ::"l"(base + l * 128));
            }
    };
    // Work queue: chunks of `chunk` consecutive cubes (neighbours along
    // latitude, so a cube's eigenvectors are a good start for the next one),
    // taken heaviest first (queue order) by an atomic cursor.
    __shared__ int s_chunk;
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
        if (ST == 0 && cube % LG_WARM_RUN == 0) have_prev = false;
        const int64_t off = loff[cube];
        const int p = lcnt[cube];
        LG_PHASE(6);
        const int64_t ci = cube - prm.cube0;                 // index of the stage intermediates
        constexpr int LDD = K + 1;                             // padded rows: conflict-free both ways
        float *Dhh = reinterpret_cast<float *>(area);
        float *Dlh = Dhh + K * LDD;
        float *W32 = reinterpret_cast<float *>(area);          // FP32 Jacobi columns (stride LDW)
        float *A32 = W32 + K * C::LDW;                          // A' in FP32 (warm start)
        float *Vprev = reinterpret_cast<float *>(area + 49152); // previous cube's X by rows, FP32
        float *X32 = reinterpret_cast<float *>(area);            // X32[j*K + r] = x_j[r]
        float *ilam32 = reinterpret_cast<float *>(misc);     // 1/lambda (misc: 2K doubles = 4K floats)
        float *hc32 = ilam32 + K, *w32 = hc32 + K, *r32 = w32 + K;
        const double cdiag = (double)(K - 1) / prm.inflation;
        (void)w32;
        (void)ci;

        if (ST == 0 || ST == 1) {
        // ---------------- phase 1: A on the tensor cores, g and diag(A) -------------
        // Tile rows: Yhat_lo (0..K-1), Yhat_hi (K..2K-1), zeros to TROWS.  The
        // A operand is rows 0..127, the B operand rows K..2K-1 (N = K), so
        // D[lo/hi m][n] = Yhat_lo/hi(m) . Yhat_hi(n).  The tensor cores'
        // accumulation drifts with the number of products summed (about 1e-8
        // of the sum per observation, one sign for sums of positive terms),
        // so the terms whose relative error reaches the analysis whole, g =
        // Yhat e (e_o = sqrt(rdiaginv rloc) dep: g = sum_o y r rloc dep) and
        // the diagonal of A, are summed on the FP32 pipe in round-to-nearest
        // by the conversion threads, which hold Yhat and e in registers; the
        // off-diagonal sums of A, whose terms cancel, stay on the tensor cores.
        unsigned long long acc_g = 0ull, acc_d = 0ull;     // packed (column tm, tm + 1)
        {
            constexpr int Z0 = 2 * K, NZ = C::TROWS - Z0;   // rows that stay zero
            for (int t = tid; t < 2 * NZ * 8; t += kT) {
                const int b = t / (NZ * 8), rest = t % (NZ * 8);
                const int r = Z0 + rest / 8, c = rest % 8;
                *reinterpret_cast<uint4 *>(area + b * C::TILE + lg_sw128_offset(r, c)) = make_uint4(0, 0, 0, 0);
            }
        }
        // Chunk x's observation rows are gathered by cp.async into stage x & 1,
        // two chunks ahead of the conversion; its list entries (index and the
        // factors sqrt(rloc), e) sit in ring slot x % 3, written before the
        // barrier after which the rows of x are requested, and are read into
        // registers one chunk before that.  Two block barriers per chunk.
        const int nch = (p + CH - 1) / CH;
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
        auto issue_rows = [&](int x) {       // all threads; ring slot x % 3 is visible
            float *st = (x & 1) ? stage1 : stage0;
            const int *gs = mg + (x % 3) * CH;
            constexpr int PPR = K / 4;        // 16-byte pieces per row
            for (int q = tid; q < CH * PPR; q += kT) {
                const int o = q / PPR, part = q % PPR;
                const int gi = gs[o];
                if (gi >= 0) cp_async16(lg_smem_u32(st + o * K + part * 4), ys32 + (int64_t)gi * K + part * 4);
            }
            cp_async_commit();               // one group per chunk, empty past the end
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
            cp_async_wait<1>();              // this chunk's rows (the next chunk's may be in flight)
            // tile b is free once the products of chunk ch - 2 are done
            if (tid == 0 && pending[b] && !lg_mbar_wait(&mbar[b], (ncommit[b] - 1u) & 1u, prm.spin_limit))
                s_fail = 1;
            __syncthreads();
            LG_PHASE(7);
            if (s_fail) {
                failed = true;         // pending[b] stays set for the drain
                break;
            }
            pending[b] = false;
            // slot (ch + 2) % 3 last served chunk ch - 1, converted before the barrier
            if (tid < CH) {
                put_meta(ch + 2, pf_g, pf_m);
                load_meta(ch + 3, pf_g, pf_m);
            }
            unsigned char *tile = area + b * C::TILE;
            const int cnt = min(CH, p - ch * CH);
            if (has_task) {
                // columns tm, tm + 1 of 8 observations: 8-byte shared loads,
                // packed scaling and split
                const float *src = st + (8 * tc) * K + tm;
                unsigned long long x[8];
                if (cnt == CH) {
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const float2 y = *reinterpret_cast<const float2 *>(src + j * K);
                        const float f = sq[8 * tc + j];
                        x[j] = lg_fmul2(lg_pk2(y.x, y.y), lg_pk2(f, f));
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        if (8 * tc + j < cnt) {
                            const float2 y = *reinterpret_cast<const float2 *>(src + j * K);
                            const float f = sq[8 * tc + j];
                            x[j] = lg_fmul2(lg_pk2(y.x, y.y), lg_pk2(f, f));
                        } else {
                            x[j] = 0ull;
                        }
                    }
                }
                uint4 h0, l0, h1, l1;
                split8x2_f16(x, h0, l0, h1, l1);
                *reinterpret_cast<uint4 *>(tile + o_h0) = h0;
                *reinterpret_cast<uint4 *>(tile + o_l0) = l0;
                *reinterpret_cast<uint4 *>(tile + o_h1) = h1;
                *reinterpret_cast<uint4 *>(tile + o_l1) = l1;
                // g and the diagonal, observation by observation (e is zero
                // past the list's end, as the rows are)
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const float e = ev[8 * tc + j];
                    acc_g = lg_ffma2(x[j], lg_pk2(e, e), acc_g);
                    acc_d = lg_ffma2(x[j], x[j], acc_d);
                }
            }
            lg_fence_async_smem();
            __syncthreads();
            LG_PHASE(9);
            if (ch > 0 && ch % LG_ACC_FLUSH == 0) {
                // the last group's sums (chunks ch - F .. ch - 1) into the
                // running ones in FP32 round to nearest (the first group's are
                // copied) before this chunk's products restart the scratch
                // accumulator; chunk ch - 2's products were waited for above
                if (!wait_bar(b ^ 1, prm.spin_limit)) {
                    failed = true;
                    break;
                }
                lg_tc_fence_after();
                if (warp < 4) {
                    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
                    for (int c0 = 0; c0 < K; c0 += 16) {
                        float v[16], u[16];
                        lg_tmem_ld16x2(tl + C::ACC1 + (uint32_t)c0, tl + (uint32_t)c0, v, u);
                        if (ch > LG_ACC_FLUSH) {
#pragma unroll
                            for (int j = 0; j < 16; j++) v[j] = u[j] + v[j];
                        }
                        lg_tmem_st16(tl + (uint32_t)c0, v);
                    }
                }
                lg_tc_fence_before();
                __syncthreads();
            }
            if (tid == 0) {
                lg_tc_fence_after();
                const uint64_t da = lg_desc_sw128(lg_smem_u32(tile));
                const uint64_t db = lg_desc_sw128(lg_smem_u32(tile + K * 128));
#pragma unroll
                for (int kk = 0; kk < 4; kk++)
                    lg_umma_bf16(tmem + C::ACC1, da + 2 * kk, db + 2 * kk, idesc_a,
                                 (ch % LG_ACC_FLUSH != 0 || kk > 0) ? 1u : 0u);
                lg_umma_commit(&mbar[b]);
            }
            ncommit[b]++;
            pending[b] = true;
            // stage b was read before the barrier, slot (ch + 2) % 3 written before it
            issue_rows(ch + 2);
            LG_PHASE(10);
        }
        cp_async_wait<0>();
        if (failed) break;
        // the partial sums of g and the diagonal through the first gather
        // stage (no copy is in flight and every chunk's rows were read before
        // the last chunk's barrier): [g | diag][tc][column]
        if (has_task) {
            float *pg = stage0 + tc * K + tm, *pd = stage0 + 8 * K + tc * K + tm;
            lg_upk2(acc_g, pg[0], pg[1]);
            lg_upk2(acc_d, pd[0], pd[1]);
        }
        // the first list entries of the next cube into L2 (its first three chunks)
        if (warp == 0 && cube + 1 < cube_end) {
            const int64_t o2 = loff[cube + 1];
            const int n2 = min(lcnt[cube + 1], 3 * CH);
            const char *li = reinterpret_cast<const char *>(lidx + o2);
            const char *lm = reinterpret_cast<const char *>(lmeta + o2);
            // addresses inside the entries only: the last line by the last byte
            const int nl = (n2 * 4 + 127) / 128 + 1, nm = (n2 * 8 + 127) / 128 + 1;
            for (int l = lane; l < nl + nm; l += 32) {
                const char *a = (l < nl) ? li + min(l * 128, n2 * 4 - 1) : lm + min((l - nl) * 128, n2 * 8 - 1);
                if (n2 > 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
            }
        }
        if (!wait_bar(0, prm.spin_limit) || !wait_bar(1, prm.spin_limit)) {
            failed = true;
            break;
        }
        lg_tc_fence_after();
        __syncthreads();
        // g and diag(A) over the 8 observation groups in a fixed order (FP64
        // sums of the FP32 partials), times 2^-2E, in misc
        if (tid < K) {
            double sg = 0.0, sd = 0.0;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                sg += (double)stage0[q * K + tid];
                sd += (double)stage0[8 * K + q * K + tid];
            }
            misc[tid] = sg * (double)yunsc;
            misc[K + tid] = sd * (double)yunsc;
        }

        LG_PHASE(0);
        // ---------------- phase 2: A' = HH + LH + LH^T + (k-1)/rho I -------------------
        if (warp < 4) {
            const int row = warp * 32 + lane;
            const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
            for (int c0 = 0; c0 < K; c0 += 16) {
                float v[16];
                if (p > 0) {
                    // the last group's sums, plus the running ones of the
                    // groups before it
                    float u[16];
                    lg_tmem_ld16x2(tl + C::ACC1 + (uint32_t)c0, tl + (uint32_t)c0, v, u);
                    if (nch > LG_ACC_FLUSH) {
#pragma unroll
                        for (int j = 0; j < 16; j++) v[j] = u[j] + v[j];
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; j++) v[j] = 0.0f;
                }
                if (row < K) {
#pragma unroll
                    for (int j = 0; j < 16; j++) Dlh[row * LDD + c0 + j] = v[j];
                } else if (row < 2 * K) {
#pragma unroll
                    for (int j = 0; j < 16; j++) Dhh[(row - K) * LDD + c0 + j] = v[j];
                }
            }
        }
        lg_tc_fence_before();
        __syncthreads();
        // A = HH + LH + LH^T is formed in FP32 (the accumulators are FP32) off
        // the diagonal, the diagonal and g from the FP32-pipe sums, then
        // A' = A + (k-1)/rho I in FP64 and in FP32 for the Jacobi
        if (tid < K) {
            gv[tid] = misc[tid];
            if (ST == 1) mgv[ci * K + tid] = gv[tid];
        }
        for (int idx = tid; idx < K * K; idx += kT) {
            const int i = idx / K, j = idx % K;
            const float a32 = i == j ? (float)misc[K + i]
                                     : (0.5f * (Dhh[i * LDD + j] + Dhh[j * LDD + i]) +
                                        (Dlh[i * LDD + j] + Dlh[j * LDD + i])) * yunsc;
            if (ST == 1) mA[ci * K * K + idx] = a32;
            else B1[idx] = (double)a32 + (i == j ? cdiag : 0.0);
        }
        __syncthreads();                                   // Dhh/Dlh are dead
        }
        if (ST == 1) continue;
        if (ST == 3) {
            // T (row-major, FP32) and wbar (FP64) from the eigensolve or the
            // FP64 refinement launch, in the slots of X and g; the next cube's
            // T, wbar and state into L2 while this one is updated
            if (!have_prev) prefetch_state(cube);
            if (cube + 1 < cube_end) {
                prefetch_state(cube + 1);
                constexpr int LA = K * K * 4 / 128, LG = (K * 8 + 127) / 128;
                for (int l = tid; l < LA + LG; l += kT) {
                    const char *a = (l < LA) ? reinterpret_cast<const char *>(mX + (ci + 1) * K * K) + l * 128
                                             : reinterpret_cast<const char *>(mgv + (ci + 1) * K) + (l - LA) * 128;
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
                }
            }
            if constexpr (!U3) {
                float *T32s = reinterpret_cast<float *>(B1);
                for (int idx = tid; idx < K * K / 4; idx += kT)
                    reinterpret_cast<float4 *>(T32s)[idx] = reinterpret_cast<const float4 *>(mX + ci * K * K)[idx];
            }
            if (tid < K) wbar[tid] = mgv[ci * K + tid];
            __syncthreads();
        }
        if (ST == 0) {
        if (!have_prev) {
            // cold start: the Jacobi works on A' itself
            for (int idx = tid; idx < K * K; idx += kT) W32[(idx / K) * C::LDW + idx % K] = (float)B1[idx];
        } else {
            // warm start from the previous (neighbouring) cube's eigenvectors:
            // the Jacobi works on A' Vprev, whose columns are nearly orthogonal
            for (int idx = tid; idx < K * K; idx += kT) A32[idx] = (float)B1[idx];
            __syncthreads();
#pragma unroll
            for (int m = 0; m < C::MF; m++) {
                if (!fok[m]) continue;
                float acc[16];
#pragma unroll
                for (int i = 0; i < 16; i++) acc[i] = 0.0f;
                for (int l = 0; l < K; l++) {
                    // A' symmetric: rows 4*fbi.. of column l = row l at 4*fbi..
                    const float4 av = *reinterpret_cast<const float4 *>(A32 + l * K + 4 * fbi[m]);
                    const float4 vv = *reinterpret_cast<const float4 *>(Vprev + l * K + 4 * fbj[m]);
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
                        W32[(4 * fbj[m] + jj) * C::LDW + 4 * fbi[m] + i] = acc[i * 4 + jj];
            }
        }
        __syncthreads();

        LG_PHASE(1);
        // ---------------- phase 3: FP32 Jacobi -> Xhat (columns of W32) ----------------
        int sw;
        if constexpr (K == 64)
            sw = lg_jacobi32b2<K, C::LDW, K>(W32, W32 + 2 * (K / 4) * 2 * K, &s_rot, LG_MIXED_JACOBI_TOL, 24);
        else if constexpr ((K & (K - 1)) == 0) sw = lg_jacobi32h<K, C::G, C::LDW>(W32, &s_rot, LG_MIXED_JACOBI_TOL, 24);
        else sw = lg_jacobi32<K, C::G, C::LDW>(W32, nrm32, &s_rot, LG_MIXED_JACOBI_TOL,
                                          LG_JACOBI32W_QSTOP > 0.0f ? LG_JACOBI32W_QSTOP : LG_MIXED_JACOBI_TOL, 24);
        if (tid == 0) {
            atomicMax(&counters[LG_CNT_MAXSWEEP], (unsigned long long)sw);
            atomicAdd(&counters[LG_CNT_SUMSWEEP], (unsigned long long)sw);
            if (sw > 24) atomicAdd(&counters[LG_CNT_NOTCONV], 1ull);
        }
        // lambda_j = |w_j| (A' is SPD, so the converged columns are lambda_j x_j),
        // one warp per column
        for (int j = warp; j < K; j += kT / 32) {
            float s = 0.0f;
            for (int r = lane; r < K; r += 32) s = fmaf(W32[j * C::LDW + r], W32[j * C::LDW + r], s);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) {
                const float lamf = sqrtf(s);
                nrm32[j] = 1.0f / lamf;
                ilam32[j] = 1.0f / lamf;
                hc32[j] = sqrtf((float)(K - 1) / lamf);   // f_j = sqrt((k-1)/lambda_j)
            }
        }
        __syncthreads();
        // condition number check: the FP32 eigenpairs are accurate to about
        // eps32 * lambda_max / lambda_min
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
        LG_PHASE(2);
        // ---------------- phase 4: X, wbar with one refinement step ------------------------
        // X by columns in FP32 (T, wbar, warm start).  W32 shares this memory, so
        // the values pass through registers first.
        {
            constexpr int PER = (K * K + kT - 1) / kT;
            float xv[PER];
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const int idx = tid + q * kT;
                xv[q] = (idx < K * K) ? W32[(idx / K) * C::LDW + idx % K] * nrm32[idx / K] : 0.0f;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const int idx = tid + q * kT;
                if (idx < K * K) X32[idx] = xv[q];
            }
        }
        }
        if constexpr (ST != 3) {
        if (tid < K) {
            nrm32[tid] = hc32[tid];                    // f for T
            r32[tid] = (float)gv[tid];                 // right-hand side of the first solve
        }
        __syncthreads();
        // wbar = X diag(1/lambda) X^T g in FP32, then one refinement step:
        // wbar += X diag(1/lambda) X^T (g - A' wbar) with the residual in FP64
        // against the FP64 A' (in B1).  The FP32 solve has a relative error of
        // about eps32 kappa; the step leaves the error of the FP32 eigenpairs
        // times that, far below the FP32 representation of A.
        for (int it = 0; it < 2; it++) {
            for (int j = warp; j < K; j += kT / 32) {          // one warp per eigenvector
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
                // four threads per row of A' (FP64, in B1), each over K/4 columns
                constexpr int Q = K / 4;
                for (int t0 = 0; t0 < 4 * K; t0 += kT) {
                    const int t = t0 + tid, i = t >> 2, q = t & 3;
                    double d = 0.0;
                    if (t < 4 * K) {
#pragma unroll 4
                        for (int l = q * Q; l < q * Q + Q; l++) d = fma(B1[i * K + l], wbar[l], d);
                    }
                    d += __shfl_xor_sync(0xffffffffu, d, 1);
                    d += __shfl_xor_sync(0xffffffffu, d, 2);
                    if (t < 4 * K && q == 0) r32[i] = (float)(gv[i] - d);
                }
                __syncthreads();
            }
        }
        }   // ST != 3
        LG_PHASE(3);

        // ---------------- phase 5: T in FP32 ------------------------------------------------
        // start moving this cube's background state into L2 for the update
        // (stage 3 has no T to form first: it fetches a cube ahead instead)
        if (ST != 3) prefetch_state(cube);
        // T = X diag(f) X^T only feeds the BF16 hi/lo tensor-core update (16
        // significant bits); FP32 eigenpairs give it to ~1e-7 relative.
        float *T32 = reinterpret_cast<float *>(B1);               // T, FP32, row-major
        if constexpr (ST != 3) {
            float tacc[C::ML][16];
#pragma unroll
            for (int m = 0; m < C::ML; m++) {
#pragma unroll
                for (int i = 0; i < 16; i++) tacc[m][i] = 0.0f;
                if (!lok[m]) continue;
                for (int j = 0; j < K; j++) {
                    const float f = nrm32[j];
                    const float4 av = *reinterpret_cast<const float4 *>(X32 + j * K + 4 * lbi[m]);
                    const float4 bv = *reinterpret_cast<const float4 *>(X32 + j * K + 4 * lbj[m]);
                    const float a[4] = {av.x, av.y, av.z, av.w};
                    const float bq[4] = {bv.x * f, bv.y * f, bv.z * f, bv.w * f};
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int jj = 0; jj < 4; jj++) tacc[m][i * 4 + jj] = fmaf(a[i], bq[jj], tacc[m][i * 4 + jj]);
                }
            }
            // keep X by rows for the next cube's warm start
            if (ST == 0)
                for (int idx = tid; idx < K * K; idx += kT) {
                    const int r = idx / K, j = idx % K;
                    Vprev[idx] = X32[j * K + r];
                }
            // B1 (A') was last read before the previous barrier
#pragma unroll
            for (int m = 0; m < C::ML; m++) {
                if (!lok[m]) continue;
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) {
                        const int r = 4 * lbi[m] + i, c = 4 * lbj[m] + jj;
                        T32[r * K + c] = tacc[m][i * 4 + jj];
                        T32[c * K + r] = tacc[m][i * 4 + jj];
                    }
            }
        }
        __syncthreads();
        if (trans_out) {
            for (int idx = tid; idx < K * K; idx += kT) {
                const int i = idx % K, j = idx / K;
                const float tij = U3 ? mX[ci * K * K + i * K + j] : T32[i * K + j];
                trans_out[(int64_t)cube * K * K + idx] = (double)tij + wbar[i];
            }
            if (tid < K) w_out[(int64_t)cube * K + tid] = wbar[tid];
            __syncthreads();
        }
        // The analysis mean is the member mean of axb + xb^T (T + wbar 1^T)
        // (xb_2_xa, letkf_compute.F90:283-295), and the member mean of xb^T T
        // is sqrt(rho) xbar exactly: Yhat 1 = 0 (H centres the members), so
        // A' 1 = (k-1)/rho 1 and T 1 = sqrt(rho) 1.  It is taken in the FP64
        // increment, xb^T (wbar + sqrt(rho)/k 1), rather than from the tensor
        // products, whose BF16 hi/lo error (~2^-16 of xb) would reach the mean.
        if (tid < K) wbar[tid] += sqrt(prm.inflation) / (double)K;
        __syncthreads();

        LG_PHASE(4);
        // ---------------- phase 6: xa = xb^T (T + wbar 1^T) -------------------------------
        unsigned char *xa_hi = area, *xa_lo = area + 16384;
        unsigned char *tb_hi = area + 32768, *tb_lo = area + 40960;
        // B operand rows e = T row e (T symmetric), K dimension = source member
        for (int t = tid; t < K * (K / 8); t += kT) {
            const int e = t / (K / 8), c = t % (K / 8);
            float v[8];
            if constexpr (U3) {
                const float4 *tg = reinterpret_cast<const float4 *>(mX + ci * K * K + e * K + 8 * c);
                const float4 a = tg[0], bq = tg[1];
                v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
                v[4] = bq.x; v[5] = bq.y; v[6] = bq.z; v[7] = bq.w;
            } else {
#pragma unroll
                for (int j = 0; j < 8; j++) v[j] = T32[e * K + 8 * c + j];
            }
            uint4 hi, lo;
            split8(v, hi, lo);
            *reinterpret_cast<uint4 *>(tb_hi + lg_sw128_offset(e, c)) = hi;
            *reinterpret_cast<uint4 *>(tb_lo + lg_sw128_offset(e, c)) = lo;
        }
        const int n = g.n;
        // FP64 mean increment xb^T wbar: partial sums over 8 members, [c][row],
        // after T in the space of A' (free in this phase)
        double *incp = U3 ? B1 : reinterpret_cast<double *>(T32 + K * K);
        // fused members run: squared perturbations summed over 8 members,
        // [c][row], beside the mean-increment partials (k >= 48) or after the
        // warm-start vectors (k = 32)
        constexpr bool SQ_IN_B1 = 128 * K + 64 * K <= 4 * K * K;
        float *sqp = SQ_IN_B1 ? reinterpret_cast<float *>(incp + 128 * (K / 8))
                              : reinterpret_cast<float *>(area + 49152 + K * K * sizeof(float));
        static_assert(128 * K <= 4 * K * K, "mean-increment partials must fit beside T");
        static_assert(SQ_IN_B1 || 49152 + (K * K + 16 * K) * sizeof(float) <= C::AREA, "members partials");
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
                    if constexpr (MEM) {
                        // full members in: each row's mean (sum / real(ens),
                        // module_da_parallel.F90:194-199) into inc, from
                        // partial sums over 8 members.  A NaN member makes its
                        // row's sum NaN; only such a row is checked member by
                        // member (module_da_parallel.F90:188-193 tests isnan)
                        for (int t = tid; t < 128 * (K / 8); t += kT) {
                            const int r = t / (K / 8), c = t % (K / 8);
                            if (r >= R) continue;
                            const double2 *src =
                                reinterpret_cast<const double2 *>(xbc + (int64_t)(r0 + r) * K + 8 * c);
                            double s = 0.0;
#pragma unroll
                            for (int j = 0; j < 4; j++) {
                                const double2 q = src[j];
                                s += q.x + q.y;
                            }
                            incp[c * 128 + r] = s;
                        }
                        __syncthreads();
                        if (tid < R) {
                            double s = 0.0;
#pragma unroll
                            for (int c = 0; c < K / 8; c++) s += incp[c * 128 + tid];
                            inc[tid] = s / (double)(float)K;
                            if (isnan(s)) {
                                bool bad = false;
                                for (int e = 0; e < K; e++) bad |= isnan(xbc[(int64_t)(r0 + tid) * K + e]);
                                if (bad) atomicOr(status, LG_ST_BAD_STATE);
                            }
                        }
                        __syncthreads();
                    }
                    for (int t = tid; t < 128 * (K / 8); t += kT) {
                        const int r = t / (K / 8), c = t % (K / 8);
                        float v[8];
                        if (r < R) {
                            const double2 *src =
                                reinterpret_cast<const double2 *>(xbc + (int64_t)(r0 + r) * K + 8 * c);
                            const double mb = MEM ? inc[r] : 0.0;
                            double s = 0.0;
                            float q2 = 0.0f;
#pragma unroll
                            for (int j = 0; j < 4; j++) {
                                double2 q = src[j];
                                if constexpr (MEM) {
                                    q.x -= mb;
                                    q.y -= mb;
                                }
                                v[2 * j] = (float)q.x;
                                v[2 * j + 1] = (float)q.y;
                                if constexpr (MEM) q2 = fmaf(v[2 * j], v[2 * j], fmaf(v[2 * j + 1], v[2 * j + 1], q2));
                                s = fma(q.x, wbar[8 * c + 2 * j], s);
                                s = fma(q.y, wbar[8 * c + 2 * j + 1], s);
                            }
                            incp[c * 128 + r] = s;
                            if constexpr (MEM) sqp[c * 128 + r] = q2;
                        } else {
#pragma unroll
                            for (int j = 0; j < 8; j++) v[j] = 0.0f;
                        }
                        uint4 hi, lo;
                        split8(v, hi, lo);
                        *reinterpret_cast<uint4 *>(xa_hi + lg_sw128_offset(r, c)) = hi;
                        *reinterpret_cast<uint4 *>(xa_lo + lg_sw128_offset(r, c)) = lo;
                    }
                    lg_fence_async_smem();
                    __syncthreads();
                    if (tid == 0) {
                        lg_tc_fence_after();
                        const uint64_t dh = lg_desc_sw128(lg_smem_u32(xa_hi)), dl = lg_desc_sw128(lg_smem_u32(xa_lo));
                        const uint64_t th = lg_desc_sw128(lg_smem_u32(tb_hi)), tl = lg_desc_sw128(lg_smem_u32(tb_lo));
#pragma unroll
                        for (int kk = 0; kk < K / 16; kk++) {
                            lg_umma_bf16(tmem, dh + 2 * kk, th + 2 * kk, idesc, kk > 0 ? 1u : 0u);
                            lg_umma_bf16(tmem, dh + 2 * kk, tl + 2 * kk, idesc, 1u);
                            lg_umma_bf16(tmem, dl + 2 * kk, th + 2 * kk, idesc, 1u);
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
                    if constexpr (ST == 3 && !MEM) {
                        // all 8 warps: warp w reads row quadrant w % 4 (the
                        // tensor-memory lanes it may access) and members
                        // (w / 4) K/2 .. +K/2 - 1.  The member mean keeps the
                        // summation order of the one-warp form: the first
                        // half's eight partial sums go to the second half
                        // through shared memory, which continues them and
                        // hands the mean back.
                        const int q4 = warp & 3, hh = warp >> 2;
                        const int r = q4 * 32 + lane;
                        float *xch = reinterpret_cast<float *>(area + 49152);   // [row][8 partials, mean]
                        float v[K / 2];
#pragma unroll
                        for (int c0 = 0; c0 < K / 2; c0 += 16)
                            lg_tmem_ld16(tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(hh * (K / 2) + c0), v + c0);
                        float part[8];
#pragma unroll
                        for (int q = 0; q < 8; q++) part[q] = 0.0f;
                        if (hh == 0) {
#pragma unroll
                            for (int e = 0; e < K / 2; e++) part[e & 7] += v[e];
#pragma unroll
                            for (int q = 0; q < 8; q++) xch[r * 9 + q] = part[q];
                        }
                        __syncthreads();
                        if (hh == 1) {
#pragma unroll
                            for (int q = 0; q < 8; q++) part[q] = xch[r * 9 + q];
#pragma unroll
                            for (int e = 0; e < K / 2; e++) part[(K / 2 + e) & 7] += v[e];
                            xch[r * 9 + 8] = (((part[0] + part[1]) + (part[2] + part[3])) +
                                              ((part[4] + part[5]) + (part[6] + part[7]))) /
                                             (float)K;
                        }
                        __syncthreads();
                        if (r < R) {
                            const float meanf = xch[r * 9 + 8];
                            const int64_t row = col * n + r0 + r;
                            double *dst = xac + (int64_t)(r0 + r) * K + hh * (K / 2);
                            if (hh == 0) {
                                double incr = incp[r];
#pragma unroll
                                for (int c = 1; c < K / 8; c++) incr += incp[c * 128 + r];
                                axa[row] = axb[row] + incr;
                            }
#pragma unroll
                            for (int e = 0; e < K / 2; e += 2)
                                *reinterpret_cast<double2 *>(dst + e) =
                                    make_double2(lg_f2d_bits(v[e] - meanf), lg_f2d_bits(v[e + 1] - meanf));
                        }
                    } else if (warp < 4) {
                        const int r = warp * 32 + lane;
                        float v[K];
#pragma unroll
                        for (int c0 = 0; c0 < K; c0 += 16)
                            lg_tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v + c0);
                        if (r < R) {
                            // member mean and perturbations in FP32 (the products
                            // are FP32 sums of BF16 hi/lo terms), written as FP64
                            // with the conversion on the integer pipe
                            float part[8];
#pragma unroll
                            for (int q = 0; q < 8; q++) part[q] = 0.0f;
#pragma unroll
                            for (int e = 0; e < K; e++) part[e & 7] += v[e];
                            const float meanf =
                                (((part[0] + part[1]) + (part[2] + part[3])) + ((part[4] + part[5]) + (part[6] + part[7]))) /
                                (float)K;
                            double incr = incp[r];
#pragma unroll
                            for (int c = 1; c < K / 8; c++) incr += incp[c * 128 + r];
                            const int64_t row = col * n + r0 + r;
                            double *dst = xac + (int64_t)(r0 + r) * K;
                            if constexpr (!MEM) {
                                axa[row] = axb[row] + incr;
#pragma unroll
                                for (int e = 0; e < K; e += 2)
                                    *reinterpret_cast<double2 *>(dst + e) =
                                        make_double2(lg_f2d_bits(v[e] - meanf), lg_f2d_bits(v[e + 1] - meanf));
                            } else {
                                members_epilogue<K>(prm, g, col, r, xbc + (int64_t)(r0 + r) * K, xa_hi, xa_lo,
                                                    inc[r], incr, meanf, v, sqp, dst, row);
                            }
                        }
                    }
                    lg_tc_fence_before();
                    __syncthreads();
                }
            }
        LG_PHASE(5);
        if (failed) break;
        have_prev = true;
    }
    if (failed) break;
    }
#ifdef LG_PHASE_CLOCKS
    if (blockIdx.x == 0 && tid == 0)
        printf("phase cycles cta0 (K %d, stage %d): A-build %lld (rows and tile wait %lld, unused %lld, "
               "convert %lld, issue %lld), A'-form %lld, jacobi32 %lld, X/wbar %lld, T %lld, update %lld, loop %lld\n",
               K, ST, ph_cyc[0] + ph_cyc[7] + ph_cyc[8] + ph_cyc[9] + ph_cyc[10], ph_cyc[7], ph_cyc[8], ph_cyc[9],
               ph_cyc[10], ph_cyc[1], ph_cyc[2], ph_cyc[3], ph_cyc[4], ph_cyc[5], ph_cyc[6]);
#endif
    if (failed && tid == 0) atomicOr(status, LG_ST_TIMEOUT);
    cp_async_wait<0>();
    // let every committed MMA finish before the TMEM is freed: a wait that ran
    // out left its commit pending, and the drain waits for it at the normal
    // limit whatever limit the run's waits had
    bool drained = true;
    for (int b = 0; b < 3; b++) drained = wait_bar(b, LG_MBAR_SPIN_LIMIT) && drained;
    if (!drained && tid == 0) atomicOr(status, LG_ST_TIMEOUT);
    lg_tc_fence_before();
    __syncthreads();
    lg_tc_fence_after();
    if (warp == 0) lg_tmem_dealloc(tmem, C::TMEM_COLS);
}

constexpr int kQueueMax = 8192;      // chunks one queue-building CTA sorts in shared memory

// The work queue of the mixed core: chunk weights sum(p + p0) over each
// chunk's cubes (p0: the per-cube work that does not grow with p, in
// observation equivalents), sorted heaviest first (bitonic, one CTA).
__global__ void __launch_bounds__(1024)
k_chunk_queue(const int32_t *__restrict__ lcnt, int64_t win0, int64_t win1, int chunk, int nchunks, int p0,
              int *__restrict__ queue)
{
    const int64_t base = win0 / chunk * chunk;
    extern __shared__ unsigned long long qkeys[];
    int np2 = 1;
    while (np2 < nchunks) np2 <<= 1;
    for (int i = threadIdx.x; i < np2; i += blockDim.x) {
        unsigned long long key = 0ull;
        if (i < nchunks) {
            unsigned long long w = 0;
            const int64_t c0 = max(win0, base + (int64_t)i * chunk);
            const int64_t c1 = min(win1, base + (int64_t)(i + 1) * chunk);
            for (int64_t c = c0; c < c1; c++) w += (unsigned long long)(lcnt[c] + p0);
            key = (w << 32) | (unsigned)i;
        }
        qkeys[i] = key;
    }
    __syncthreads();
    for (int k2 = 2; k2 <= np2; k2 <<= 1)
        for (int j = k2 >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < np2; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = qkeys[i], b = qkeys[ixj];
                    const bool desc = (i & k2) == 0;
                    if ((a < b) == desc) {
                        qkeys[i] = b;
                        qkeys[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < nchunks; i += blockDim.x) queue[i] = (int)(qkeys[i] & 0xffffffffull);
}

// The eigensolve runs run0 .. run0 + nruns - 1 ordered by their cost in the
// last call (sweeps summed over the run), longest first, ties in run order
// (bitonic, one CTA; nruns <= kQueueMax).
__global__ void __launch_bounds__(1024)
k_run_order(const int *__restrict__ runcost, int64_t run0, int nruns, int *__restrict__ order)
{
    extern __shared__ unsigned long long rkeys[];
    int np2 = 1;
    while (np2 < nruns) np2 <<= 1;
    for (int i = threadIdx.x; i < np2; i += blockDim.x) {
        unsigned long long key = 0ull;
        if (i < nruns) {
            const unsigned long long w = (unsigned long long)(unsigned)max(runcost[run0 + i], 0);
            key = (w << 32) | (0xffffffffu - (unsigned)i);
        }
        rkeys[i] = key;
    }
    __syncthreads();
    for (int k2 = 2; k2 <= np2; k2 <<= 1)
        for (int j = k2 >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < np2; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = rkeys[i], b = rkeys[ixj];
                    const bool desc = (i & k2) == 0;
                    if ((a < b) == desc) {
                        rkeys[i] = b;
                        rkeys[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < nruns; i += blockDim.x) order[i] = (int)(0xffffffffu - (unsigned)(rkeys[i] & 0xffffffffull));
}

}  // namespace

// Cubes per work-queue chunk for the run's cube range: the context's
// schedule (16 by default; at least LG_WARM_RUN for the one-launch cores, so
// that chunks hold whole warm-start runs), grown until any window of the
// range takes at most kQueueMax chunks.  Windows end on chunk boundaries.
int lg_run_chunk(const letkf_ctx *ctx)
{
    const int64_t n = ctx->range1 - ctx->range0;
    int chunk = ctx->sched_chunk > 0 ? ctx->sched_chunk : 16;
    if (ctx->k != 64 && chunk < LG_WARM_RUN) chunk = LG_WARM_RUN;
    while ((n + chunk - 1) / chunk + 1 > kQueueMax) chunk *= 2;
    return chunk;
}

// Build the mixed core's work queue for the cubes of the last search (the
// window win0 .. win1 - 1): the chunks of lg_run_chunk cubes that meet the
// window (aligned to multiples of the chunk size in cube numbering), heaviest
// first, into ctx->d_queue.  The staged k = 64 core's launches (the A build
// and the update: no warm start) halve the chunk, down to 8 cubes, while the
// window has fewer than 8 chunks per A-build CTA: the blocks of a run that
// goes back to host memory are small, and with two chunks per CTA the
// heaviest ones leave a tail (1.6 ms of A build over the three blocks at the
// 1-degree configuration).  The chunk only decides which CTA takes which
// cubes, so the analysis is the same.
cudaError_t lg_build_chunk_queue(letkf_ctx *ctx, int &chunk, int &nchunks)
{
    chunk = lg_run_chunk(ctx);
    if (ctx->k == 64) {
        int nsm = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
        const int64_t want = 8LL * 3 * (nsm > 0 ? nsm : 152), n = ctx->win1 - ctx->win0;
        while (chunk > 8 && (n + chunk - 1) / chunk < want && 2 * ((n + chunk - 1) / chunk) + 2 <= kQueueMax)
            chunk /= 2;
    }
    const int64_t base = ctx->win0 / chunk * chunk;
    nchunks = (int)((ctx->win1 - base + chunk - 1) / chunk);
    cudaError_t e = ctx->d_queue.reserve((size_t)nchunks);
    if (e != cudaSuccess) return e;
    int np2 = 1;
    while (np2 < nchunks) np2 <<= 1;
    const size_t qsmem = sizeof(unsigned long long) * np2;
    e = cudaFuncSetAttribute(k_chunk_queue, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)qsmem);
    if (e != cudaSuccess) return e;
    lg_count_launch();
    k_chunk_queue<<<1, 1024, qsmem, ctx->stream>>>(ctx->d_lcnt.p, ctx->win0, ctx->win1, chunk, nchunks,
                                                   ctx->sched_p0 > 0 ? ctx->sched_p0 : 4400, ctx->d_queue.p);
    return cudaGetLastError();
}

namespace {

// Eigenpairs of A' = A + (k-1)/rho I for the cubes cube0 .. cube_end-1, one
// warp per eigenproblem (the staged form of k_core_mixed): each lane owns a
// column pair of the one-sided Jacobi in registers (lg_jacobi32w), so a step
// needs no block barrier and moves columns by shuffles.  The cubes go in runs
// of R consecutive cubes aligned to multiples of R in cube numbering; inside a
// run each cube starts from the previous one's
// eigenvectors, W = A' V_prev, the first cold from W = A'.  Writes x_j
// (columns, FP32, [j][r]) and lambda_j, and the sweep and conditioning
// counters.
#ifndef LG_EIG_THREADS
#define LG_EIG_THREADS 384
#endif
constexpr int kTE = LG_EIG_THREADS;     // threads of an eigensolve block (one problem per warp)

template <int K>
__global__ void __launch_bounds__(kTE, 1)
k_eig_warp(int64_t cube0, int64_t cube_end, int R, double cdiag, float tol, const float *__restrict__ mA,
           float *__restrict__ mX, float *__restrict__ mlam, double *__restrict__ mgv, int emit_tw,
           unsigned long long *__restrict__ counters, const int *__restrict__ order, int *__restrict__ runcost)
{
    constexpr int LDW = K + 4, NS = K / 2;
    static_assert(NS == 32, "one lane per column pair");
    extern __shared__ float smw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *Wp = smw + (size_t)warp * K * LDW;           // this warp's columns
    // this warp's vectors (emit_tw): wbar (FP64), then g or the residual,
    // X^T g / lambda, f = sqrt((k-1)/lambda) and 1/lambda (FP32)
    double *wv = reinterpret_cast<double *>(smw + (size_t)(kTE / 32) * K * LDW) + (size_t)warp * 3 * K;
    float *gs = reinterpret_cast<float *>(wv + K), *cs = gs + K, *fs = cs + K, *ils = fs + K;
    const int64_t base = cube0 / R * R;
    const int64_t nruns = (cube_end - base + R - 1) / R;
    const float cd = (float)cdiag;
#ifdef LG_PHASE_CLOCKS
    long long ec[3] = {0, 0, 0}, et = clock64();
#define LG_EPHASE(i)                                   \
    do {                                               \
        const long long n_ = clock64();                \
        ec[i] += n_ - et;                              \
        et = n_;                                       \
    } while (0)
#else
#define LG_EPHASE(i) \
    do {             \
    } while (0)
#endif
    for (;;) {
        // the next run from the queue cursor (runs cost different numbers of
        // sweeps, so a fixed deal leaves some warps with the longest tail)
        int64_t run = 0;
        if (lane == 0) run = (int64_t)atomicAdd(&counters[LG_CNT_QUEUE], 1ull);
        run = __shfl_sync(0xffffffffu, run, 0);
        if (run >= nruns) break;
        // longest runs of the last call first (the order only decides which
        // warp takes a run; each run is solved the same way)
        if (order) run = order[run];
        int run_sweeps = 0;
        const int64_t c0 = max(cube0, base + run * R), c1 = min(cube_end, base + (run + 1) * R);
        for (int64_t c = c0; c < c1; c++) {
            const float *Ac = mA + (c - cube0) * K * K;
            // W columns lane and lane + NS into Wp (each lane reads and writes
            // only its own two columns)
            if (c == c0) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    // cold: column j of A' is row j (A' symmetric)
                    const int j = lane + h * NS;
                    float4 *dst = reinterpret_cast<float4 *>(Wp + j * LDW);
                    const float4 *row = reinterpret_cast<const float4 *>(Ac + j * K);
#pragma unroll
                    for (int q = 0; q < K / 4; q++) {
                        float4 x = row[q];
                        if (4 * q == (j & ~3)) {
                            const int r = j & 3;
                            if (r == 0) x.x += cd; else if (r == 1) x.y += cd; else if (r == 2) x.z += cd; else x.w += cd;
                        }
                        dst[q] = x;
                    }
                }
            } else {
                // warm: w_j = A' v_j = sum_l A[l][:] v_j[l] + cd v_j for both columns
                // in one pass over A (A symmetric; all lanes read the same row of
                // A at once, each its own v_j[l])
                const float *v0 = Wp + lane * LDW, *v1 = Wp + (lane + NS) * LDW;
                unsigned long long acc0[K / 2], acc1[K / 2];
#pragma unroll
                for (int q = 0; q < K / 4; q++) {
                    const float4 x = reinterpret_cast<const float4 *>(v0)[q];
                    const float4 y = reinterpret_cast<const float4 *>(v1)[q];
                    acc0[2 * q] = lg_pk2(cd * x.x, cd * x.y);
                    acc0[2 * q + 1] = lg_pk2(cd * x.z, cd * x.w);
                    acc1[2 * q] = lg_pk2(cd * y.x, cd * y.y);
                    acc1[2 * q + 1] = lg_pk2(cd * y.z, cd * y.w);
                }
#pragma unroll 1
                for (int l = 0; l < K; l++) {
                    const float4 *row = reinterpret_cast<const float4 *>(Ac + l * K);
                    const float a0 = v0[l], a1 = v1[l];
                    const unsigned long long p0 = lg_pk2(a0, a0), p1 = lg_pk2(a1, a1);
#pragma unroll
                    for (int q = 0; q < K / 4; q++) {
                        const float4 x = row[q];
                        const unsigned long long xl = lg_pk2(x.x, x.y), xh = lg_pk2(x.z, x.w);
                        acc0[2 * q] = lg_ffma2(xl, p0, acc0[2 * q]);
                        acc0[2 * q + 1] = lg_ffma2(xh, p0, acc0[2 * q + 1]);
                        acc1[2 * q] = lg_ffma2(xl, p1, acc1[2 * q]);
                        acc1[2 * q + 1] = lg_ffma2(xh, p1, acc1[2 * q + 1]);
                    }
                }
                __syncwarp();                  // every lane has read its v_j before W replaces them
#pragma unroll
                for (int q = 0; q < K / 4; q++) {
                    float a, b, cc, d;
                    lg_upk2(acc0[2 * q], a, b);
                    lg_upk2(acc0[2 * q + 1], cc, d);
                    reinterpret_cast<float4 *>(Wp + lane * LDW)[q] = make_float4(a, b, cc, d);
                    lg_upk2(acc1[2 * q], a, b);
                    lg_upk2(acc1[2 * q + 1], cc, d);
                    reinterpret_cast<float4 *>(Wp + (lane + NS) * LDW)[q] = make_float4(a, b, cc, d);
                }
            }
            // the next cube's A into L2 while this one is solved (16 KB, 128 lines)
            if (c + 1 < c1) {
                const char *nxt = reinterpret_cast<const char *>(Ac + K * K);
                for (int l = lane; l < K * K * 4 / 128; l += 32)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(nxt + l * 128));
            }
            __syncwarp();
            LG_EPHASE(0);
            const int sw = lg_jacobi32w<K, LDW>(Wp, tol, 24);
            run_sweeps += sw;
            LG_EPHASE(1);
            // lambda_j = |w_j|, x_j = w_j / lambda_j (kept in Wp for the next cube)
            float lo = 3.0e38f, hi = 0.0f;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = lane + h * NS;
                float4 *col = reinterpret_cast<float4 *>(Wp + j * LDW);
                float s = 0.0f;
#pragma unroll
                for (int q = 0; q < K / 4; q++) {
                    const float4 x = col[q];
                    s = fmaf(x.x, x.x, fmaf(x.y, x.y, fmaf(x.z, x.z, fmaf(x.w, x.w, s))));
                }
                const float lamf = sqrtf(s), il = 1.0f / lamf;
                float4 *out = reinterpret_cast<float4 *>(mX + (c - cube0) * K * K + j * K);
#pragma unroll
                for (int q = 0; q < K / 4; q++) {
                    float4 x = col[q];
                    x.x *= il; x.y *= il; x.z *= il; x.w *= il;
                    col[q] = x;
                    if (!emit_tw) out[q] = x;
                }
                if (!emit_tw) {
                    mlam[(c - cube0) * K + j] = lamf;
                } else {
                    fs[j] = sqrtf((float)(K - 1) / lamf);
                    ils[j] = il;
                }
                lo = fminf(lo, lamf);
                hi = fmaxf(hi, lamf);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            if (lane == 0) {
                atomicMax(&counters[LG_CNT_MAXSWEEP], (unsigned long long)sw);
                atomicAdd(&counters[LG_CNT_SUMSWEEP], (unsigned long long)sw);
                if (sw > 24) atomicAdd(&counters[LG_CNT_NOTCONV], 1ull);
                if (hi > 1.0e4f * lo) atomicAdd(&counters[LG_CNT_ILLCOND], 1ull);
            }
            __syncwarp();
            if (emit_tw) {
                // wbar = X diag(1/lambda) X^T g in FP32, then one refinement
                // step wbar += X diag(1/lambda) X^T (g - A' wbar) with the
                // residual in FP64 against A' = (double)A + (k-1)/rho I; the
                // FP32 solve has a relative error of about eps32 kappa, the step
                // leaves that times the FP32 eigenpairs' error.  Then T = X
                // diag(sqrt((k-1)/lambda)) X^T in FP32 (it feeds the BF16 hi/lo
                // update).  wbar goes over g in mgv, T (row-major) over X's slot.
                const int64_t ci = c - cube0;
                const double g0 = mgv[ci * K + lane], g1 = mgv[ci * K + lane + NS];
                gs[lane] = (float)g0;
                gs[lane + NS] = (float)g1;
                double w0 = 0.0, w1 = 0.0;
                for (int it = 0; it < 2; it++) {
                    __syncwarp();
                    // c_j = x_j . rhs / lambda_j for this lane's two columns
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int j = lane + h * NS;
                        const float4 *col = reinterpret_cast<const float4 *>(Wp + j * LDW);
                        const float4 *rv = reinterpret_cast<const float4 *>(gs);
                        float d0 = 0.0f, d1 = 0.0f;
#pragma unroll
                        for (int q = 0; q < K / 4; q++) {
                            const float4 x = col[q], y = rv[q];
                            d0 = fmaf(x.x, y.x, fmaf(x.y, y.y, d0));
                            d1 = fmaf(x.z, y.z, fmaf(x.w, y.w, d1));
                        }
                        cs[j] = (d0 + d1) * ils[j];
                    }
                    __syncwarp();
                    // rows lane and lane + NS of X c
                    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll 8
                    for (int j = 0; j < K; j++) {
                        const float cj = cs[j];
                        a0 = fmaf(Wp[j * LDW + lane], cj, a0);
                        a1 = fmaf(Wp[j * LDW + lane + NS], cj, a1);
                    }
                    w0 += (double)a0;
                    w1 += (double)a1;
                    if (it == 1) break;
                    wv[lane] = w0;
                    wv[lane + NS] = w1;
                    __syncwarp();
                    // residual rows lane and lane + NS in FP64 (A symmetric:
                    // row r of A from the build launch, FP32 values converted
                    // exactly on the integer pipe)
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int r = lane + h * NS;
                        const float4 *arow = reinterpret_cast<const float4 *>(mA + ci * K * K + r * K);
                        double d = 0.0;
#pragma unroll 4
                        for (int q = 0; q < K / 4; q++) {
                            const float4 a = arow[q];
                            d = fma(lg_f2d_bits(a.x), wv[4 * q], d);
                            d = fma(lg_f2d_bits(a.y), wv[4 * q + 1], d);
                            d = fma(lg_f2d_bits(a.z), wv[4 * q + 2], d);
                            d = fma(lg_f2d_bits(a.w), wv[4 * q + 3], d);
                        }
                        d = fma(cdiag, wv[r], d);
                        gs[r] = (float)((h ? g1 : g0) - d);
                    }
                }
                mgv[ci * K + lane] = w0;
                mgv[ci * K + lane + NS] = w1;
                // T rows lane and lane + NS, one at a time: sum_j f_j x_j[r] x_j
#pragma unroll 1
                for (int h = 0; h < 2; h++) {
                    const int r = lane + h * NS;
                    unsigned long long t0[K / 2];
#pragma unroll
                    for (int q = 0; q < K / 2; q++) t0[q] = 0ull;
#pragma unroll 2
                    for (int j = 0; j < K; j++) {
                        const float b0 = fs[j] * Wp[j * LDW + r];
                        const unsigned long long p0 = lg_pk2(b0, b0);
                        const float4 *col = reinterpret_cast<const float4 *>(Wp + j * LDW);
#pragma unroll
                        for (int q = 0; q < K / 4; q++) {
                            const float4 x = col[q];
                            t0[2 * q] = lg_ffma2(lg_pk2(x.x, x.y), p0, t0[2 * q]);
                            t0[2 * q + 1] = lg_ffma2(lg_pk2(x.z, x.w), p0, t0[2 * q + 1]);
                        }
                    }
                    float4 *o0 = reinterpret_cast<float4 *>(mX + ci * K * K + (int64_t)r * K);
#pragma unroll
                    for (int q = 0; q < K / 4; q++) {
                        float a, b, cc, d;
                        lg_upk2(t0[2 * q], a, b);
                        lg_upk2(t0[2 * q + 1], cc, d);
                        o0[q] = make_float4(a, b, cc, d);
                    }
                }
                __syncwarp();
            }
            LG_EPHASE(2);
        }
        // this run's cost for the next call's order
        if (runcost && lane == 0) runcost[base / R + run] = run_sweeps;
    }
#ifdef LG_PHASE_CLOCKS
    if (blockIdx.x == 0 && threadIdx.x == 0)
        printf("eig cycles warp 0 of cta 0: W build %lld, jacobi %lld, outputs %lld\n", ec[0], ec[1], ec[2]);
#endif
#undef LG_EPHASE
}

// FP64 refinement of the eigenpairs of A' = A + cdiag I (LETKF_PREC_MIXED_F64EIG)
// for the cubes cube0 .. cube_end - 1, one cube per CTA at a time: one step
// of the iterative refinement of Ogita and Aishima (Japan J. Indust. Appl.
// Math. 35 (2018) 1007-1035, Algorithm 1) on the FP32 Jacobi eigenvectors
// X^ (columns of mX):
//     R = I - X^T X^,  S = X^T A' X^                          (FP64)
//     lambda_i = S_ii / (1 - R_ii)
//     E_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i)   if |lambda_i - lambda_j| > delta
//          = R_ij / 2                                          otherwise, and for i = j
//     delta = 2 (||S - diag(lambda)||_F + max|lambda| ||R||_F)
//     X = X^ + X^ E
// The step squares the eigenvectors' error (about 1e-6 from the FP32 Jacobi,
// so about 1e-12 after it).  E is of that size, so the product X^ E is taken
// in FP32 (its rounding is ~1e-13 of X) and added in FP64.  Then, in FP64,
// f_j = sqrt((k-1)/lambda_j), T = X diag(f) X^T (letkf_core.F90:98-160) and
// wbar = X diag(1/lambda) X^T g (:162-195).  T goes as FP32 row-major into
// the cube's slot of mX (it only feeds the BF16 hi/lo update) and wbar into
// the cube's slot of g in mgv.  Every product of the step runs on the FP64
// pipe: about 0.69 M DFMA per cube at k = 64.
constexpr int kTR = 256;
// Largest first-order correction the step applies to a pair of eigenvectors
// (above it the pair is treated as a cluster): the step's second-order
// remainder, ~kRefineMaxRot^2 of non-orthogonality, stays near 1e-8.  On
// k = 64 test matrices (a CPU replica of the FP32 warp Jacobi and of this
// step) T comes out within 6e-7 of an FP64 eigendecomposition of the same A'
// (FP32 eigenpairs alone: 5e-6); the rest is the pairs kept as clusters, whose
// FP32 rotation changes T by their angle times the difference of their f.
constexpr double kRefineMaxRot = 1e-4;

template <int K>
__global__ void __launch_bounds__(kTR, 2)
k_eig_refine(int64_t cube0, int64_t cube_end, double cdiag, const float *mA, float *mX, double *mgv)
{
    static_assert(K == 64, "one 4x4 tile of the k x k products per thread");
    constexpr int KB = K / 4, NLOW = KB * (KB + 1) / 2;
    extern __shared__ double smr[];
    double *Xd = smr;                 // X^ by rows: Xd[r*K + j] = x^_j[r]
    double *Bd = Xd + K * K;          // B = A' X^ by rows; then E (FP32, [i*K + j])
    double *RS = Bd + K * K;          // R below the diagonal ([i*K + j], i > j), S above ([j*K + i]); then X^T
    double *rdg = RS + K * K;         // R_ii
    double *sdg = rdg + K;            // S_ii
    double *lam = sdg + K;            // refined eigenvalues
    double *fv = lam + K;             // sqrt((k-1)/lambda)
    double *ilv = fv + K;             // 1/lambda
    double *gvv = ilv + K;            // g
    double *cv = gvv + K;             // X^T g / lambda
    double *red = cv + K;             // 3 x 8 warp partial sums
    float *Ef = reinterpret_cast<float *>(Bd);
    double *Xt = RS;                  // refined X by eigenvector: Xt[j*K + r]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // this thread's full tile and (threads < NLOW) lower tile
    const int fi = tid / KB, fj = tid % KB;
    int li = 0, lj = 0;
    const bool has_low = tid < NLOW;
    lg_decode_block(has_low ? tid : 0, li, lj);

    for (int64_t c = cube0 + blockIdx.x; c < cube_end; c += gridDim.x) {
        const int64_t ci = c - cube0;
        const float *Ac = mA + ci * K * K;
        float *Xc = mX + ci * K * K;
        for (int idx = tid; idx < K * K; idx += kTR) {
            const int j = idx / K, r = idx % K;
            Xd[r * K + j] = (double)Xc[idx];
        }
        if (tid < K) gvv[tid] = mgv[ci * K + tid];
        __syncthreads();

        // R (lower tiles) and B = A X^ + cdiag X^ (all tiles)
        if (has_low) {
            double acc[16];
#pragma unroll
            for (int q = 0; q < 16; q++) acc[q] = 0.0;
            for (int r = 0; r < K; r++) {
                const double *row = Xd + r * K;
                double a[4], b[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    a[q] = row[4 * li + q];
                    b[q] = row[4 * lj + q];
                }
#pragma unroll
                for (int p = 0; p < 4; p++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[p * 4 + q] = fma(a[p], b[q], acc[p * 4 + q]);
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int i = 4 * li + p, j = 4 * lj + q;
                    if (i > j) RS[i * K + j] = -acc[p * 4 + q];
                    else if (i == j) rdg[i] = 1.0 - acc[p * 4 + q];
                }
        }
        {
            double acc[16];
#pragma unroll
            for (int q = 0; q < 16; q++) acc[q] = 0.0;
            for (int l = 0; l < K; l++) {
                // A symmetric: rows 4 fi .. of column l = row l at 4 fi ..
                const float4 av = *reinterpret_cast<const float4 *>(Ac + l * K + 4 * fi);
                const double a[4] = {(double)av.x, (double)av.y, (double)av.z, (double)av.w};
                const double *xr = Xd + l * K + 4 * fj;
                const double b[4] = {xr[0], xr[1], xr[2], xr[3]};
#pragma unroll
                for (int p = 0; p < 4; p++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[p * 4 + q] = fma(a[p], b[q], acc[p * 4 + q]);
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int r = 4 * fi + p, j = 4 * fj + q;
                    Bd[r * K + j] = fma(cdiag, Xd[r * K + j], acc[p * 4 + q]);
                }
        }
        __syncthreads();

        // S = X^T B (lower tiles)
        if (has_low) {
            double acc[16];
#pragma unroll
            for (int q = 0; q < 16; q++) acc[q] = 0.0;
            for (int r = 0; r < K; r++) {
                double a[4], b[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    a[q] = Xd[r * K + 4 * li + q];
                    b[q] = Bd[r * K + 4 * lj + q];
                }
#pragma unroll
                for (int p = 0; p < 4; p++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[p * 4 + q] = fma(a[p], b[q], acc[p * 4 + q]);
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int i = 4 * li + p, j = 4 * lj + q;
                    if (i > j) RS[j * K + i] = acc[p * 4 + q];
                    else if (i == j) sdg[i] = acc[p * 4 + q];
                }
        }
        __syncthreads();

        // lambda_i and the cluster threshold delta
        if (tid < K) lam[tid] = sdg[tid] / (1.0 - rdg[tid]);
        __syncthreads();
        {
            double so = 0.0, ro = 0.0, lm = 0.0;
            for (int idx = tid; idx < K * K; idx += kTR) {
                const int i = idx / K, j = idx % K;
                if (i > j) {
                    const double s = RS[j * K + i], r = RS[i * K + j];
                    so += 2.0 * s * s;
                    ro += 2.0 * r * r;
                } else if (i == j) {
                    const double s = sdg[i] - lam[i], r = rdg[i];
                    so += s * s;
                    ro += r * r;
                    lm = fmax(lm, fabs(lam[i]));
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                so += __shfl_xor_sync(0xffffffffu, so, o);
                ro += __shfl_xor_sync(0xffffffffu, ro, o);
                lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
            }
            if (lane == 0) {
                red[warp] = so;
                red[8 + warp] = ro;
                red[16 + warp] = lm;
            }
        }
        __syncthreads();
        double so = 0.0, ro = 0.0, lm = 0.0;
#pragma unroll
        for (int w8 = 0; w8 < kTR / 32; w8++) {
            so += red[w8];
            ro += red[8 + w8];
            lm = fmax(lm, red[16 + w8]);
        }
        const double delta = 2.0 * (sqrt(so) + lm * sqrt(ro));
        // E (FP32) over B, which is dead after S
        for (int idx = tid; idx < K * K; idx += kTR) {
            const int i = idx / K, j = idx % K;
            double e;
            if (i == j) {
                e = 0.5 * rdg[i];
            } else {
                const int hi = i > j ? i : j, lo = i > j ? j : i;
                const double s = RS[lo * K + hi], r = RS[hi * K + lo];
                const double gap = lam[j] - lam[i];
                e = 0.5 * r;
                if (fabs(gap) > delta) {
                    // the pair is rotated only when both first-order terms are
                    // small: the step leaves O(e^2) of non-orthogonality in X,
                    // and a pair whose FP32 vectors are far off (eigenvalues
                    // close at FP32 resolution) is kept as a cluster instead,
                    // where its rotation changes T by less than its gap does
                    const double eij = (s + lam[j] * r) / gap, eji = -(s + lam[i] * r) / gap;
                    if (fmax(fabs(eij), fabs(eji)) <= kRefineMaxRot) e = eij;
                }
            }
            Ef[idx] = (float)e;
        }
        __syncthreads();

        // X = X^ + X^ E: the correction in FP32 from X^ (mX) and E, added in
        // FP64; written by eigenvector (Xt over R and S, dead now)
        {
            float acc[16];
#pragma unroll
            for (int q = 0; q < 16; q++) acc[q] = 0.0f;
            for (int i = 0; i < K; i++) {
                // X^ rows 4 fi .. of column i, E row i at 4 fj ..
                const float4 xv = *reinterpret_cast<const float4 *>(Xc + i * K + 4 * fi);
                const float4 ev = *reinterpret_cast<const float4 *>(Ef + i * K + 4 * fj);
                const float a[4] = {xv.x, xv.y, xv.z, xv.w}, b[4] = {ev.x, ev.y, ev.z, ev.w};
#pragma unroll
                for (int p = 0; p < 4; p++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[p * 4 + q] = fmaf(a[p], b[q], acc[p * 4 + q]);
            }
            __syncthreads();               // every thread is done with R and S
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int r = 4 * fi + p, j = 4 * fj + q;
                    Xt[j * K + r] = Xd[r * K + j] + (double)acc[p * 4 + q];
                }
        }
        if (tid < K) {
            fv[tid] = sqrt((double)(K - 1) / lam[tid]);
            ilv[tid] = 1.0 / lam[tid];
        }
        __syncthreads();

        // T = X diag(f) X^T (lower tiles), FP32 row-major into the slot of X^
        if (has_low) {
            double acc[16];
#pragma unroll
            for (int q = 0; q < 16; q++) acc[q] = 0.0;
            for (int j = 0; j < K; j++) {
                const double f = fv[j];
                const double *xj = Xt + j * K;
                double a[4], b[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    a[q] = xj[4 * li + q];
                    b[q] = xj[4 * lj + q] * f;
                }
#pragma unroll
                for (int p = 0; p < 4; p++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[p * 4 + q] = fma(a[p], b[q], acc[p * 4 + q]);
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int r = 4 * li + p, s = 4 * lj + q;
                    const float t = (float)acc[p * 4 + q];
                    Xc[r * K + s] = t;
                    Xc[s * K + r] = t;
                }
        }
        // wbar = X diag(1/lambda) X^T g
        if (tid < K) {
            double d = 0.0;
            for (int r = 0; r < K; r++) d = fma(Xt[tid * K + r], gvv[r], d);
            cv[tid] = d * ilv[tid];
        }
        __syncthreads();
        if (tid < K) {
            double d = 0.0;
            for (int j = 0; j < K; j++) d = fma(Xt[j * K + tid], cv[j], d);
            mgv[ci * K + tid] = d;
        }
        __syncthreads();
    }
}

// Most cubes one staged launch sequence holds intermediates for (A, X: 2 k^2
// floats, g: k doubles, lambda: k floats per cube); a multiple of every
// work-queue chunk size and of the eigensolve run.
constexpr int64_t kStagedCubes = 1 << 17;

template <int K, int ST>
cudaError_t launch_stage(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb, double *xa,
                         double *axa, double *trans_out, double *w_out, int chunk, int nchunks, int nsm)
{
    // the update without the members takes the compact layout
    const bool u3 = ST == 3 && !ctx->members_on;
    const size_t smem = ST == 1 ? MCfg<K>::SMEM1 : u3 ? MCfg<K>::SMEM3 : MCfg<K>::SMEM;
    auto kern = (ST != 1 && ctx->members_on) ? k_core_mixed<K, ST, ST != 1> : k_core_mixed<K, ST, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    int dev = 0, smem_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    // CTAs per SM: as many as the launch bounds give registers for (2; 3 for
    // the A build and the plain update) when their shared memory (plus the 1 KB the system keeps per
    // CTA and the static barriers) fits
    int per_sm = (ST == 1 || u3) ? 3 : 2;
    while (per_sm > 1 && (size_t)per_sm * (smem + 1024 + 64) > (size_t)smem_sm) per_sm--;
    // persistent grid: each CTA allocates its tensor memory once
    const int64_t want = (int64_t)nsm * per_sm;
    const unsigned blocks = (unsigned)(nchunks < want ? nchunks : want);
    // the CTAs take chunks with the queue cursor
    e = cudaMemsetAsync(ctx->d_counters.p + LG_CNT_QUEUE, 0, sizeof(unsigned long long), ctx->stream);
    if (e != cudaSuccess) return e;
    lg_count_launch();
    kern<<<blocks, kT, smem, ctx->stream>>>(
        g, lg_params(ctx), ctx->d_ys32.p, ctx->d_lidx.p, ctx->d_lmeta.p, ctx->d_queue.p, nchunks, chunk,
        ctx->d_loff.p, ctx->d_lcnt.p, ctx->win1, xb, axb, xa, axa, trans_out, w_out, ctx->d_counters.p,
        ctx->d_status.p, ctx->d_mA.p, ctx->d_mg.p, ctx->d_mX.p, ctx->d_ymax.p);
    return cudaGetLastError();
}

template <int K>
cudaError_t launch_mixed(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb,
                         double *xa, double *axa, double *trans_out, double *w_out)
{
    if (ctx->win1 <= ctx->win0) return cudaSuccess;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int chunk = 0, nchunks = 0;
    if constexpr (K != 64) {
        // one launch: A build, eigensolve and update per cube
        cudaError_t e = lg_build_chunk_queue(ctx, chunk, nchunks);
        if (e != cudaSuccess) return e;
        return launch_stage<K, 0>(ctx, g, xb, axb, xa, axa, trans_out, w_out, chunk, nchunks, nsm);
    } else {
        // staged: the A build (work queue), the eigenproblems one warp each,
        // the update (work queue), over blocks of at most kStagedCubes cubes
        const int64_t w0 = ctx->win0, w1 = ctx->win1;
        // eigensolve runs of 8 cubes: short enough to spread evenly over the
        // warps, aligned so that every window boundary (a multiple of the
        // work-queue chunk, itself a multiple of 8) is a run boundary
        const int R = 8;
        // each warp: its K x (K+4) columns, then 3K doubles of vectors
        const size_t ew = ((size_t)K * (K + 4) * sizeof(float) + 3 * K * sizeof(double)) * (kTE / 32);
        cudaError_t e = cudaFuncSetAttribute(k_eig_warp<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ew);
        // blocks end at multiples of `step` in cube numbering (so the runs and
        // chunks, and the results, do not depend on the blocking), at most
        // kStagedCubes each; when the analysis goes back to host memory, three
        // blocks of 1/2, 3/10 and 1/5 of the cubes, each copied out while the
        // next ones run (copying a block takes about 0.64 of its analysis
        // time; smaller blocks leave the eigensolve's warps short of runs)
        const int64_t step = max((int64_t)4096, (int64_t)lg_run_chunk(ctx));
        auto align_up = [&](int64_t c) { return min(w1, (c + step - 1) / step * step); };
        int64_t cut[2] = {w1, w1};
        if (ctx->sink_xa) {
            cut[0] = align_up(w0 + (w1 - w0) / 2);
            cut[1] = align_up(w0 + (w1 - w0) * 4 / 5);
        }
        int64_t b1 = w0;
        for (int64_t b0 = w0; b0 < w1 && e == cudaSuccess; b0 = b1) {
            b1 = min(w1, (b0 / kStagedCubes + 1) * kStagedCubes);
            for (int i = 0; i < 2; i++)
                if (cut[i] > b0 && cut[i] < b1) b1 = cut[i];
            const int64_t nb = b1 - b0;
            ctx->win0 = b0;
            ctx->win1 = b1;
            if ((e = ctx->d_mA.reserve((size_t)nb * K * K)) != cudaSuccess) break;
            if ((e = ctx->d_mX.reserve((size_t)nb * K * K)) != cudaSuccess) break;
            if ((e = ctx->d_mg.reserve((size_t)nb * K)) != cudaSuccess) break;
            if ((e = ctx->d_mlam.reserve((size_t)nb * K)) != cudaSuccess) break;
            if ((e = lg_build_chunk_queue(ctx, chunk, nchunks)) != cudaSuccess) break;
            lg_stage_mark(ctx, 0, false);
            e = launch_stage<K, 1>(ctx, g, xb, axb, xa, axa, trans_out, w_out, chunk, nchunks, nsm);
            lg_stage_mark(ctx, 0, true);
            if (e != cudaSuccess) break;
            const int64_t runs = (b1 - b0 / R * R + R - 1) / R;
            const int64_t eb = (runs + kTE / 32 - 1) / (kTE / 32);
            const unsigned eblocks = (unsigned)(eb < nsm ? eb : nsm);
            if ((e = cudaMemsetAsync(ctx->d_counters.p + LG_CNT_QUEUE, 0, sizeof(unsigned long long),
                                     ctx->stream)) != cudaSuccess)
                break;
            // the block's runs longest first by their sweeps in the last call
            // (all equal before the first: cube order), so that the warps end
            // together instead of waiting on a few long runs
            const int64_t nrun_all = (ctx->ncubes + R - 1) / R;
            if (ctx->d_runcost.n < (size_t)nrun_all) {
                if ((e = ctx->d_runcost.reserve((size_t)nrun_all)) != cudaSuccess) break;
                if ((e = cudaMemsetAsync(ctx->d_runcost.p, 0, sizeof(int) * nrun_all, ctx->stream)) != cudaSuccess)
                    break;
            }
            int *rorder = nullptr;
            if (runs <= kQueueMax) {
                if ((e = ctx->d_rorder.reserve((size_t)runs)) != cudaSuccess) break;
                int np2 = 1;
                while (np2 < runs) np2 <<= 1;
                const size_t rsm = sizeof(unsigned long long) * np2;
                if ((e = cudaFuncSetAttribute(k_run_order, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm)) !=
                    cudaSuccess)
                    break;
                lg_count_launch();
                k_run_order<<<1, 1024, rsm, ctx->stream>>>(ctx->d_runcost.p, b0 / R, (int)runs, ctx->d_rorder.p);
                if ((e = cudaGetLastError()) != cudaSuccess) break;
                rorder = ctx->d_rorder.p;
            }
            lg_count_launch();
            lg_stage_mark(ctx, 1, false);
            // LETKF_PREC_MIXED: the warps also form wbar and T (for the update
            // launch); LETKF_PREC_MIXED_F64EIG: they write X and lambda for the
            // FP64 refinement
            const bool f64eig = ctx->params.precision == LETKF_PREC_MIXED_F64EIG;
            k_eig_warp<K><<<eblocks, kTE, ew, ctx->stream>>>(b0, b1, R, (double)(K - 1) / ctx->params.inflation,
                                                          LG_MIXED_JACOBI_TOL, ctx->d_mA.p, ctx->d_mX.p,
                                                          ctx->d_mlam.p, ctx->d_mg.p, f64eig ? 0 : 1,
                                                          ctx->d_counters.p, rorder, ctx->d_runcost.p);
            lg_stage_mark(ctx, 1, true);
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            if (f64eig) {
                // FP64 eigenpairs, T and wbar, then the update from them
                constexpr size_t rs = sizeof(double) * (3 * K * K + 7 * K + 32);
                if ((e = cudaFuncSetAttribute(k_eig_refine<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)rs)) != cudaSuccess)
                    break;
                const int64_t rb = std::min<int64_t>(b1 - b0, (int64_t)nsm * 2);
                lg_count_launch();
                lg_stage_mark(ctx, 3, false);
                k_eig_refine<K><<<(unsigned)rb, kTR, rs, ctx->stream>>>(b0, b1, (double)(K - 1) / ctx->params.inflation,
                                                                         ctx->d_mA.p, ctx->d_mX.p, ctx->d_mg.p);
                lg_stage_mark(ctx, 3, true);
                if ((e = cudaGetLastError()) != cudaSuccess) break;
            }
            // the update from T and wbar, once the block's columns of the state
            // are in (a run from host buffers copies them in meanwhile)
            if (ctx->params.cube_n == 1) e = lg_state_wait(ctx, b0, b1);
            else e = lg_state_wait(ctx, 0, ctx->ncol);
            if (e != cudaSuccess) break;
            lg_stage_mark(ctx, 2, false);
            e = launch_stage<K, 3>(ctx, g, xb, axb, xa, axa, trans_out, w_out, chunk, nchunks, nsm);
            lg_stage_mark(ctx, 2, true);
            if (e == cudaSuccess) e = lg_sink_columns(ctx, b0, b1);
        }
        ctx->win0 = w0;
        ctx->win1 = w1;
        return e;
    }
}

}  // namespace

bool lg_mixed_supports(int k) { return k == 32 || k == 48 || k == 64 || k == 96 || k == 128; }

cudaError_t lg_launch_core_mixed(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb,
                                 double *xa, double *axa, bool keep_trans)
{
    double *tr = keep_trans ? ctx->d_trans.p : nullptr;
    double *w = keep_trans ? ctx->d_w.p : nullptr;
    switch (g.k) {
    case 32: return launch_mixed<32>(ctx, g, xb, axb, xa, axa, tr, w);
    case 48: return launch_mixed<48>(ctx, g, xb, axb, xa, axa, tr, w);
    case 64: return launch_mixed<64>(ctx, g, xb, axb, xa, axa, tr, w);
    case 96:
    case 128: return lg_launch_core_mixed_wide(ctx, g, xb, axb, xa, axa, tr, w);
    default: return cudaErrorInvalidValue;
    }
}
