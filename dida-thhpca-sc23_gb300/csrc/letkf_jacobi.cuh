// letkf_jacobi.cuh -- one-sided (Hestenes) Jacobi eigensolve of a symmetric
// positive definite k x k matrix held by columns in shared memory, and the
// lower-triangle 4x4 block numbering of the register-tiled products.
#pragma once

template <typename T> struct LgVec2;
template <> struct LgVec2<double> { using type = double2; };
template <> struct LgVec2<float> { using type = float2; };

// Rotation (c, s, t) that zeroes the inner product gam of two columns with
// squared norms al, be (t = tan of the angle, c = cos, s = sin).
__device__ __forceinline__ void lg_rotation(double al, double be, double gam, double &c, double &s,
                                            double &t)
{
    const double zeta = (be - al) / (2.0 * gam);
    t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
    c = 1.0 / sqrt(1.0 + t * t);
    s = c * t;
}

// FP32 variant for the approximate eigenpairs of the mixed form, written for
// a short dependency chain: with d = be - al, r = sqrt(d^2 + (2 gam)^2),
//     t = sign(d) 2 gam / (|d| + r),   c = 1 / sqrt(1 + t^2),   s = c t
// (the same t as above, multiplied through by |2 gam|), using the hardware
// approximate reciprocal and reciprocal square root (relative error ~1e-7).
// The caller only rotates when gam^2 > tol^2 al be > 0, so r > 0.
__device__ __forceinline__ float lg_rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg_rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void lg_rotation(float al, float be, float gam, float &c, float &s, float &t)
{
    const float d = be - al, g2 = 2.0f * gam;
    const float r2 = fmaf(d, d, g2 * g2);
    const float r = r2 * lg_rsqrt_approx(r2);
    t = (d >= 0.0f ? g2 : -g2) * lg_rcp_approx(fabsf(d) + r);
    c = lg_rsqrt_approx(fmaf(t, t, 1.0f));
    s = c * t;
}

// Packed pairs of FP32 (the f32x2 arithmetic of sm_100 and later): two
// independent IEEE single-precision operations per instruction.
__device__ __forceinline__ unsigned long long lg_pk2(float a, float b)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void lg_upk2(unsigned long long r, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ unsigned long long lg_ffma2(unsigned long long a, unsigned long long b,
                                                       unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long lg_fmul2(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ void lg_decode_block(int b, int &bi, int &bj)
{
    int i = (int)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= b) i++;
    while (i * (i + 1) / 2 > b) i--;
    bi = i;
    bj = b - i * (i + 1) / 2;
}

// One-sided Jacobi on the columns of W (column j at W[j*LD ..]).  Each step of
// a sweep rotates K/2 disjoint column pairs (round-robin ordering); a group of
// G threads forms each pair's inner product with shuffles and rotates the two
// columns.  With ONE_THREAD_SCALARS (for FP64, where every warp instruction
// costs FP64 pipe time) one thread per pair turns (alpha, beta, gamma) into the
// rotation between two barriers, so the divisions and square roots are done
// once per pair; otherwise (FP32) every lane of the group computes them and a
// step needs one barrier.  For an SPD matrix the converged columns are
// lambda_j v_j.  Returns the sweeps used, or max_sweeps+1 if not converged.
template <typename T, int K, int G, int LD = K, bool ONE_THREAD_SCALARS = true>
__device__ int lg_jacobi(T *W, T *nrm, typename LgVec2<T>::type *rot, int *s_rot, T tol,
                         int max_sweeps)
{
    constexpr int NP = K / 2;
    const int tid = threadIdx.x;
    const int pair = tid / G, lane = tid % G;
    const bool act = pair < NP;
    const T tol2 = tol * tol;
    int sweep;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        if (tid < K) {
            T s = 0;
            for (int r = 0; r < K; r++) s += W[tid * LD + r] * W[tid * LD + r];
            nrm[tid] = s;
        }
        if (tid == 0) *s_rot = 0;
        __syncthreads();
        // round-robin pairs: pair 0 is (K-1, r); pair m > 0 is
        // ((r + m) mod (K-1), (r - m) mod (K-1)), advanced incrementally
        int pr = pair % (K - 1), qr = (K - 1 - pair) % (K - 1);
        for (int r = 0; r < K - 1; r++) {
            int p = 0, q = 0;
            T gam = 0;
            if (act) {
                if (pair == 0) {
                    p = K - 1;
                    q = r;
                } else {
                    p = pr;
                    q = qr;
                }
                if (++pr == K - 1) pr = 0;
                if (++qr == K - 1) qr = 0;
                const T *wp = W + p * LD, *wq = W + q * LD;
#pragma unroll
                for (int rr = lane; rr < K; rr += G) gam += wp[rr] * wq[rr];
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) gam += __shfl_xor_sync(0xffffffffu, gam, o);
            }
            if (ONE_THREAD_SCALARS) {
                if (act && lane == 0) rot[pair].x = gam;
                __syncthreads();
                if (tid < NP) {
                    int pp, qq;
                    if (tid == 0) {
                        pp = K - 1;
                        qq = r;
                    } else {
                        pp = (r + tid) % (K - 1);
                        qq = (r - tid + (K - 1)) % (K - 1);
                    }
                    const T g2 = rot[tid].x;
                    const T al = nrm[pp], be = nrm[qq];
                    T c = 1, s = 0;
                    if (g2 * g2 > tol2 * (al * be)) {
                        T t;
                        lg_rotation(al, be, g2, c, s, t);
                        nrm[pp] = al - t * g2;
                        nrm[qq] = be + t * g2;
                        *s_rot = 1;
                    }
                    rot[tid].x = c;
                    rot[tid].y = s;
                }
                __syncthreads();
                if (act) {
                    const T c = rot[pair].x, s = rot[pair].y;
                    if (s != T(0)) {
                        T *wp = W + p * LD, *wq = W + q * LD;
#pragma unroll
                        for (int rr = lane; rr < K; rr += G) {
                            const T a = wp[rr], b = wq[rr];
                            wp[rr] = c * a - s * b;
                            wq[rr] = s * a + c * b;
                        }
                    }
                }
            } else if (act) {
                const T al = nrm[p], be = nrm[q];
                __syncwarp();
                if (gam * gam > tol2 * (al * be)) {
                    T c, s, t;
                    lg_rotation(al, be, gam, c, s, t);
                    T *wp = W + p * LD, *wq = W + q * LD;
#pragma unroll
                    for (int rr = lane; rr < K; rr += G) {
                        const T a = wp[rr], b = wq[rr];
                        wp[rr] = c * a - s * b;
                        wq[rr] = s * a + c * b;
                    }
                    if (lane == 0) {
                        nrm[p] = al - t * gam;
                        nrm[q] = be + t * gam;
                        *s_rot = 1;
                    }
                }
            }
            __syncthreads();
        }
        const int rotated = *s_rot;
        __syncthreads();
        if (!rotated) break;
    }
    return sweep;
}

// FP32 one-sided Jacobi for the mixed-precision form.  Same round-robin
// scheme as lg_jacobi, but each lane of a pair group owns a contiguous run of
// K/G rows, keeps the pair's rows in registers between the inner product and
// the rotation, and moves them with vector shared-memory accesses; every lane
// computes the rotation (FP32, cheap) so a step needs one barrier.  LD (the
// column stride) must keep the rows of a lane aligned for the vector width.
// Pairs whose cosine exceeds tol are rotated; the sweeps stop after one in
// which no cosine exceeded tol_continue (>= tol; tol itself is the usual
// choice, a larger value skips the last, confirming sweep).
template <int K, int G, int LD>
__device__ int lg_jacobi32(float *W, float *nrm, int *s_rot, float tol, float tol_continue, int max_sweeps)
{
    constexpr int NP = K / 2, RPL = K / G;
    constexpr int VW = (RPL % 4 == 0) ? 4 : ((RPL % 2 == 0) ? 2 : 1);
    constexpr int NC = RPL / VW;                 // vector chunks per lane
    static_assert(K % G == 0, "rows per lane");
    static_assert(LD % VW == 0, "vector alignment of columns");
    const int tid = threadIdx.x;
    const int pair = tid / G, lane = tid % G;
    const int warp = tid >> 5, wl = tid & 31;
    const bool act = pair < NP;
    const float tol2 = tol * tol, cont2 = tol_continue * tol_continue;
    int sweep;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        // squared column norms, one warp per column
        for (int j = warp; j < K; j += (int)(blockDim.x >> 5)) {
            float s = 0.0f;
            for (int r = wl; r < K; r += 32) s = fmaf(W[j * LD + r], W[j * LD + r], s);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (wl == 0) nrm[j] = s;
        }
        if (tid == 0) *s_rot = 0;
        __syncthreads();
        int pr = pair % (K - 1), qr = (K - 1 - pair) % (K - 1);
        for (int r = 0; r < K - 1; r++) {
            if (act) {
                const int p = (pair == 0) ? K - 1 : pr;
                const int q = (pair == 0) ? r : qr;
                if (++pr == K - 1) pr = 0;
                if (++qr == K - 1) qr = 0;
                // lane rows: chunks c*G + lane of VW rows, so the G lanes of a
                // pair read consecutive vectors (no bank conflicts for VW = 4)
                float *wp = W + p * LD + lane * VW, *wq = W + q * LD + lane * VW;
                float a[RPL], b[RPL];
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    const int o = c * G * VW, i = c * VW;
                    if (VW == 4) {
                        const float4 x = *reinterpret_cast<const float4 *>(wp + o);
                        const float4 y = *reinterpret_cast<const float4 *>(wq + o);
                        a[i] = x.x; a[i + 1] = x.y; a[i + 2] = x.z; a[i + 3] = x.w;
                        b[i] = y.x; b[i + 1] = y.y; b[i + 2] = y.z; b[i + 3] = y.w;
                    } else if (VW == 2) {
                        const float2 x = *reinterpret_cast<const float2 *>(wp + o);
                        const float2 y = *reinterpret_cast<const float2 *>(wq + o);
                        a[i] = x.x; a[i + 1] = x.y;
                        b[i] = y.x; b[i + 1] = y.y;
                    } else {
                        a[i] = wp[o];
                        b[i] = wq[o];
                    }
                }
                float g0 = 0.0f, g1 = 0.0f;
#pragma unroll
                for (int i = 0; i < RPL; i += 2) {
                    g0 = fmaf(a[i], b[i], g0);
                    if (i + 1 < RPL) g1 = fmaf(a[i + 1], b[i + 1], g1);
                }
                float gam = g0 + g1;
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) gam += __shfl_xor_sync(0xffffffffu, gam, o);
                const float al = nrm[p], be = nrm[q];
                __syncwarp();
                if (gam * gam > tol2 * (al * be)) {
                    float c, s, t;
                    lg_rotation(al, be, gam, c, s, t);
#pragma unroll
                    for (int i = 0; i < RPL; i++) {
                        const float x = a[i], y = b[i];
                        a[i] = c * x - s * y;
                        b[i] = s * x + c * y;
                    }
#pragma unroll
                    for (int cc = 0; cc < NC; cc++) {
                        const int o = cc * G * VW, i = cc * VW;
                        if (VW == 4) {
                            *reinterpret_cast<float4 *>(wp + o) = make_float4(a[i], a[i + 1], a[i + 2], a[i + 3]);
                            *reinterpret_cast<float4 *>(wq + o) = make_float4(b[i], b[i + 1], b[i + 2], b[i + 3]);
                        } else if (VW == 2) {
                            *reinterpret_cast<float2 *>(wp + o) = make_float2(a[i], a[i + 1]);
                            *reinterpret_cast<float2 *>(wq + o) = make_float2(b[i], b[i + 1]);
                        } else {
                            wp[o] = a[i];
                            wq[o] = b[i];
                        }
                    }
                    if (lane == 0) {
                        nrm[p] = al - t * gam;
                        nrm[q] = be + t * gam;
                        if (gam * gam > cont2 * (al * be)) *s_rot = 1;
                    }
                }
            }
            __syncthreads();
        }
        const int rotated = *s_rot;
        __syncthreads();
        if (!rotated) break;
    }
    return sweep;
}

// FP32 one-sided Jacobi with a hierarchical parallel ordering (K a power of
// two): the K columns are split into halves; for K/2 steps the K/2 slots each
// hold one column of the first half fixed in registers and rotate it against
// the second half's columns, which move one slot per step, so every step
// moves one column per slot through shared memory instead of two.  Then each
// half is split again (two sub-problems of K/2 columns side by side), and so on
// down to pairs: K/2 + K/4 + ... + 1 = K-1 steps cover every pair once per
// sweep, as the round-robin ordering does.  Columns are stored back into W
// (column j at W[j*LD ..]) after every level.  The moving columns pass through
// buffers that reuse W's memory while the columns live in registers (slot
// stride BS: with G = 4 lanes two slots share a quarter-warp of 16-byte
// accesses, so BS = K + 16 puts them on disjoint bank halves); their norms and
// ids go to `extra` (4 * (K/2) words; by default right after the buffers).
// The inner products and rotations use packed f32x2 arithmetic.
// Returns the sweeps used, or max_sweeps+1 if not converged.
template <int K, int G, int LD, int BS = K>
__device__ int lg_jacobi32h(float *W, int *s_rot, float tol, int max_sweeps, float *extra = nullptr)
{
    constexpr int NS = K / 2, RPL = K / G;
    constexpr int VW = (RPL % 4 == 0) ? 4 : ((RPL % 2 == 0) ? 2 : 1);
    constexpr int NC = RPL / VW;
    static_assert((K & (K - 1)) == 0, "K must be a power of two");
    static_assert(K % G == 0 && LD % VW == 0 && BS % VW == 0 && RPL % 2 == 0, "rows per lane");
    static_assert(2 * NS * BS <= K * LD, "moving-column buffers must fit in W");
    const int tid = threadIdx.x;
    const int slot = tid / G, lane = tid % G;
    const bool act = slot < NS;
    const float tol2 = tol * tol;
    float *buf = W;                                   // [2][NS] moving columns, stride BS
    float *bnrm = extra ? extra : W + 2 * NS * BS;     // [2][NS] their squared norms
    int *bid = reinterpret_cast<int *>(bnrm + 2 * NS);  // [2][NS] their column ids
    float F[RPL], M[RPL];

    auto ld = [&](const float *src, float *r) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int o = (c * G + lane) * VW, i = c * VW;
            if (VW == 4) {
                const float4 x = *reinterpret_cast<const float4 *>(src + o);
                r[i] = x.x; r[i + 1] = x.y; r[i + 2] = x.z; r[i + 3] = x.w;
            } else if (VW == 2) {
                const float2 x = *reinterpret_cast<const float2 *>(src + o);
                r[i] = x.x; r[i + 1] = x.y;
            } else {
                r[i] = src[o];
            }
        }
    };
    auto st = [&](float *dst, const float *r) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int o = (c * G + lane) * VW, i = c * VW;
            if (VW == 4) *reinterpret_cast<float4 *>(dst + o) = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
            else if (VW == 2) *reinterpret_cast<float2 *>(dst + o) = make_float2(r[i], r[i + 1]);
            else dst[o] = r[i];
        }
    };
    auto dot = [&](const float *x, const float *y) {
        unsigned long long a0 = 0ull, a1 = 0ull;
#pragma unroll
        for (int i = 0; i < RPL; i += 4) {
            a0 = lg_ffma2(lg_pk2(x[i], x[i + 1]), lg_pk2(y[i], y[i + 1]), a0);
            if (i + 3 < RPL) a1 = lg_ffma2(lg_pk2(x[i + 2], x[i + 3]), lg_pk2(y[i + 2], y[i + 3]), a1);
        }
        float p0, p1, p2, p3;
        lg_upk2(a0, p0, p1);
        lg_upk2(a1, p2, p3);
        float d = (p0 + p1) + (p2 + p3);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        return d;
    };

    int sweep;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        if (tid == 0) *s_rot = 0;
        for (int B = K; B >= 2; B >>= 1) {
            const int half = B / 2, u = slot / half, i = slot % half;
            const int fc = u * B + i;
            int mc = u * B + half + i;
            __syncthreads();                           // W holds every column
            if (act) {
                ld(W + fc * LD, F);
                ld(W + mc * LD, M);
            }
            float fa = 0.0f, mb = 0.0f;
            if (act) {
                fa = dot(F, F);
                mb = dot(M, M);
            }
            __syncthreads();                           // W becomes the moving-column buffers
            for (int t = 0; t < half; t++) {
                if (act) {
                    const float gam = dot(F, M);
                    if (gam * gam > tol2 * (fa * mb)) {
                        float c, s, tt;
                        lg_rotation(fa, mb, gam, c, s, tt);
                        const unsigned long long c2 = lg_pk2(c, c), s2 = lg_pk2(s, s), ns2 = lg_pk2(-s, -s);
#pragma unroll
                        for (int r = 0; r < RPL; r += 2) {
                            const unsigned long long x = lg_pk2(F[r], F[r + 1]), y = lg_pk2(M[r], M[r + 1]);
                            lg_upk2(lg_ffma2(c2, x, lg_fmul2(ns2, y)), F[r], F[r + 1]);
                            lg_upk2(lg_ffma2(s2, x, lg_fmul2(c2, y)), M[r], M[r + 1]);
                        }
                        fa = fa - tt * gam;
                        mb = mb + tt * gam;
                        if (lane == 0) *s_rot = 1;
                    }
                }
                if (t == half - 1) break;
                // pass the moving column to the previous slot of the group
                const int par = t & 1;
                if (act) {
                    st(buf + (par * NS + slot) * BS, M);
                    if (lane == 0) {
                        bnrm[par * NS + slot] = mb;
                        bid[par * NS + slot] = mc;
                    }
                }
                __syncthreads();
                if (act) {
                    const int src = u * half + (i + 1) % half;
                    ld(buf + (par * NS + src) * BS, M);
                    mb = bnrm[par * NS + src];
                    mc = bid[par * NS + src];
                }
            }
            __syncthreads();                           // every read of the buffers is done
            if (act) {
                st(W + fc * LD, F);
                st(W + mc * LD, M);
            }
        }
        __syncthreads();
        const int rotated = *s_rot;
        __syncthreads();
        if (!rotated) break;
    }
    return sweep;
}

// Stop level of the early exit of the FP32 Jacobis (lg_jacobi32b2 and
// lg_jacobi32w): a sweep whose rotations all had |cos| below it ends the solve
// (Jacobi converges quadratically, so the next sweep would find every pair
// below tol).  On the 1 deg, k = 64 workload
// 3e-4 gives the same analysis as sweeping until no pair is above tol, with
// 5.3 instead of 6.1 sweeps per cube; 3e-3 raised the spread error to 2.6e-4.
// 0 turns it off.
#ifndef LG_JACOBI32W_QSTOP
#define LG_JACOBI32W_QSTOP 3e-4f
#endif

// FP32 one-sided Jacobi with the hierarchical ordering over blocks of two
// columns (K = 64 or 128, 256 threads): the K/4 slots each hold a fixed block
// (F1, F2) and a moving block (M1, M2), G = 1024/K lanes per slot and K/G rows
// per lane; a step does the four rotations between the two blocks, (F1, M1)
// with (F2, M2) and then (F1, M2) with (F2, M1), each pair of rotations with
// interleaved inner products, and the last level also rotates the pairs
// inside the two blocks.  K/2 - 1 steps cover every pair once per sweep, so
// the moving columns go through half as many passes as in lg_jacobi32h.  A
// moving block passes to the next slot of its group by warp shuffles; where a
// group spans warps, every 32/G steps the warps hand their moving blocks on
// through shared memory (buffers reuse W while the columns are in registers,
// slot stride 2 BS, alternating by hand-over parity) with one block barrier.
// Norms and block ids of the handed-on blocks go to `extra` (6 * K/4 words).
// Returns the sweeps used, or max_sweeps+1 if not converged.
template <int K, int LD, int BS>
__device__ int lg_jacobi32b2(float *W, float *extra, int *s_rot, float tol, int max_sweeps)
{
    constexpr int NB = K / 2, NSL = NB / 2, G = 256 / NSL, RPL = K / G, SPW = 32 / G;
    constexpr int VW = (RPL % 4 == 0) ? 4 : 2, NC = RPL / VW;
    static_assert(K == 64 || K == 128, "block-2 ordering for K = 64 and 128");
    static_assert(2 * NSL * 2 * BS <= K * LD && LD % VW == 0 && BS % VW == 0, "moving-block buffers fit in W");
    const int tid = threadIdx.x;
    const int slot = tid / G, lane = tid % G;
    const int lw = tid & 31, ws = lw / G, wl = lw % G;
    const float tol2 = tol * tol;
    float *buf = W;                                    // [2][NSL][2 columns][BS]
    float *bn = extra;                                 // [2][NSL][2] squared norms
    int *bid = reinterpret_cast<int *>(bn + 4 * NSL);  // [2][NSL] block ids
    float F1[RPL], F2[RPL], M1[RPL], M2[RPL];
    auto ld = [&](const float *src, float *r) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int o = (c * G + lane) * VW, i = c * VW;
            if constexpr (VW == 4) {
                const float4 x = *reinterpret_cast<const float4 *>(src + o);
                r[i] = x.x; r[i + 1] = x.y; r[i + 2] = x.z; r[i + 3] = x.w;
            } else {
                const float2 x = *reinterpret_cast<const float2 *>(src + o);
                r[i] = x.x; r[i + 1] = x.y;
            }
        }
    };
    auto st = [&](float *dst, const float *r) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int o = (c * G + lane) * VW, i = c * VW;
            if constexpr (VW == 4) *reinterpret_cast<float4 *>(dst + o) = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
            else *reinterpret_cast<float2 *>(dst + o) = make_float2(r[i], r[i + 1]);
        }
    };
    auto pdot = [&](const float *x, const float *y) {
        unsigned long long a = 0ull;
#pragma unroll
        for (int i = 0; i < RPL; i += 2) a = lg_ffma2(lg_pk2(x[i], x[i + 1]), lg_pk2(y[i], y[i + 1]), a);
        float p0, p1;
        lg_upk2(a, p0, p1);
        return p0 + p1;
    };
    auto red2 = [&](float &a, float &b) {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
    };
    bool rotated_any = false, big_any = false;
    auto apply = [&](float *X, float *Y, float &nx, float &ny, float gam) {
        if (LG_JACOBI32W_QSTOP > 0.0f && gam * gam > LG_JACOBI32W_QSTOP * LG_JACOBI32W_QSTOP * (nx * ny))
            big_any = true;
        if (gam * gam > tol2 * (nx * ny)) {
            float c, s, tt;
            lg_rotation(nx, ny, gam, c, s, tt);
            const unsigned long long c2 = lg_pk2(c, c), s2 = lg_pk2(s, s), ns2 = lg_pk2(-s, -s);
#pragma unroll
            for (int r = 0; r < RPL; r += 2) {
                const unsigned long long x = lg_pk2(X[r], X[r + 1]), y = lg_pk2(Y[r], Y[r + 1]);
                lg_upk2(lg_ffma2(c2, x, lg_fmul2(ns2, y)), X[r], X[r + 1]);
                lg_upk2(lg_ffma2(s2, x, lg_fmul2(c2, y)), Y[r], Y[r + 1]);
            }
            nx = nx - tt * gam;
            ny = ny + tt * gam;
            rotated_any = true;
        }
    };
    // two independent rotations with their inner products reduced together
    auto rot2 = [&](float *X1, float *Y1, float &nx1, float &ny1, float *X2, float *Y2, float &nx2, float &ny2) {
        float g1 = pdot(X1, Y1), g2 = pdot(X2, Y2);
        red2(g1, g2);
        apply(X1, Y1, nx1, ny1, g1);
        apply(X2, Y2, nx2, ny2, g2);
    };
    int sweep, moves = 0;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        if (tid == 0) *s_rot = 0;
        rotated_any = false;
        big_any = false;
        for (int B = NB; B >= 2; B >>= 1) {            // B blocks per group
            const int half = B / 2, u = slot / half, i = slot % half;
            const int fb = u * B + i;
            int mbk = u * B + half + i;
            __syncthreads();                           // W holds every column
            ld(W + (2 * fb) * LD, F1);
            ld(W + (2 * fb + 1) * LD, F2);
            ld(W + (2 * mbk) * LD, M1);
            ld(W + (2 * mbk + 1) * LD, M2);
            float f1 = pdot(F1, F1), f2 = pdot(F2, F2), m1 = pdot(M1, M1), m2 = pdot(M2, M2);
            red2(f1, f2);
            red2(m1, m2);
            __syncthreads();                           // W becomes the hand-over buffers
            for (int t = 0; t < half; t++) {
                rot2(F1, M1, f1, m1, F2, M2, f2, m2);
                rot2(F1, M2, f1, m2, F2, M1, f2, m1);
                if (B == 2) rot2(F1, F2, f1, f2, M1, M2, m1, m2);
                if (t == half - 1) break;
                const bool handover = half > SPW && (t + 1) % SPW == 0;
                if (!handover) {
                    // the next slot of the group inside the warp (cyclic)
                    const int gs = half < SPW ? half : SPW;
                    const int gbase = (ws / gs) * gs;
                    const int src = (gbase + (ws - gbase + 1) % gs) * G + wl;
#pragma unroll
                    for (int r = 0; r < RPL; r++) {
                        M1[r] = __shfl_sync(0xffffffffu, M1[r], src);
                        M2[r] = __shfl_sync(0xffffffffu, M2[r], src);
                    }
                    m1 = __shfl_sync(0xffffffffu, m1, src);
                    m2 = __shfl_sync(0xffffffffu, m2, src);
                    mbk = __shfl_sync(0xffffffffu, mbk, src);
                } else {
                    // the same slot of the next warp of the group
                    const int par = moves & 1;
                    moves++;
                    const int gw = i / SPW, nw = half / SPW;
                    const int ss = u * half + ((gw + 1) % nw) * SPW + ws;
                    float *mine = buf + (size_t)(par * NSL + slot) * 2 * BS;
                    st(mine, M1);
                    st(mine + BS, M2);
                    if (lane == 0) {
                        bn[(par * NSL + slot) * 2] = m1;
                        bn[(par * NSL + slot) * 2 + 1] = m2;
                        bid[par * NSL + slot] = mbk;
                    }
                    __syncthreads();
                    const float *theirs = buf + (size_t)(par * NSL + ss) * 2 * BS;
                    ld(theirs, M1);
                    ld(theirs + BS, M2);
                    m1 = bn[(par * NSL + ss) * 2];
                    m2 = bn[(par * NSL + ss) * 2 + 1];
                    mbk = bid[par * NSL + ss];
                }
            }
            __syncthreads();                           // every read of the buffers is done
            st(W + (2 * fb) * LD, F1);
            st(W + (2 * fb + 1) * LD, F2);
            st(W + (2 * mbk) * LD, M1);
            st(W + (2 * mbk + 1) * LD, M2);
        }
        if (lane == 0 && (rotated_any || big_any)) atomicOr(s_rot, (rotated_any ? 1 : 0) | (big_any ? 2 : 0));
        __syncthreads();
        const int rotated = *s_rot;
        __syncthreads();
        if (!(rotated & 1)) break;
        // the early exit of lg_jacobi32w: a sweep of rotations all below the
        // stop level ends the solve
        if (LG_JACOBI32W_QSTOP > 0.0f && !(rotated & 2)) break;
    }
    return sweep;
}


// FP32 one-sided Jacobi with the hierarchical ordering over blocks of three
// columns, for K = 96 (32 blocks, a power of two): K/6 slots of 256/(K/6)
// lanes each keep a fixed block in registers and rotate it against a moving
// block, nine rotations per step taken three at a time on disjoint pairs
// (F_a with M_(a+s) mod 3 for s = 0, 1, 2) with their inner products reduced
// together; at the last level each block's own three pairs are rotated too.
// A sweep takes K/3 - 1 steps, with a block barrier only where the moving
// blocks pass to another warp (every second step), against K - 1 barriered
// steps of the round-robin lg_jacobi32.  Buffers, norms, the early exit and
// the hand-overs are those of lg_jacobi32b2 with three columns per block.
template <int K, int LD, int BS>
__device__ int lg_jacobi32b3(float *W, float *extra, int *s_rot, float tol, int max_sweeps)
{
    constexpr int BW = 3, NB = K / BW, NSL = NB / 2, G = 256 / NSL, RPL = K / G, SPW = 32 / G;
    constexpr int VW = (RPL % 4 == 0) ? 4 : 2, NC = RPL / VW;
    static_assert(K == 96, "block-3 ordering for K = 96");
    static_assert((NB & (NB - 1)) == 0 && 32 % G == 0 && RPL % 2 == 0, "power-of-two blocks, packed rows");
    static_assert(2 * NSL * BW * BS <= K * LD && LD % VW == 0 && BS % VW == 0, "moving-block buffers fit in W");
    const int tid = threadIdx.x;
    const int slot = tid / G, lane = tid % G;
    const int lw = tid & 31, ws = lw / G, wl = lw % G;
    const float tol2 = tol * tol;
    float *buf = W;                                    // [2][NSL][BW columns][BS]
    float *bn = extra;                                 // [2][NSL][BW] squared norms
    int *bid = reinterpret_cast<int *>(bn + 2 * NSL * BW);   // [2][NSL] block ids
    float F[BW][RPL], M[BW][RPL], fn[BW], mn[BW];
    auto ld = [&](const float *src, float *r) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int o = (c * G + lane) * VW, i = c * VW;
            if constexpr (VW == 4) {
                const float4 x = *reinterpret_cast<const float4 *>(src + o);
                r[i] = x.x; r[i + 1] = x.y; r[i + 2] = x.z; r[i + 3] = x.w;
            } else {
                const float2 x = *reinterpret_cast<const float2 *>(src + o);
                r[i] = x.x; r[i + 1] = x.y;
            }
        }
    };
    auto st = [&](float *dst, const float *r) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int o = (c * G + lane) * VW, i = c * VW;
            if constexpr (VW == 4) *reinterpret_cast<float4 *>(dst + o) = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
            else *reinterpret_cast<float2 *>(dst + o) = make_float2(r[i], r[i + 1]);
        }
    };
    auto pdot = [&](const float *x, const float *y) {
        unsigned long long a = 0ull;
#pragma unroll
        for (int i = 0; i < RPL; i += 2) a = lg_ffma2(lg_pk2(x[i], x[i + 1]), lg_pk2(y[i], y[i + 1]), a);
        float p0, p1;
        lg_upk2(a, p0, p1);
        return p0 + p1;
    };
    auto red3 = [&](float &a, float &b, float &c) {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
    };
    bool rotated_any = false, big_any = false;
    auto apply = [&](float *X, float *Y, float &nx, float &ny, float gam) {
        if (LG_JACOBI32W_QSTOP > 0.0f && gam * gam > LG_JACOBI32W_QSTOP * LG_JACOBI32W_QSTOP * (nx * ny))
            big_any = true;
        if (gam * gam > tol2 * (nx * ny)) {
            float c, s, tt;
            lg_rotation(nx, ny, gam, c, s, tt);
            const unsigned long long c2 = lg_pk2(c, c), s2 = lg_pk2(s, s), ns2 = lg_pk2(-s, -s);
#pragma unroll
            for (int r = 0; r < RPL; r += 2) {
                const unsigned long long x = lg_pk2(X[r], X[r + 1]), y = lg_pk2(Y[r], Y[r + 1]);
                lg_upk2(lg_ffma2(c2, x, lg_fmul2(ns2, y)), X[r], X[r + 1]);
                lg_upk2(lg_ffma2(s2, x, lg_fmul2(c2, y)), Y[r], Y[r + 1]);
            }
            nx = nx - tt * gam;
            ny = ny + tt * gam;
            rotated_any = true;
        }
    };
    int sweep, moves = 0;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        if (tid == 0) *s_rot = 0;
        rotated_any = false;
        big_any = false;
        for (int B = NB; B >= 2; B >>= 1) {            // B blocks per group
            const int half = B / 2, u = slot / half, i = slot % half;
            const int fb = u * B + i;
            int mbk = u * B + half + i;
            __syncthreads();                           // W holds every column
#pragma unroll
            for (int a = 0; a < BW; a++) {
                ld(W + (BW * fb + a) * LD, F[a]);
                ld(W + (BW * mbk + a) * LD, M[a]);
            }
#pragma unroll
            for (int a = 0; a < BW; a++) {
                fn[a] = pdot(F[a], F[a]);
                mn[a] = pdot(M[a], M[a]);
            }
            red3(fn[0], fn[1], fn[2]);
            red3(mn[0], mn[1], mn[2]);
            __syncthreads();                           // W becomes the hand-over buffers
            for (int t = 0; t < half; t++) {
                // the nine pairs of the fixed and the moving block
#pragma unroll
                for (int s = 0; s < BW; s++) {
                    float g0 = pdot(F[0], M[s]), g1 = pdot(F[1], M[(s + 1) % BW]), g2 = pdot(F[2], M[(s + 2) % BW]);
                    red3(g0, g1, g2);
                    apply(F[0], M[s], fn[0], mn[s], g0);
                    apply(F[1], M[(s + 1) % BW], fn[1], mn[(s + 1) % BW], g1);
                    apply(F[2], M[(s + 2) % BW], fn[2], mn[(s + 2) % BW], g2);
                }
                if (B == 2) {
                    // each block's own pairs, the fixed and the moving block's together
#pragma unroll
                    for (int q = 0; q < BW; q++) {
                        const int a = q == 2 ? 1 : 0, b = q == 0 ? 1 : 2;
                        float g0 = pdot(F[a], F[b]), g1 = pdot(M[a], M[b]), g2 = 0.0f;
                        red3(g0, g1, g2);
                        apply(F[a], F[b], fn[a], fn[b], g0);
                        apply(M[a], M[b], mn[a], mn[b], g1);
                    }
                }
                if (t == half - 1) break;
                const bool handover = half > SPW && (t + 1) % SPW == 0;
                if (!handover) {
                    // the next slot of the group inside the warp (cyclic)
                    const int gs = half < SPW ? half : SPW;
                    const int gbase = (ws / gs) * gs;
                    const int src = (gbase + (ws - gbase + 1) % gs) * G + wl;
#pragma unroll
                    for (int a = 0; a < BW; a++) {
#pragma unroll
                        for (int r = 0; r < RPL; r++) M[a][r] = __shfl_sync(0xffffffffu, M[a][r], src);
                        mn[a] = __shfl_sync(0xffffffffu, mn[a], src);
                    }
                    mbk = __shfl_sync(0xffffffffu, mbk, src);
                } else {
                    // the same slot of the next warp of the group
                    const int par = moves & 1;
                    moves++;
                    const int gw = i / SPW, nw = half / SPW;
                    const int ss = u * half + ((gw + 1) % nw) * SPW + ws;
                    float *mine = buf + (size_t)(par * NSL + slot) * BW * BS;
#pragma unroll
                    for (int a = 0; a < BW; a++) st(mine + a * BS, M[a]);
                    if (lane == 0) {
#pragma unroll
                        for (int a = 0; a < BW; a++) bn[(par * NSL + slot) * BW + a] = mn[a];
                        bid[par * NSL + slot] = mbk;
                    }
                    __syncthreads();
                    const float *theirs = buf + (size_t)(par * NSL + ss) * BW * BS;
#pragma unroll
                    for (int a = 0; a < BW; a++) {
                        ld(theirs + a * BS, M[a]);
                        mn[a] = bn[(par * NSL + ss) * BW + a];
                    }
                    mbk = bid[par * NSL + ss];
                }
            }
            __syncthreads();                           // every read of the buffers is done
#pragma unroll
            for (int a = 0; a < BW; a++) {
                st(W + (BW * fb + a) * LD, F[a]);
                st(W + (BW * mbk + a) * LD, M[a]);
            }
        }
        if (lane == 0 && (rotated_any || big_any)) atomicOr(s_rot, (rotated_any ? 1 : 0) | (big_any ? 2 : 0));
        __syncthreads();
        const int rotated = *s_rot;
        __syncthreads();
        if (!(rotated & 1)) break;
        // the early exit of lg_jacobi32w: a sweep of rotations all below the
        // stop level ends the solve
        if (LG_JACOBI32W_QSTOP > 0.0f && !(rotated & 2)) break;
    }
    return sweep;
}

// FP32 one-sided Jacobi of one K x K problem by one warp (K = 64): lane l
// owns a column pair in registers, so the inner products need no reduction
// and a step needs no barrier; the hierarchical ordering passes the moving
// column to the next lane of its group by shuffles, and the columns are
// re-dealt through W (column j at W[j*LD ..], this warp's own memory) at each
// level.  Returns the sweeps used, or max_sweeps+1 if not converged.
template <int K, int LD>
__device__ int lg_jacobi32w(float *W, float tol, int max_sweeps)
{
    constexpr int NS = K / 2;
    static_assert(NS == 32 && LD % 4 == 0, "one lane per column pair");
    const int lane = threadIdx.x & 31;
    const float tol2 = tol * tol;
    float F[K], M[K];
    auto ldc = [&](int col, float *r) {
        const float4 *src = reinterpret_cast<const float4 *>(W + col * LD);
#pragma unroll
        for (int c = 0; c < K / 4; c++) {
            const float4 x = src[c];
            r[4 * c] = x.x; r[4 * c + 1] = x.y; r[4 * c + 2] = x.z; r[4 * c + 3] = x.w;
        }
    };
    auto stc = [&](int col, const float *r) {
        float4 *dst = reinterpret_cast<float4 *>(W + col * LD);
#pragma unroll
        for (int c = 0; c < K / 4; c++) dst[c] = make_float4(r[4 * c], r[4 * c + 1], r[4 * c + 2], r[4 * c + 3]);
    };
    auto dot = [&](const float *x, const float *y) {
        unsigned long long a[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
        for (int i = 0; i < K; i += 8) {
#pragma unroll
            for (int q = 0; q < 4; q++)
                a[q] = lg_ffma2(lg_pk2(x[i + 2 * q], x[i + 2 * q + 1]), lg_pk2(y[i + 2 * q], y[i + 2 * q + 1]), a[q]);
        }
        float s = 0.0f;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float p0, p1;
            lg_upk2(a[q], p0, p1);
            s += p0 + p1;
        }
        return s;
    };
    int sweep;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        bool rot = false, big = false;
        for (int B = K; B >= 2; B >>= 1) {
            const int half = B / 2, u = lane / half, i = lane % half;
            const int fc = u * B + i;
            int mc = u * B + half + i;
            __syncwarp();
            ldc(fc, F);
            ldc(mc, M);
            float fa = dot(F, F), mb = dot(M, M);
            for (int t = 0; t < half; t++) {
                const float gam = dot(F, M);
                if (LG_JACOBI32W_QSTOP > 0.0f && gam * gam > LG_JACOBI32W_QSTOP * LG_JACOBI32W_QSTOP * (fa * mb))
                    big = true;
                if (gam * gam > tol2 * (fa * mb)) {
                    float c, s, tt;
                    lg_rotation(fa, mb, gam, c, s, tt);
                    const unsigned long long c2 = lg_pk2(c, c), s2 = lg_pk2(s, s), ns2 = lg_pk2(-s, -s);
#pragma unroll
                    for (int r = 0; r < K; r += 2) {
                        const unsigned long long x = lg_pk2(F[r], F[r + 1]), y = lg_pk2(M[r], M[r + 1]);
                        lg_upk2(lg_ffma2(c2, x, lg_fmul2(ns2, y)), F[r], F[r + 1]);
                        lg_upk2(lg_ffma2(s2, x, lg_fmul2(c2, y)), M[r], M[r + 1]);
                    }
                    fa = fa - tt * gam;
                    mb = mb + tt * gam;
                    rot = true;
                }
                if (t == half - 1) break;
                // the moving column of the next lane of the group
                const int src = u * half + (i + 1) % half;
#pragma unroll
                for (int r = 0; r < K; r++) M[r] = __shfl_sync(0xffffffffu, M[r], src);
                mb = __shfl_sync(0xffffffffu, mb, src);
                mc = __shfl_sync(0xffffffffu, mc, src);
            }
            __syncwarp();
            stc(fc, F);
            stc(mc, M);
        }
        if (!__any_sync(0xffffffffu, rot)) break;
        // quadratic convergence: after a sweep whose rotations were all below
        // the stop level, the next one would find every pair under tol
        if (LG_JACOBI32W_QSTOP > 0.0f && !__any_sync(0xffffffffu, big)) break;
    }
    __syncwarp();
    return sweep;
}
