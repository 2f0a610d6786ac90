// letkf_jacobi.cuh -- one-sided (Hestenes) Jacobi eigensolve of a symmetric
// positive definite k x k matrix held by columns in shared memory, and the
// lower-triangle 4x4 block numbering of the register-tiled products.
#pragma once

template <typename T> struct LgVec2;
template <> struct LgVec2<double> { using type = double2; };
template <> struct LgVec2<float> { using type = float2; };

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
        for (int r = 0; r < K - 1; r++) {
            int p = 0, q = 0;
            T gam = 0;
            if (act) {
                if (pair == 0) {
                    p = K - 1;
                    q = r;
                } else {
                    p = (r + pair) % (K - 1);
                    q = (r - pair + (K - 1)) % (K - 1);
                }
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
                        const T zeta = (be - al) / (T(2) * g2);
                        const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
                        c = T(1) / sqrt(T(1) + t * t);
                        s = c * t;
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
                    const T zeta = (be - al) / (T(2) * gam);
                    const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
                    const T c = T(1) / sqrt(T(1) + t * t);
                    const T s = c * t;
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
