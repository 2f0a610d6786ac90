// letkf_search.cu -- localized observation search over the bucket grid.
//
// Reference: gen_yb_dis (code/x86/TradDA/DA/LETKF/src/letkf_yb.F90:3-133).  For
// every cube centre the reference scans all candidate obs in canonical order,
// keeps an obs iff |lat| <= obs_polar and gc = schr2(dist/c) > 0, and stops at
// MAX_OBS.  Here one CTA handles one cube:
//   1. it visits only the buckets that intersect the cap of radius 2c (plus
//      the few buckets at the antipode, where rounding can make acos return
//      NaN and schr2(NaN) = 1 keeps the obs, as in the reference);
//   2. a float chord-length test classifies candidates that are clearly
//      inside or outside (a 2e-5 relative margin around 2c); only candidates
//      in the margin get the reference's double-precision formula;
//   3. canonical order: while a bitmap over all obs indices fits shared
//      memory (k_search_bitmap, up to 786,432 obs), every kept obs sets its
//      bit and one ordered pass over the bitmap lists them by index; above
//      that (k_search), kept indices are sorted in shared memory (bitonic),
//      and if more are kept than shared memory holds, a histogram of the kept
//      indices by their high bits (2048 bins, filled in the first pass) gives
//      the bin of the max_obs-th smallest index, and a second pass collects
//      the indices up to that bin (a threshold search inside the bin when
//      even those overflow shared memory); lists stop at max_obs;
//   4. the localization weight of every kept obs is computed with the
//      reference's double formula (FP32 from the chord for the mixed form)
//      and the list is written at a slot reserved with one atomic add.
// The decomposed observation sets (k_search_dec) scan the blocks of the
// cube's neighbour set instead of the buckets.  A count-only launch
// (LgParams::count_only) writes each cube's list length and nothing else:
// the first step of a run whose lists are cut into windows.
#include <climits>

#include "letkf_internal.cuh"

namespace {

constexpr int kMaxSeg = 128;
constexpr int kThreads = 256;
constexpr size_t kBitmapMaxBytes = 96 * 1024;   // obs-index bitmap of k_search_bitmap (786,432 obs)
constexpr int kHistBins = 2048;                   // k_search: kept indices by high bits

struct Seg {
    int b, e, exact;   // [b, e) in bucket order; exact: skip the float prefilter
};

struct CubeGeo {
    double s2, c2, y2r;      // centre sin/cos latitude, longitude (rad)
    float cx, cy, cz;        // centre unit vector
    float lo2, hi2;          // chord^2 thresholds: below lo2 keep, above hi2 drop
    int anti_far;            // exact candidates beyond a 1e-5 chord of the antipode are out
};

// The buckets of band `band` between longitudes lon0 and lon1 (degrees,
// wrapping around the circle) as up to two [b, e) ranges of bucket order.
__device__ __forceinline__ int band_segments(const LgBuckets &bk, int band, float lon0, float lon1, int exact,
                                             Seg &s0, Seg &s1)
{
    const int nbl = bk.nblon;
    const int base = band * nbl;
    const float cl = (float)bk.cell_lon;
    const int j0 = (int)floorf(lon0 / cl), j1 = (int)floorf(lon1 / cl);
    int a0 = 0, e0 = -1, a1 = 0, e1 = -1;       // bucket column ranges [a, e]
    if (j1 - j0 + 1 >= nbl) {
        e0 = nbl - 1;
    } else if (j0 < 0) {
        a0 = j0 + nbl; e0 = nbl - 1;
        e1 = j1;
    } else if (j1 >= nbl) {
        a0 = j0; e0 = nbl - 1;
        e1 = j1 - nbl;
    } else {
        a0 = j0; e0 = j1;
    }
    int n = 0;
    if (a0 <= e0) {
        s0 = {bk.start[base + a0], bk.start[base + e0 + 1], exact};
        n = 1;
    }
    if (a1 <= e1) {
        const Seg t = {bk.start[base + a1], bk.start[base + e1 + 1], exact};
        if (n == 0) s0 = t; else s1 = t;
        n++;
    }
    return n;
}

// Classify one candidate; returns true if kept.  Counts borderline pairs.
__device__ __forceinline__ bool keep_candidate(const float4 &p, int exact, const CubeGeo &cg,
                                               const LgObsGeo &geo, const LgParams &prm,
                                               unsigned long long *border)
{
    if (!exact) {
        const float dx = p.x - cg.cx, dy = p.y - cg.cy, dz = p.z - cg.cz;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > cg.hi2) return false;
        if (d2 < cg.lo2) return true;
    } else if (cg.anti_far) {
        // near the antipode the double distance is about pi (out) unless the
        // acos argument rounds below -1 (NaN, kept), which needs a chord to
        // the antipode far below 1e-5
        const float ax = p.x + cg.cx, ay = p.y + cg.cy, az = p.z + cg.cz;
        if (ax * ax + ay * ay + az * az > 1e-10f) return false;
    }
    const int o = __float_as_int(p.w);
    const double dist = lg_dist(geo.s[o], geo.c[o], geo.yr[o], cg.s2, cg.c2, cg.y2r);
    const double ri = lg_ri(dist, prm.local_dist);
    if (fabs(ri - 2.0) < 1e-12) atomicAdd(border, 1ull);
    const double gc = prm.gc_filter ? lg_schr2(ri) : lg_schr(ri);
    return gc > 0.0;
}

// Visit every candidate of the segments once, four per thread at a time with
// their loads in flight together: f(p, exact) for the candidate's float4
// (unit vector, index in w).
template <typename Fn>
__device__ __forceinline__ void each_candidate(const Seg *seg, const int *soff, int ns, const LgBuckets &bk, Fn &&f)
{
    const int total = soff[ns];
    int si = 0;
    for (int k0 = 0; k0 < total; k0 += 4 * kThreads) {
        int idx[4], ex[4];
        bool v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int k = k0 + u * kThreads + (int)threadIdx.x;
            v[u] = k < total;
            idx[u] = 0;
            ex[u] = 0;
            if (v[u]) {
                while (soff[si + 1] <= k) si++;
                idx[u] = seg[si].b + (k - soff[si]);
                ex[u] = seg[si].exact;
            }
        }
        float4 p[4];
#pragma unroll
        for (int u = 0; u < 4; u++) p[u] = v[u] ? bk.xyz[idx[u]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (v[u]) f(p[u], ex[u]);
    }
}

// One pass over all candidate segments.
//   mode 0: append every kept index (up to cap), count them and, with hist,
//           count them by bin o >> shift
//   mode 1: count kept indices below `thr`
//   mode 2: append kept indices below `thr`
__device__ int scan_pass(int mode, int thr, const Seg *seg, const int *soff, int ns, const LgBuckets &bk,
                         const CubeGeo &cg, const LgObsGeo &geo, const LgParams &prm,
                         int32_t *keys, int cap, int *s_count, unsigned long long *border,
                         int *hist = nullptr, int shift = 0)
{
    if (threadIdx.x == 0) *s_count = 0;
    __syncthreads();
    each_candidate(seg, soff, ns, bk, [&](const float4 &p, int exact) {
        const int o = __float_as_int(p.w);
        if (mode != 0 && o >= thr) return;
        if (!keep_candidate(p, exact, cg, geo, prm, mode == 0 ? border : nullptr)) return;
        const int pos = atomicAdd(s_count, 1);
        if (mode != 1 && pos < cap) keys[pos] = o;
        if (hist) atomicAdd(&hist[o >> shift], 1);
    });
    __syncthreads();
    const int c = *s_count;
    __syncthreads();
    return c;
}

// The bin where the running count of hist[0..kHistBins) reaches target
// (the total is at least target >= 1) and the count up to and including it.
__device__ void hist_select(const int *hist, int target, int *s_bin, int *s_through, int *s_warp)
{
    constexpr int per = kHistBins / kThreads;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    int loc = 0;
#pragma unroll
    for (int i = 0; i < per; i++) loc += hist[t * per + i];
    int incl = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int before = incl - loc;
    for (int w = 0; w < warp; w++) before += s_warp[w];
    if (before < target && before + loc >= target) {
        int run = before;
        for (int i = 0; i < per; i++) {
            run += hist[t * per + i];
            if (run >= target) {
                *s_bin = t * per + i;
                *s_through = run;
                break;
            }
        }
    }
    __syncthreads();
}

__device__ void bitonic_sort(int32_t *keys, int n_pow2)
{
    for (int k2 = 2; k2 <= n_pow2; k2 <<= 1) {
        for (int j = k2 >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n_pow2; i += kThreads) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int32_t a = keys[i], b = keys[ixj];
                    const bool up = (i & k2) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Observation terms the mixed form's list entries carry.
struct LgListMeta {
    const float *ef;          // sqrt(rdiaginv) dep per obs, or null before the departures exist
    float2 *meta;             // out, mixed form only
    int32_t *need;            // out: each cube's list length, written even when the pool is full
};

// One list entry: the obs index and its localization weight (the reference's
// double formula; FP32 from the unit-vector chord for the mixed form, which
// also stores its per-entry factors).
__device__ __forceinline__ void write_entry(int o, long long at, const CubeGeo &cg, const LgObsGeo &geo,
                                            const LgParams &prm, const LgListMeta &lm,
                                            int32_t *__restrict__ lidx, double *__restrict__ lrloc)
{
    if (lg_is_mixed(prm.precision)) {
        // the selection used the reference's double formula where it mattered
        const float scale = (float)(LG_EARTH_A / prm.local_dist);
        const float4 q = geo.xyz[o];
        const float dx = q.x - cg.cx, dy = q.y - cg.cy, dz = q.z - cg.cz;
        const float half = fminf(1.0f, 0.5f * sqrtf(dx * dx + dy * dy + dz * dz));
        const float ri = 2.0f * asinf(half) * scale;
        const float rl = prm.gc_filter ? lg_schr2f(ri) : (ri > 2.0f ? 0.0f : 1.0f);
        lidx[at] = o;
        lrloc[at] = (double)rl;
        // the mixed core's per-entry factors: Yhat = y sqrt(rdiaginv) sqrt(rloc)
        // and e = sqrt(rdiaginv rloc) dep (g = Yhat e); the second waits for
        // the departures when the search runs first (k_list_efactor)
        const float sr = sqrtf(rl);
        lm.meta[at] = make_float2(sr, lm.ef ? sr * lm.ef[o] : 0.0f);
    } else {
        const double dist = lg_dist(geo.s[o], geo.c[o], geo.yr[o], cg.s2, cg.c2, cg.y2r);
        const double ri = lg_ri(dist, prm.local_dist);
        lidx[at] = o;
        lrloc[at] = prm.gc_filter ? lg_schr2(ri) : lg_schr(ri);
    }
}

// Entries at .. at + 3 for the indices o4[u] >= 0 (a prefix of the four),
// their gathers issued together.
__device__ __forceinline__ void write_entries4(const int *o4, long long at, const CubeGeo &cg, const LgObsGeo &geo,
                                               const LgParams &prm, const LgListMeta &lm,
                                               int32_t *__restrict__ lidx, double *__restrict__ lrloc)
{
    if (lg_is_mixed(prm.precision)) {
        const float scale = (float)(LG_EARTH_A / prm.local_dist);
        float4 q[4];
        float ef[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            q[u] = o4[u] >= 0 ? geo.xyz[o4[u]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            ef[u] = (o4[u] >= 0 && lm.ef) ? lm.ef[o4[u]] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (o4[u] < 0) continue;
            const float dx = q[u].x - cg.cx, dy = q[u].y - cg.cy, dz = q[u].z - cg.cz;
            const float half = fminf(1.0f, 0.5f * sqrtf(dx * dx + dy * dy + dz * dz));
            const float ri = 2.0f * asinf(half) * scale;
            const float rl = prm.gc_filter ? lg_schr2f(ri) : (ri > 2.0f ? 0.0f : 1.0f);
            lidx[at + u] = o4[u];
            lrloc[at + u] = (double)rl;
            const float sr = sqrtf(rl);
            lm.meta[at + u] = make_float2(sr, sr * ef[u]);
        }
    } else {
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (o4[u] >= 0) write_entry(o4[u], at + u, cg, geo, prm, lm, lidx, lrloc);
    }
}

// Reserve the cube's slot in the list pool with one atomic add (thread 0;
// the caller synchronizes before reading *s_off).
__device__ __forceinline__ void reserve_list(int nout, bool truncated, int64_t cube, int64_t list_cap,
                                             int64_t *__restrict__ loff, int32_t *__restrict__ lcnt,
                                             int32_t *__restrict__ need,
                                             unsigned long long *__restrict__ counters,
                                             unsigned *__restrict__ status, long long *s_off)
{
    need[cube] = nout;
    long long off = (long long)atomicAdd(&counters[LG_CNT_CURSOR], (unsigned long long)nout);
    if (off + nout > list_cap) {
        atomicOr(status, LG_ST_LIST_FULL);
        off = -1;
    }
    *s_off = off;
    loff[cube] = off < 0 ? 0 : off;
    lcnt[cube] = off < 0 ? 0 : nout;
    atomicAdd(&counters[LG_CNT_SUMP], (unsigned long long)nout);
    atomicMax(&counters[LG_CNT_MAXP], (unsigned long long)nout);
    if (truncated) atomicAdd(&counters[LG_CNT_TRUNC], 1ull);
}

// Reserve the cube's slot in the list pool with one atomic add and write its
// kept obs (keys[0..nout), in list order) with their localization weights.
__device__ void write_list(const int32_t *keys, int nout, bool truncated, int64_t cube, const CubeGeo &cg,
                           const LgObsGeo &geo, const LgParams &prm, const LgListMeta &lm,
                           int32_t *__restrict__ lidx,
                           double *__restrict__ lrloc, int64_t list_cap, int64_t *__restrict__ loff,
                           int32_t *__restrict__ lcnt, unsigned long long *__restrict__ counters,
                           unsigned *__restrict__ status, long long *s_off)
{
    if (threadIdx.x == 0)
        reserve_list(nout, truncated, cube, list_cap, loff, lcnt, lm.need, counters, status, s_off);
    __syncthreads();
    const long long off = *s_off;
    if (off >= 0)
        for (int i = threadIdx.x; i < nout; i += kThreads) write_entry(keys[i], off + i, cg, geo, prm, lm, lidx, lrloc);
}

// Centre geometry of cube (as k_search's): unit vector, sin/cos, the chord
// thresholds of the float prefilter.
__device__ CubeGeo cube_geo(const LgGrid &g, const LgParams &prm, const LgSearchGeo &sg, int64_t cube,
                            float &clat, float &clon)
{
    const int bj = (int)(cube % prm.nbj), bi = (int)(cube / prm.nbj);
    const int sj = bj * prm.cube_step, ej = min(sj + prm.cube_n - 1, g.nlat - 1);
    const int si = bi * prm.cube_step, ei = min(si + prm.cube_n - 1, g.nlon - 1);
    const int cj = ((sj + 1) + (ej + 1)) / 2 - 1, ci = ((si + 1) + (ei + 1)) / 2 - 1;
    clat = g.glat[cj];
    clon = g.glon[ci];
    CubeGeo cg;
    cg.s2 = sg.row_s[cj];
    cg.c2 = sg.row_c[cj];
    cg.y2r = sg.col_yr[ci];
    cg.cx = (float)(cg.c2 * sg.col_cos[ci]);
    cg.cy = (float)(cg.c2 * sg.col_sin[ci]);
    cg.cz = (float)cg.s2;
    cg.lo2 = sg.lo2;
    cg.hi2 = sg.hi2;
    cg.anti_far = sg.anti_far;
    return cg;
}

// Bucket segments of the cap of radius 2c around (clat, clon), plus the
// buckets within 1e-6 rad of the antipode (exact test there).  FP32 with
// margins of 1e-4 degrees (and the full circle of longitudes whenever the cap
// comes within 1e-4 rad of a pole): the segments are a superset of the cap.
// Built by one warp, one latitude band per lane; writes seg[0..ns) and the
// exclusive prefix of their lengths soff[0..ns] and returns ns (at most
// kMaxSeg; *overflow set when the cap needed kMaxSeg or more).
__device__ int cap_segments_warp(Seg *seg, int *soff, const LgBuckets &bk, float clat, float clon, float theta,
                                 bool *overflow)
{
    const int lane = threadIdx.x & 31;
    const float deg = 57.295779513f, cla = (float)bk.cell_lat;
    const float band = (theta + 1e-6f) * deg + 1e-4f;
    const int b0 = max(0, (int)floorf((clat - band + 90.0f) / cla));
    const int b1 = min(bk.nblat - 1, (int)floorf((clat + band + 90.0f) / cla));
    const float clat_r = clat / deg;
    bool full = true;
    float dlon = 360.0f;
    if (fabsf(clat_r) + theta < 1.5707963f - 1e-4f) {
        const float sv = sinf(theta) / cosf(clat_r);
        if (sv < 1.0f - 1e-4f) {
            full = false;
            dlon = (asinf(sv) + 1e-6f) * deg + 1e-4f;
        }
    }
    // buckets within 1e-6 rad of the antipode
    const float alat = -clat, alon = fmodf(clon + 180.0f, 360.0f);
    const float ad = 1e-6f * deg + 1e-4f;
    const int a0 = max(0, (int)floorf((alat - ad + 90.0f) / cla));
    const int a1 = min(bk.nblat - 1, (int)floorf((alat + ad + 90.0f) / cla));
    const float ca = cosf(alat / deg);
    const int nmain = max(0, b1 - b0 + 1), nanti = max(0, a1 - a0 + 1);
    int ns = 0;
    for (int t0 = 0; t0 < nmain + nanti; t0 += 32) {
        const int t = t0 + lane;
        Seg s0{0, 0, 0}, s1{0, 0, 0};
        int n = 0;
        if (t < nmain) {
            if (full) n = band_segments(bk, b0 + t, 0.0f, 720.0f, 0, s0, s1);
            else n = band_segments(bk, b0 + t, clon - dlon, clon + dlon, 0, s0, s1);
        } else if (t < nmain + nanti) {
            if (ca < 1e-3f) n = band_segments(bk, a0 + t - nmain, 0.0f, 720.0f, 1, s0, s1);
            else n = band_segments(bk, a0 + t - nmain, alon - ad / ca, alon + ad / ca, 1, s0, s1);
        }
        int incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int pos = ns + incl - n;
        if (n > 0 && pos < kMaxSeg) seg[pos] = s0;
        if (n > 1 && pos + 1 < kMaxSeg) seg[pos + 1] = s1;
        ns += __shfl_sync(0xffffffffu, incl, 31);
    }
    *overflow = ns >= kMaxSeg;
    ns = min(ns, kMaxSeg);
    __syncwarp();
    // exclusive prefix of the segment lengths, four segments per lane
    int len[4], sum = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int i = lane * 4 + q;
        len[q] = (i < ns) ? seg[i].e - seg[i].b : 0;
        sum += len[q];
    }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    int run = incl - sum;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int i = lane * 4 + q;
        if (i <= ns) soff[i] = run;
        run += len[q];
    }
    static_assert(kMaxSeg == 128, "four segments per lane");
    return ns;
}

__global__ void __launch_bounds__(kThreads)
k_search(LgGrid g, LgParams prm, LgSearchGeo sgeo, LgBuckets bk, LgObsGeo geo, LgListMeta lm, int64_t nobs,
         int cap_sort,
         int32_t *__restrict__ lidx, double *__restrict__ lrloc, int64_t list_cap,
         int64_t *__restrict__ loff, int32_t *__restrict__ lcnt,
         unsigned long long *__restrict__ counters, unsigned *__restrict__ status, int64_t ncubes)
{
    extern __shared__ int32_t keys[];   // cap_sort keys, then kHistBins bins
    int *hist = keys + cap_sort;
    __shared__ Seg seg[kMaxSeg];
    __shared__ int soff[kMaxSeg + 1];
    __shared__ int s_ns, s_count, s_bin, s_through;
    __shared__ int s_warp[kThreads / 32];
    __shared__ CubeGeo s_cg;
    __shared__ long long s_off;
    int shift = 0;
    while (((nobs - 1) >> shift) >= kHistBins) shift++;

    for (int64_t cube = prm.cube0 + blockIdx.x; cube < ncubes; cube += gridDim.x) {
        for (int i = threadIdx.x; i < kHistBins; i += kThreads) hist[i] = 0;
        if (threadIdx.x < 32) {
            float clat, clon;
            const CubeGeo cg = cube_geo(g, prm, sgeo, cube, clat, clon);
            bool over;
            const int ns = cap_segments_warp(seg, soff, bk, clat, clon, sgeo.theta, &over);
            if (threadIdx.x == 0) {
                s_cg = cg;
                if (over) atomicOr(status, LG_ST_SEGMENTS);
                s_ns = ns;
            }
        }
        __syncthreads();
        const int ns = s_ns;
        const CubeGeo cg = s_cg;

        int nk = scan_pass(0, 0, seg, soff, ns, bk, cg, geo, prm, keys, cap_sort, &s_count,
                           &counters[LG_CNT_BORDER], hist, shift);
        if (prm.count_only) {
            if (threadIdx.x == 0) lm.need[cube] = min(nk, prm.max_obs);
            __syncthreads();
            continue;
        }
        int nout;
        if (nk <= cap_sort) {
            int np2 = 1;
            while (np2 < nk) np2 <<= 1;
            for (int i = nk + threadIdx.x; i < np2; i += kThreads) keys[i] = INT_MAX;
            __syncthreads();
            bitonic_sort(keys, np2);
            nout = min(nk, prm.max_obs);
        } else {
            // the histogram bin that holds the max_obs-th smallest kept index
            hist_select(hist, prm.max_obs, &s_bin, &s_through, s_warp);
            const int bin = s_bin;
            const int thr = (int)min((int64_t)(bin + 1) << shift, nobs);
            int lo = thr, hi = thr;
            if (s_through > cap_sort) {
                // even the indices up to that bin overflow: the smallest
                // threshold T inside the bin with max_obs kept indices below it
                lo = (bin << shift) + 1;
            }
            while (lo < hi) {
                const int mid = lo + (hi - lo) / 2;
                const int c = scan_pass(1, mid, seg, soff, ns, bk, cg, geo, prm, keys, cap_sort, &s_count,
                                        nullptr);
                if (c >= prm.max_obs) hi = mid; else lo = mid + 1;
            }
            const int c = scan_pass(2, lo, seg, soff, ns, bk, cg, geo, prm, keys, cap_sort, &s_count,
                                    nullptr);
            int np2 = 1;
            while (np2 < c) np2 <<= 1;
            for (int i = c + threadIdx.x; i < np2; i += kThreads) keys[i] = INT_MAX;
            __syncthreads();
            bitonic_sort(keys, np2);
            nout = min(c, prm.max_obs);
        }
        write_list(keys, nout, nk > prm.max_obs, cube, cg, geo, prm, lm, lidx, lrloc, list_cap, loff, lcnt,
                   counters, status, &s_off);
        __syncthreads();
    }
}

// The search with the kept set held as a bitmap over observation indices
// (when nobs/8 bytes fit in shared memory): each kept candidate sets its bit,
// and one ordered pass over the bitmap yields the list in canonical (index)
// order, so no sort is needed and no list length is limited by shared memory.
__global__ void __launch_bounds__(kThreads, 4)
k_search_bitmap(LgGrid g, LgParams prm, LgSearchGeo sgeo, LgBuckets bk, LgObsGeo geo, LgListMeta lm,
                int64_t nobs,
                int32_t *__restrict__ lidx, double *__restrict__ lrloc, int64_t list_cap,
                int64_t *__restrict__ loff, int32_t *__restrict__ lcnt,
                unsigned long long *__restrict__ counters, unsigned *__restrict__ status, int64_t ncubes)
{
    extern __shared__ uint32_t bits[];
    __shared__ Seg seg[kMaxSeg];
    __shared__ int soff[kMaxSeg + 1];
    __shared__ int s_ns;
    __shared__ CubeGeo s_cg;
    __shared__ long long s_off;
    __shared__ int s_warp[kThreads / 32];
    const int nw = (int)((nobs + 31) / 32);
    const int per = (nw + kThreads - 1) / kThreads;
    const int w0 = min(nw, (int)threadIdx.x * per), w1 = min(nw, w0 + per);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    for (int64_t cube = prm.cube0 + blockIdx.x; cube < ncubes; cube += gridDim.x) {
        for (int w = threadIdx.x; w < nw; w += kThreads) bits[w] = 0u;
        if (threadIdx.x < 32) {
            float clat, clon;
            const CubeGeo cg = cube_geo(g, prm, sgeo, cube, clat, clon);
            bool over;
            const int ns = cap_segments_warp(seg, soff, bk, clat, clon, sgeo.theta, &over);
            if (threadIdx.x == 0) {
                s_cg = cg;
                if (over) atomicOr(status, LG_ST_SEGMENTS);
                s_ns = ns;
            }
        }
        __syncthreads();
        const int ns = s_ns;
        const CubeGeo cg = s_cg;
        each_candidate(seg, soff, ns, bk, [&](const float4 &p, int exact) {
            if (keep_candidate(p, exact, cg, geo, prm, &counters[LG_CNT_BORDER])) {
                const int o = __float_as_int(p.w);
                atomicOr(&bits[o >> 5], 1u << (o & 31));
            }
        });
        __syncthreads();
        // exclusive prefix of the kept counts of each thread's word range
        int cnt = 0;
        for (int w = w0; w < w1; w++) cnt += __popc(bits[w]);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        int before = incl - cnt, total = 0;
#pragma unroll
        for (int w = 0; w < kThreads / 32; w++) {
            before += (w < warp) ? s_warp[w] : 0;
            total += s_warp[w];
        }
        const int nout = min(total, prm.max_obs);
        if (prm.count_only) {
            if (threadIdx.x == 0) lm.need[cube] = nout;
            __syncthreads();
            continue;
        }
        if (threadIdx.x == 0)
            reserve_list(nout, total > prm.max_obs, cube, list_cap, loff, lcnt, lm.need, counters, status,
                         &s_off);
        __syncthreads();
        const long long off = s_off;
        if (off >= 0 && w0 < w1) {
            // this thread's kept indices in order, four entries at a time
            // (their gathers in flight together)
            int pos = before, w = w0;
            uint32_t m = bits[w];
            while (pos < nout) {
                int o4[4];
                int nv = 0;
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    while (m == 0u && w + 1 < w1) m = bits[++w];
                    o4[u] = -1;
                    if (m != 0u && pos + u < nout) {
                        o4[u] = w * 32 + __ffs(m) - 1;
                        m &= m - 1u;
                        nv++;
                    }
                }
                write_entries4(o4, off + pos, cg, geo, prm, lm, lidx, lrloc);
                pos += nv;
                if (nv < 4) break;
            }
        }
        __syncthreads();
    }
}

// Decomposed observation sets: the cube's list is the scan of gen_yb_dis
// (letkf_yb.F90:71-133) over the obs of its block's neighbour blocks, block
// by block in the neighbour order and by index within a block, kept iff
// |lat| <= obs_polar and gc > 0, stopped at max_obs.  An obs that two scanned
// blocks hold is listed twice, as in the reference.  Each chunk of 256
// candidates is tested in parallel and compacted in order (ballots and warp
// totals); candidates whose float chord is near the antipode's take the
// double test, where the reference keeps NaN distances.
__global__ void __launch_bounds__(kThreads)
k_search_dec(LgGrid g, LgParams prm, LgSearchGeo sgeo, LgObsGeo geo, LgListMeta lm,
             const double *__restrict__ olat, int NY,
             int nchunk,
             const int *__restrict__ row_blk, const int *__restrict__ col_blk,
             const int *__restrict__ slot_off, const int *__restrict__ slot_blk,
             const int *__restrict__ blk_pos, const int *__restrict__ blk_obs, int32_t *__restrict__ lidx,
             double *__restrict__ lrloc, int64_t list_cap, int64_t *__restrict__ loff,
             int32_t *__restrict__ lcnt, unsigned long long *__restrict__ counters,
             unsigned *__restrict__ status, int64_t ncubes)
{
    extern __shared__ int32_t keys[];
    __shared__ CubeGeo s_cg;
    __shared__ int s_blk;
    __shared__ int s_warp[kThreads / 32];
    __shared__ long long s_off;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int max_obs = prm.max_obs;

    for (int64_t cube = prm.cube0 + blockIdx.x; cube < ncubes; cube += gridDim.x) {
        if (threadIdx.x == 0) {
            float clat, clon;
            s_cg = cube_geo(g, prm, sgeo, cube, clat, clon);
            const int sj = (int)(cube % prm.nbj), si = (int)(cube / prm.nbj);   // cube_n is 1
            s_blk = row_blk[sj] * NY + col_blk[si];
        }
        __syncthreads();
        const CubeGeo cg = s_cg;
        const int blk = s_blk;
        int n = 0;
        for (int sl = slot_off[blk]; sl < slot_off[blk + 1] && n < max_obs; sl++) {
            const int B = slot_blk[sl];
            const int beg = blk_pos[(int64_t)B * nchunk], end = blk_pos[(int64_t)(B + 1) * nchunk];
            for (int base = beg; base < end && n < max_obs; base += kThreads) {
                const int i = base + threadIdx.x;
                bool keep = false;
                int o = 0;
                if (i < end) {
                    o = blk_obs[i];
                    if (fabs(olat[o]) <= prm.obs_polar) {
                        const float4 p = geo.xyz[o];
                        const float dx = p.x - cg.cx, dy = p.y - cg.cy, dz = p.z - cg.cz;
                        const int exact = (dx * dx + dy * dy + dz * dz) > 3.9999f;
                        keep = keep_candidate(p, exact, cg, geo, prm, &counters[LG_CNT_BORDER]);
                    }
                }
                const unsigned ball = __ballot_sync(0xffffffffu, keep);
                if (lane == 0) s_warp[warp] = __popc(ball);
                __syncthreads();
                int before = 0, all = 0;
#pragma unroll
                for (int w = 0; w < kThreads / 32; w++) {
                    before += (w < warp) ? s_warp[w] : 0;
                    all += s_warp[w];
                }
                const int pos = n + before + __popc(ball & ((1u << lane) - 1u));
                if (keep && pos < max_obs) keys[pos] = o;
                n += all;
                __syncthreads();
            }
        }
        if (prm.count_only) {
            if (threadIdx.x == 0) lm.need[cube] = min(n, max_obs);
        } else {
            write_list(keys, min(n, max_obs), n >= max_obs, cube, cg, geo, prm, lm, lidx, lrloc, list_cap,
                       loff, lcnt, counters, status, &s_off);
        }
        __syncthreads();
    }
}

}  // namespace

int lg_search_cap(int max_obs)
{
    int c = 1024;
    while (c < max_obs) c <<= 1;
    return c;
}

namespace {

// meta[i].y = meta[i].x * ef[lidx[i]] for the entries of the last search
// (the first *cursor of the pool).
__global__ void k_list_efactor(const int32_t *__restrict__ lidx, float2 *__restrict__ meta,
                               const float *__restrict__ ef, const unsigned long long *__restrict__ cursor,
                               int64_t cap)
{
    const int64_t n = min((int64_t)*cursor, cap);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float2 m = meta[i];
        m.y = m.x * ef[lidx[i]];
        meta[i] = m;
    }
}

}  // namespace

cudaError_t lg_launch_list_efactor(letkf_ctx *ctx)
{
    lg_count_launch();
    k_list_efactor<<<152 * 8, 256, 0, ctx->stream>>>(ctx->d_lidx.p, ctx->d_lmeta.p, ctx->d_oef.p,
                                                     ctx->d_counters.p + LG_CNT_CURSOR, ctx->list_cap);
    return cudaGetLastError();
}

cudaError_t lg_launch_search(letkf_ctx *ctx, const LgGrid &g, int64_t nobs)
{
    const LgParams prm = lg_params(ctx);
    LgBuckets bk;
    bk.nblat = ctx->nblat;
    bk.nblon = ctx->nblon;
    bk.cell_lat = ctx->cell_lat;
    bk.cell_lon = ctx->cell_lon;
    bk.start = ctx->d_bstart.p;
    bk.idx = ctx->d_bidx.p;
    bk.xyz = ctx->d_bxyz.p;
    LgObsGeo geo{ctx->d_os.p, ctx->d_oc.p, ctx->d_oyr.p, ctx->d_oxyz.p};
    const int64_t nwin = ctx->win1 - ctx->win0;
    const int64_t blocks = nwin < (1 << 30) ? nwin : (1 << 30);
    const size_t bitmap_bytes = sizeof(uint32_t) * (size_t)((nobs + 31) / 32 > 0 ? (nobs + 31) / 32 : 1);
    if (bitmap_bytes <= kBitmapMaxBytes) {
        cudaError_t e = cudaFuncSetAttribute(k_search_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)bitmap_bytes);
        if (e != cudaSuccess) return e;
        lg_count_launch();
        k_search_bitmap<<<(unsigned)(blocks > 0 ? blocks : 1), kThreads, bitmap_bytes, ctx->stream>>>(
            g, prm, lg_search_geo(ctx), bk, geo, LgListMeta{ctx->lists_need_ef ? nullptr : ctx->d_oef.p, ctx->d_lmeta.p, ctx->d_lneed.p}, nobs, ctx->d_lidx.p,
            ctx->d_lrloc.p, ctx->list_cap, ctx->d_loff.p, ctx->d_lcnt.p, ctx->d_counters.p, ctx->d_status.p,
            ctx->win1);
        return cudaGetLastError();
    }
    const int cap = lg_search_cap(prm.max_obs);
    const size_t smem = sizeof(int32_t) * (cap + kHistBins);
    cudaError_t e = cudaFuncSetAttribute(k_search, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    lg_count_launch();
    k_search<<<(unsigned)(blocks > 0 ? blocks : 1), kThreads, smem, ctx->stream>>>(
        g, prm, lg_search_geo(ctx), bk, geo, LgListMeta{ctx->lists_need_ef ? nullptr : ctx->d_oef.p, ctx->d_lmeta.p, ctx->d_lneed.p}, nobs, cap, ctx->d_lidx.p, ctx->d_lrloc.p, ctx->list_cap, ctx->d_loff.p,
        ctx->d_lcnt.p, ctx->d_counters.p, ctx->d_status.p, ctx->win1);
    return cudaGetLastError();
}

cudaError_t lg_launch_search_dec(letkf_ctx *ctx, const LgGrid &g, const double *olat)
{
    const LgParams prm = lg_params(ctx);
    LgObsGeo geo{ctx->d_os.p, ctx->d_oc.p, ctx->d_oyr.p, ctx->d_oxyz.p};
    const int cap = lg_search_cap(prm.max_obs);
    const size_t smem = sizeof(int32_t) * cap;
    cudaError_t e = cudaFuncSetAttribute(k_search_dec, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t nwin = ctx->win1 - ctx->win0;
    const int64_t blocks = nwin < (1 << 30) ? nwin : (1 << 30);
    lg_count_launch();
    k_search_dec<<<(unsigned)(blocks > 0 ? blocks : 1), kThreads, smem, ctx->stream>>>(
        g, prm, lg_search_geo(ctx), geo, LgListMeta{ctx->lists_need_ef ? nullptr : ctx->d_oef.p, ctx->d_lmeta.p, ctx->d_lneed.p}, olat, ctx->dec_ny, ctx->dec_nchunk, ctx->d_dec_row_blk.p, ctx->d_dec_col_blk.p,
        ctx->d_dec_slot_off.p, ctx->d_dec_slot_blk.p, ctx->d_dec_pos.p, ctx->d_dec_obs.p, ctx->d_lidx.p,
        ctx->d_lrloc.p, ctx->list_cap, ctx->d_loff.p, ctx->d_lcnt.p, ctx->d_counters.p, ctx->d_status.p,
        ctx->win1);
    return cudaGetLastError();
}
