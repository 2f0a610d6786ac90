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
};

__device__ __forceinline__ void add_lon_range(Seg *seg, int &ns, const LgBuckets &bk, int band,
                                              float lon0, float lon1, int exact)
{
    const int nbl = bk.nblon;
    const int base = band * nbl;
    const float cl = (float)bk.cell_lon;
    int j0 = (int)floorf(lon0 / cl), j1 = (int)floorf(lon1 / cl);
    if (j1 - j0 + 1 >= nbl) {
        if (ns < kMaxSeg) seg[ns++] = {bk.start[base], bk.start[base + nbl], exact};
        return;
    }
    auto add = [&](int a, int b) {
        if (a > b) return;
        if (ns < kMaxSeg) seg[ns++] = {bk.start[base + a], bk.start[base + b + 1], exact};
    };
    if (j0 < 0) {
        add(j0 + nbl, nbl - 1);
        add(0, j1);
    } else if (j1 >= nbl) {
        add(j0, nbl - 1);
        add(0, j1 - nbl);
    } else {
        add(j0, j1);
    }
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
    }
    const int o = __float_as_int(p.w);
    const double dist = lg_dist(geo.s[o], geo.c[o], geo.yr[o], cg.s2, cg.c2, cg.y2r);
    const double ri = lg_ri(dist, prm.local_dist);
    if (fabs(ri - 2.0) < 1e-12) atomicAdd(border, 1ull);
    const double gc = prm.gc_filter ? lg_schr2(ri) : lg_schr(ri);
    return gc > 0.0;
}

// One pass over all candidate segments.
//   mode 0: append every kept index (up to cap), count them and, with hist,
//           count them by bin o >> shift
//   mode 1: count kept indices below `thr`
//   mode 2: append kept indices below `thr`
__device__ int scan_pass(int mode, int thr, const Seg *seg, int ns, const LgBuckets &bk,
                         const CubeGeo &cg, const LgObsGeo &geo, const LgParams &prm,
                         int32_t *keys, int cap, int *s_count, unsigned long long *border,
                         int *hist = nullptr, int shift = 0)
{
    if (threadIdx.x == 0) *s_count = 0;
    __syncthreads();
    for (int si = 0; si < ns; si++) {
        const Seg s = seg[si];
        for (int i = s.b + threadIdx.x; i < s.e; i += kThreads) {
            const float4 p = bk.xyz[i];
            const int o = __float_as_int(p.w);
            if (mode != 0 && o >= thr) continue;
            if (!keep_candidate(p, s.exact, cg, geo, prm, mode == 0 ? border : nullptr)) continue;
            const int pos = atomicAdd(s_count, 1);
            if (mode != 1 && pos < cap) keys[pos] = o;
            if (hist) atomicAdd(&hist[o >> shift], 1);
        }
    }
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
    const float *ef;          // sqrt(rdiaginv) dep per obs (mixed form)
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
    if (prm.precision == LETKF_PREC_MIXED) {
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
        // and e = sqrt(rdiaginv rloc) dep (g = Yhat e)
        const float sr = sqrtf(rl);
        lm.meta[at] = make_float2(sr, sr * lm.ef[o]);
    } else {
        const double dist = lg_dist(geo.s[o], geo.c[o], geo.yr[o], cg.s2, cg.c2, cg.y2r);
        const double ri = lg_ri(dist, prm.local_dist);
        lidx[at] = o;
        lrloc[at] = prm.gc_filter ? lg_schr2(ri) : lg_schr(ri);
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
    return cg;
}

// Bucket segments of the cap of radius 2c around (clat, clon), plus the
// buckets within 1e-6 rad of the antipode (exact test there).  FP32 with
// margins of 1e-4 degrees (and the full circle of longitudes whenever the cap
// comes within 1e-4 rad of a pole): the segments are a superset of the cap.
__device__ int cap_segments(Seg *seg, const LgBuckets &bk, float clat, float clon, float theta)
{
    int ns = 0;
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
    for (int b = b0; b <= b1; b++) {
        if (full) add_lon_range(seg, ns, bk, b, 0.0f, 720.0f, 0);
        else add_lon_range(seg, ns, bk, b, clon - dlon, clon + dlon, 0);
    }
    // buckets within 1e-6 rad of the antipode
    {
        const float alat = -clat, alon = fmodf(clon + 180.0f, 360.0f);
        const float ad = 1e-6f * deg + 1e-4f;
        const int a0 = max(0, (int)floorf((alat - ad + 90.0f) / cla));
        const int a1 = min(bk.nblat - 1, (int)floorf((alat + ad + 90.0f) / cla));
        const float ca = cosf(alat / deg);
        for (int b = a0; b <= a1; b++) {
            if (ca < 1e-3f) add_lon_range(seg, ns, bk, b, 0.0f, 720.0f, 1);
            else add_lon_range(seg, ns, bk, b, alon - ad / ca, alon + ad / ca, 1);
        }
    }
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
    __shared__ int s_ns, s_count, s_bin, s_through;
    __shared__ int s_warp[kThreads / 32];
    __shared__ CubeGeo s_cg;
    __shared__ long long s_off;
    int shift = 0;
    while (((nobs - 1) >> shift) >= kHistBins) shift++;

    for (int64_t cube = prm.cube0 + blockIdx.x; cube < ncubes; cube += gridDim.x) {
        for (int i = threadIdx.x; i < kHistBins; i += kThreads) hist[i] = 0;
        if (threadIdx.x == 0) {
            float clat, clon;
            const CubeGeo cg = cube_geo(g, prm, sgeo, cube, clat, clon);
            s_cg = cg;
            int ns = cap_segments(seg, bk, clat, clon, sgeo.theta);
            if (ns >= kMaxSeg) atomicOr(status, LG_ST_SEGMENTS);
            s_ns = ns;
        }
        __syncthreads();
        const int ns = s_ns;
        const CubeGeo cg = s_cg;

        int nk = scan_pass(0, 0, seg, ns, bk, cg, geo, prm, keys, cap_sort, &s_count,
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
                const int c = scan_pass(1, mid, seg, ns, bk, cg, geo, prm, keys, cap_sort, &s_count,
                                        nullptr);
                if (c >= prm.max_obs) hi = mid; else lo = mid + 1;
            }
            const int c = scan_pass(2, lo, seg, ns, bk, cg, geo, prm, keys, cap_sort, &s_count,
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
__global__ void __launch_bounds__(kThreads)
k_search_bitmap(LgGrid g, LgParams prm, LgSearchGeo sgeo, LgBuckets bk, LgObsGeo geo, LgListMeta lm,
                int64_t nobs,
                int32_t *__restrict__ lidx, double *__restrict__ lrloc, int64_t list_cap,
                int64_t *__restrict__ loff, int32_t *__restrict__ lcnt,
                unsigned long long *__restrict__ counters, unsigned *__restrict__ status, int64_t ncubes)
{
    extern __shared__ uint32_t bits[];
    __shared__ Seg seg[kMaxSeg];
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
        if (threadIdx.x == 0) {
            float clat, clon;
            const CubeGeo cg = cube_geo(g, prm, sgeo, cube, clat, clon);
            s_cg = cg;
            const int ns = cap_segments(seg, bk, clat, clon, sgeo.theta);
            if (ns >= kMaxSeg) atomicOr(status, LG_ST_SEGMENTS);
            s_ns = ns;
        }
        __syncthreads();
        const int ns = s_ns;
        const CubeGeo cg = s_cg;
        for (int si = 0; si < ns; si++) {
            const Seg sg = seg[si];
            for (int i = sg.b + threadIdx.x; i < sg.e; i += kThreads) {
                const float4 p = bk.xyz[i];
                if (keep_candidate(p, sg.exact, cg, geo, prm, &counters[LG_CNT_BORDER])) {
                    const int o = __float_as_int(p.w);
                    atomicOr(&bits[o >> 5], 1u << (o & 31));
                }
            }
        }
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
        if (off >= 0) {
            int pos = before;
            for (int w = w0; w < w1 && pos < nout; w++) {
                uint32_t m = bits[w];
                while (m && pos < nout) {
                    const int b = __ffs(m) - 1;
                    m &= m - 1u;
                    write_entry(w * 32 + b, off + pos, cg, geo, prm, lm, lidx, lrloc);
                    pos++;
                }
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
            g, prm, lg_search_geo(ctx), bk, geo, LgListMeta{ctx->d_oef.p, ctx->d_lmeta.p, ctx->d_lneed.p}, nobs, ctx->d_lidx.p,
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
        g, prm, lg_search_geo(ctx), bk, geo, LgListMeta{ctx->d_oef.p, ctx->d_lmeta.p, ctx->d_lneed.p}, nobs, cap, ctx->d_lidx.p, ctx->d_lrloc.p, ctx->list_cap, ctx->d_loff.p,
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
        g, prm, lg_search_geo(ctx), geo, LgListMeta{ctx->d_oef.p, ctx->d_lmeta.p, ctx->d_lneed.p}, olat, ctx->dec_ny, ctx->dec_nchunk, ctx->d_dec_row_blk.p, ctx->d_dec_col_blk.p,
        ctx->d_dec_slot_off.p, ctx->d_dec_slot_blk.p, ctx->d_dec_pos.p, ctx->d_dec_obs.p, ctx->d_lidx.p,
        ctx->d_lrloc.p, ctx->list_cap, ctx->d_loff.p, ctx->d_lcnt.p, ctx->d_counters.p, ctx->d_status.p,
        ctx->win1);
    return cudaGetLastError();
}
