// letkf_internal.cuh -- shared definitions of the GB300 LETKF kernels and host code.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "letkf_gpu.h"

// ---------------------------------------------------------------------------
// Constants of the reference's distance and localization functions.
// pi = atan(1.0)*4 in single precision (code/x86/TradDA/DA/utils/pro_info.F90:156),
// a = 6371.393 as a default-real literal (pro_info.F90:148), and the
// default-real literals of schr2 (DA/LETKF/src/letkf_yb.F90:256-261), all
// promoted to double exactly as the Fortran promotes them.
#define LG_PI_F32 3.1415927410125732421875
#define LG_EARTH_A 6371.39306640625
#define LG_GC_C1 1.66666698455810546875
#define LG_GC_C2 0.666666686534881591796875

#define LG_THREADS 256          // threads of the per-cube kernels
#ifndef LG_MBAR_SPIN_LIMIT
#define LG_MBAR_SPIN_LIMIT (1u << 22)   // polls of a bounded tensor-core wait
#endif
#define LG_MAX_ENS 128          // largest ensemble the kernels are built for
// The one-launch mixed cores (k != 64) warm-start each cube's eigensolve from
// the cube before it only inside aligned runs of this many cubes, and their
// work-queue chunks are multiples of it: a cube's result does not depend on
// the chunk size.  (The staged k = 64 core's eigensolve runs are 8 cubes.)
#define LG_WARM_RUN 16

// The precision forms whose products run on the tensor cores.
__host__ __device__ __forceinline__ bool lg_is_mixed(int precision)
{
    return precision == LETKF_PREC_MIXED || precision == LETKF_PREC_MIXED_F64EIG;
}

// Status bits written by kernels into ctx->d_status.
#define LG_ST_BAD_OBS      1u   // obs outside the grid / bad variable or level
#define LG_ST_LIST_FULL    2u   // local-list storage too small
#define LG_ST_NOT_CONV     4u   // an eigensolve hit its sweep limit
#define LG_ST_SEGMENTS     8u   // a cap needed more bucket segments than the search holds
#define LG_ST_TIMEOUT     16u   // a bounded wait on the tensor cores ran out
#define LG_ST_BAD_STATE   32u   // a background member is NaN (members entry point)

// Counters in ctx->d_counters.
enum {
    LG_CNT_CURSOR = 0,    // list allocation cursor
    LG_CNT_SUMP,
    LG_CNT_MAXP,
    LG_CNT_TRUNC,
    LG_CNT_BORDER,
    LG_CNT_NOTCONV,
    LG_CNT_MAXSWEEP,
    LG_CNT_SUMSWEEP,
    LG_CNT_ILLCOND,
    LG_CNT_QUEUE,         // work-queue cursor of the mixed core
    LG_CNT_N
};

// ---------------------------------------------------------------------------
// Exact-arithmetic helpers: every operation rounded separately (no fused
// multiply-add), matching the left-to-right evaluation of the Fortran source.
__device__ __forceinline__ double lg_rad(double deg)
{
    return __dmul_rn(__ddiv_rn(deg, 180.0), LG_PI_F32);
}

// schr2, DA/LETKF/src/letkf_yb.F90:245-269.  NaN fails every test -> 1.0.
__device__ __forceinline__ double lg_schr2(double ri)
{
    if (ri > 2.0) return 0.0;
    if (ri > 1.0) {
        double rj = __dsub_rn(__ddiv_rn(ri, 12.0), 0.5);
        rj = __dadd_rn(__dmul_rn(rj, ri), 0.625);
        rj = __dadd_rn(__dmul_rn(rj, ri), LG_GC_C1);
        return __dsub_rn(__dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(rj, ri), 5.0), ri), 4.0),
                         __ddiv_rn(LG_GC_C2, ri));
    }
    if (ri > 0.0) {
        double rk = __dmul_rn(ri, ri);
        double rj = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(-0.25, ri), 0.5), ri), 0.625);
        return __dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(rj, ri), LG_GC_C1), rk), 1.0);
    }
    return 1.0;
}

// schr2 evaluated in FP32 with the same (default-real) literals, for
// localization weights of the mixed-precision form; clamped at zero.
__device__ __forceinline__ float lg_schr2f(float ri)
{
    if (ri > 2.0f) return 0.0f;
    float r;
    if (ri > 1.0f) {
        float rj = ri / 12.0f - 0.5f;
        rj = rj * ri + 0.625f;
        rj = rj * ri + 1.666667f;
        r = (rj * ri - 5.0f) * ri + 4.0f - 0.6666667f / ri;
    } else if (ri > 0.0f) {
        const float rk = ri * ri;
        const float rj = (-0.25f * ri + 0.5f) * ri + 0.625f;
        r = (rj * ri - 1.666667f) * rk + 1.0f;
    } else {
        r = 1.0f;
    }
    return r > 0.0f ? r : 0.0f;
}

// schr (box-car), letkf_yb.F90:270-285.
__device__ __forceinline__ double lg_schr(double ri) { return (ri > 2.0) ? 0.0 : 1.0; }

// latlon_dist_r8 (pro_info.F90:149-161) with sin/cos of both latitudes and
// the longitudes in radians precomputed: a*acos(min(c1*c2*cos(y1-y2)+s1*s2, 1)).
__device__ __forceinline__ double lg_dist(double s1, double c1, double y1r,
                                          double s2, double c2, double y2r)
{
    double v = __dadd_rn(__dmul_rn(__dmul_rn(c1, c2), cos(__dsub_rn(y1r, y2r))),
                         __dmul_rn(s1, s2));
    if (v > 1.0) v = 1.0;
    return __dmul_rn(LG_EARTH_A, acos(v));
}

// ri = obs_dist * 1d0 / local_dist (letkf_yb.F90:89)
__device__ __forceinline__ double lg_ri(double dist, double local_dist)
{
    return __ddiv_rn(__dmul_rn(dist, 1.0), local_dist);
}

// ---------------------------------------------------------------------------
// Device-side parameter blocks passed by value to kernels.
struct LgGrid {
    int nlat, nlon, nz, nvar2d, nvar3d, k, n;
    int ps_row;
    double p0, ptop;
    const float *glat;    // nlat+1 (last = 90)
    const float *glon;    // nlon+1 (last = 360)
    const double *hyai, *hybi;
};

struct LgParams {
    double local_dist, vert_dist, inflation, obs_polar;
    int gc_filter, gc_filter_vertical, max_obs, cube_n, cube_nz, overlap, h_mode, precision;
    int nbj, nbi;         // cube counts along lat and lon
    int cube_step;        // grid points between cube starts (cube_n - overlap)
    int64_t cube0;        // first cube of the launch's window
    int count_only;       // search: only each cube's list length (LgListMeta::need)
    uint32_t spin_limit;  // polls of each bounded mbarrier wait of the mixed cores
    // The caller's conversion around the analysis fused into it
    // (letkf_gpu_run_members, run_da_parallel in module_da_parallel.F90:
    // 163-261): the state input is the full members and there is no mean
    // array; H reads the members as they are, the update forms each row's
    // mean (sum / real(ens)) and perturbations as it reads the row, and writes
    // the blended members gamma1 (axb + xb) + gamma2 (axa + xa) in place of the
    // analysis perturbations (the background where |grid_lat| > polar) and the
    // background and analysis spreads to spb, spa instead of the mean.
    int members;
    double gamma1, gamma2, polar;
    double *spb, *spa;
};

// Lat-lon bucket grid of the observations.
struct LgBuckets {
    int nblat, nblon;
    double cell_lat, cell_lon;   // 180/nblat and 360/nblon degrees
    const int *start;     // nblat*nblon+1
    const int *idx;       // obs index, bucket order
    const float4 *xyz;    // unit vector (x, y, z) and obs index bits, bucket order
};

// Per-obs precomputed search data (original order).
// Geometry of the cube centres for the search: sin/cos of the grid latitudes,
// the grid longitudes in radians with their cos/sin, the cut-off angle and the
// chord^2 band of the float prefilter.
struct LgSearchGeo {
    const double *row_s, *row_c;
    const double *col_yr, *col_cos, *col_sin;
    float theta, lo2, hi2;
    // the cap stays far from the antipode's buckets: there only obs within a
    // chord of 1e-5 of the antipode (where the double acos can give NaN)
    // need the double test, the rest are out
    int anti_far;
};

struct LgObsGeo {
    const double *s, *c, *yr;   // sin, cos of latitude, longitude in radians
    const float4 *xyz;          // unit vector (x, y, z) and index bits, obs order
};

// ---------------------------------------------------------------------------
// Grow-only device buffer.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t reserve(size_t count)
    {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t bytes = (count ? count : 1) * sizeof(T);
        cudaError_t e = cudaMalloc((void **)&p, bytes);
        if (e == cudaSuccess) n = count ? count : 1;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
};

// Copies on one stream: after the main-stream point `after` (if any), the
// parts in one direction (height 1: a plain copy of width bytes; else width
// bytes of each of height lines, pitches apart), then the event `done`.
struct LgCopyJob {
    cudaStream_t stream = nullptr;
    cudaEvent_t after = nullptr, done = nullptr;
    cudaMemcpyKind kind = cudaMemcpyDefault;
    struct Part {
        void *dst;
        size_t dpitch;
        const void *src;
        size_t spitch;
        size_t width, height;
    };
    std::vector<Part> part;
};

// A host thread that issues copy jobs in order.  A cudaMemcpyAsync between
// the device and pageable host memory returns only when the runtime has moved
// the bytes, so issued by the thread that enqueues the analysis it would hold
// every later launch behind the copy; issued here, the launches go on and the
// copies keep the host link busy beside them.
class LgCopyAgent {
  public:
    explicit LgCopyAgent(int device);
    ~LgCopyAgent();     // issues what is queued, then joins the thread
    // queues a job; returns its number (1, 2, ... over the agent's life)
    uint64_t push(const LgCopyJob &job);
    // waits until job `seq` and those before it have been issued
    void wait_issued(uint64_t seq);
    // waits until every pushed job has been issued (pageable copies: done);
    // returns and clears the first error of those jobs
    cudaError_t drain();
    LgCopyAgent(const LgCopyAgent &) = delete;
    LgCopyAgent &operator=(const LgCopyAgent &) = delete;

  private:
    void loop();
    int device_;
    std::mutex mu_;
    std::condition_variable work_, idle_;
    std::deque<LgCopyJob> queue_;
    bool stop_ = false;
    uint64_t pushed_ = 0, issued_ = 0;
    cudaError_t err_ = cudaSuccess;
    std::thread thread_;
};

struct letkf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    letkf_params params{};
    int nlat = 0, nlon = 0, nz = 0, nvar2d = 0, nvar3d = 0, k = 0, n = 0, ps_row = 0;
    double p0 = 0, ptop = 0;
    int64_t ncol = 0, ncubes = 0;
    int64_t win0 = 0, win1 = 0;       // cube window of the current search and core launches
    int64_t range0 = 0, range1 = 0;   // cubes a run analyses (letkf_gpu_set_cube_range)
    int nbj = 0, nbi = 0;
    bool have_hybrid = false;

    DevBuf<float> d_glat, d_glon;
    DevBuf<double> d_hyai, d_hybi;
    DevBuf<double> d_xb, d_axb, d_xa, d_axa;          // host-pointer runs
    DevBuf<double> d_spb, d_spa;                      // members entry point: spreads
    // observations
    DevBuf<double> d_olat, d_olon, d_oph, d_oyo, d_orinv;
    DevBuf<int32_t> d_olev, d_ovar;
    DevBuf<double> d_yb, d_dep;
    DevBuf<double> d_olnp;        // vertical localization: ln(ph) per obs
    // observations built on the device from raw obs-store buffers (letkf_ingest.cu)
    DevBuf<double> d_plat, d_plon, d_pph, d_pyo, d_prinv;
    DevBuf<int32_t> d_plev, d_pvar, d_pvarof;
    DevBuf<float> d_raw;
    // staged mixed core (k = 64): per cube A, X (k x k FP32), g (FP64), lambda
    DevBuf<float> d_mA, d_mX, d_mlam;
    DevBuf<double> d_mg;
    DevBuf<float> d_ys32;         // yb * sqrt(rinv) in FP32 (mixed precision)
    DevBuf<float> d_rinvf;
    DevBuf<float> d_oef;          // mixed form: sqrt(rdiaginv) dep per obs
    DevBuf<unsigned> d_ymax;      // mixed form: bits of the largest |ys32| or |oef| (H)
    DevBuf<double> d_row_s, d_row_c, d_col_yr, d_col_cos, d_col_sin;   // search geometry tables
    DevBuf<double> d_os, d_oc, d_oyr;
    DevBuf<float4> d_oxyz;
    DevBuf<int> d_obucket;
    // bucket grid
    int nblat = 0, nblon = 0;
    double cell_lat = 1.0, cell_lon = 1.0;
    DevBuf<int> d_bcount, d_bstart, d_bidx;
    DevBuf<float4> d_bxyz;
    // local lists
    DevBuf<int64_t> d_loff;
    DevBuf<int32_t> d_lcnt;
    DevBuf<int32_t> d_lidx;
    DevBuf<double> d_lrloc;
    DevBuf<float2> d_lmeta;       // mixed form: (sqrt(rloc), sqrt(rdiaginv rloc) dep) per entry
    DevBuf<int32_t> d_lneed;      // each cube's list length from the last search
    int64_t list_cap = 0;
    int64_t list_limit = 0;       // most list entries the pool may hold (0: from free memory)
    bool lists_whole = false;     // the pool holds every cube's list of the last run
    int last_windows = 0;         // cube windows of the last run
    bool count_pass = false;      // the next search only counts (lg_params.count_only)
    // decomposed observation sets (letkf_decomp.cu)
    int dec_nx = 0, dec_ny = 0, dec_nchunk = 0;
    DevBuf<double> d_dec_box;                    // lat0[nx], lat1[nx], lon0[ny], lon1[ny]
    DevBuf<int> d_dec_row_blk, d_dec_col_blk;    // lat block of each row, lon block of each column
    DevBuf<int> d_dec_slot_off, d_dec_slot_blk;  // neighbour blocks of each block, scan order
    DevBuf<int> d_dec_cnt, d_dec_pos, d_dec_obs; // per (block, chunk) counts, offsets; obs of blocks
    // mixed core schedule (0: defaults) and its work queue
    int sched_chunk = 0, sched_p0 = 0;
    // polls of each bounded tensor-core wait (letkf_gpu_set_wait_limit; < 0: the default)
    int64_t wait_limit = -1;
    DevBuf<int> d_queue;
    // the staged k = 64 core's eigensolve runs (8 cubes, by cube / 8): the
    // sweeps each took in the last call, and a block's runs ordered longest
    // first by them (the next call's warps take the long runs first)
    DevBuf<int> d_runcost, d_rorder;
    // per-cube results
    DevBuf<double> d_trans, d_w;
    // core_batch staging
    DevBuf<double> d_bhx, d_bdep, d_brloc;
    DevBuf<float> d_brdi;
    DevBuf<int64_t> d_boff;
    // status
    DevBuf<unsigned int> d_status;
    DevBuf<unsigned long long> d_counters;
    int64_t last_nobs = -1;
    bool have_run = false;

    cudaEvent_t ev[8] = {};
    // device-event marks around each launch of the staged core's stages (A
    // build, eigensolve, update, FP64 refinement; letkf_stats.ms_stage), at
    // most kStageMarks launches per stage and run
    static constexpr int kStages = 4, kStageMarks = 32;
    cudaEvent_t stg_ev[kStages][2][kStageMarks] = {};
    int stg_n[kStages] = {};
    letkf_stats stats{};
    std::string last_error;

    // Host copies beside the analysis (letkf_gpu_run with host pointers): the
    // state goes in on the copy streams in parts, and the staged k = 64 core
    // hands each finished block of cubes to lg_sink_columns, which copies its
    // analysis columns out on a copy stream while the next block runs.
    static constexpr int kCopyStreams = 2;
    cudaStream_t cstream[kCopyStreams] = {};
    cudaEvent_t cev[kCopyStreams] = {};      // a copy stream's work so far
    cudaEvent_t sev[kCopyStreams] = {};      // the main stream's work before a copy
    double *sink_xa = nullptr, *sink_axa = nullptr;          // host outputs, or null
    const double *sink_dxa = nullptr, *sink_daxa = nullptr;  // device outputs
    int sink_next = 0;
    int64_t sink_cols = 0;                   // columns handed to the copy streams
    // a host buffer of the run is pageable: the copy-stream copies go
    // through the copy agent, each job with its own main-stream event
    bool agent_on = false;
    // The state copy of a run with host buffers, in pieces of columns: piece
    // i holds columns [piece_c0[i], piece_c1[i]) (xb and axb), its copy
    // stream records pev[i] once they are in, and piece_seq[i] is its copy
    // agent job (0: issued by the calling thread).  lg_state_wait makes the
    // main stream wait for the pieces a launch reads.
    static constexpr int kPieces = 8;
    cudaEvent_t pev[kPieces] = {};
    int64_t piece_c0[kPieces] = {}, piece_c1[kPieces] = {};
    uint64_t piece_seq[kPieces] = {};
    bool piece_waited[kPieces] = {};
    int npieces = 0;
    // H reads the state rows it needs straight from the host arrays through
    // these device views (null: H waits for the whole state), while the bulk
    // copy runs; d_rowmark marks the (column, row) pairs already read
    const double *gather_xb = nullptr, *gather_axb = nullptr;
    bool gathered = false;                   // this run's H rows come from the gather
    cudaEvent_t gev = nullptr;               // the gather done (first copy stream)
    // the host arrays of a state copy that lg_run_analysis starts once the
    // observations are staged (small copies that would otherwise queue
    // behind the bulk copy on the copy engines)
    const double *copy_xb = nullptr, *copy_axb = nullptr;
    int host_read = 1;                       // letkf_gpu_set_host_read
    DevBuf<unsigned> d_rowmark;
    // the host arrays' column layout: column c (c % nlat along latitude,
    // c / nlat along longitude) sits at host column host_off + c % nlat +
    // host_ld * (c / nlat); host_ld = nlat, host_off = 0 without a halo
    int64_t host_ld = 0, host_off = 0;
    std::unique_ptr<LgCopyAgent> agent;
    std::vector<cudaEvent_t> agent_ev;
    size_t agent_ev_next = 0;
    // H on the members waits for the state copy: the geometry, buckets and
    // search run while it is on the way, and the first core launch runs the
    // members pass first (lg_members_if_pending)
    bool members_pending = false;
    const double *pend_xb = nullptr, *pend_axb = nullptr;
    const double *pend_lat = nullptr, *pend_lon = nullptr, *pend_ph = nullptr, *pend_yo = nullptr,
                 *pend_rinv = nullptr;
    const int32_t *pend_lev = nullptr, *pend_var = nullptr;
    int64_t pend_no = 0;
    // the search ran before the departures: its list entries hold sqrt(rloc)
    // only, and each core launch first completes them (lg_launch_list_efactor)
    bool lists_need_ef = false;
    // a fused members run is in progress (LgParams::members and the blend)
    bool members_on = false;
    double members_g1 = 0.0, members_g2 = 1.0, members_polar = 90.0;
    double *members_spb = nullptr, *members_spa = nullptr;
};

// ---------------------------------------------------------------------------
// Launch counting (every kernel launch of this library goes through it).
void lg_count_launch();
// Device-event mark before (end = false) or after a launch of stage s of the
// staged core (0 A build, 1 eigensolve, 2 update, 3 FP64 refinement of the
// eigenpairs); skipped while the stream
// is being captured into a graph.
void lg_stage_mark(letkf_ctx *ctx, int s, bool end);

// Kernel launchers (letkf_prep.cu, letkf_search.cu, letkf_core.cu).
// H: mode 0 everything; 1 the per-observation geometry, weights and bucket
// (no state read); 2 the members, the means and the departures.
// Copy the state rows the observation operator reads from the host arrays
// (device views hxb, haxb in the run's host layout) into dxb, daxb.
cudaError_t lg_launch_gather_rows(letkf_ctx *ctx, cudaStream_t stream, const LgGrid &g, int64_t nobs,
                                  const double *olat, const double *olon, const double *oph,
                                  const int32_t *olev, const int32_t *ovar, const double *hxb,
                                  const double *haxb, double *dxb, double *daxb);
// Make the main stream wait for the pieces of the state copy that hold
// columns [c0, c1) (no-op when the state is not being copied in).
cudaError_t lg_state_wait(letkf_ctx *ctx, int64_t c0, int64_t c1);
cudaError_t lg_launch_obs_prepare(letkf_ctx *ctx, const LgGrid &g, const double *xb,
                                  const double *axb, int64_t nobs, const double *olat,
                                  const double *olon, const double *oph, const int32_t *olev,
                                  const int32_t *ovar, const double *oyo, const double *orinv, int mode = 0);
// The members pass of H when a run deferred it behind the state copy.
cudaError_t lg_members_if_pending(letkf_ctx *ctx);
cudaError_t lg_launch_buckets(letkf_ctx *ctx, int64_t nobs);
void lg_launch_scan_exclusive(const int *in, int *out, int n, cudaStream_t stream);
cudaError_t lg_launch_geo_tables(letkf_ctx *ctx);
LgSearchGeo lg_search_geo(letkf_ctx *ctx);
cudaError_t lg_launch_search(letkf_ctx *ctx, const LgGrid &g, int64_t nobs);
// The second factor of the mixed form's list entries of the last search,
// sqrt(rloc) sqrt(rdiaginv) dep, once the departures exist.
cudaError_t lg_launch_list_efactor(letkf_ctx *ctx);
// decomposed observation sets (letkf_decomp.cu, letkf_search.cu)
int lg_decomp_dims(int nranks, int &lat_blocks, int &lon_blocks);
cudaError_t lg_decomp_setup(letkf_ctx *ctx, const std::vector<float> &glat_ext,
                            const std::vector<float> &glon_ext);
cudaError_t lg_launch_block_members(letkf_ctx *ctx, int64_t nobs, const double *olat, const double *olon);
cudaError_t lg_launch_search_dec(letkf_ctx *ctx, const LgGrid &g, const double *olat);
// Overlapped cubes: every column's analysis is the average over the cubes
// that cover it, from the cubes' trans (with w) in ctx->d_trans.
cudaError_t lg_launch_overlap_update(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb,
                                     double *xa, double *axa);
cudaError_t lg_launch_obs_lnp(letkf_ctx *ctx, int64_t nobs, const double *oph);
// Copy the analysis columns of cubes [c0, c1) (one column per cube) to the
// host outputs of a letkf_gpu_run on a copy stream, after the main stream's
// work so far; no-op without host outputs.
cudaError_t lg_sink_columns(letkf_ctx *ctx, int64_t c0, int64_t c1);
// Issue one copy job on its stream (from the calling thread).
cudaError_t lg_issue_copy(const LgCopyJob &j);

// The analysis of letkf_gpu_run on device state: observations staged (host or
// device pointers), H, search and core (cube windows), overlapped-cube
// averaging; events 1-4 recorded.  state_in_flight: dxb is still being
// copied in on the copy streams (H on the members waits for it).
// lg_finish_run records event 5, reads the status and counters, fills the
// stats and maps the status to a return code.
int lg_run_analysis(letkf_ctx *ctx, const letkf_obs *obs, bool host_obs, const double *dxb,
                    const double *daxb, double *dxa, double *daxa, unsigned long long *cnt,
                    bool state_in_flight = false);
int lg_finish_run(letkf_ctx *ctx, const letkf_obs *obs, unsigned long long *cnt);
int lg_check_run(letkf_ctx *ctx, const letkf_obs *obs);
int lg_reset_status(letkf_ctx *ctx);
int lg_read_status(letkf_ctx *ctx, unsigned &status, unsigned long long *cnt);
int lg_set_err(letkf_ctx *ctx, int code, const char *msg);
cudaError_t lg_launch_core_fp64(letkf_ctx *ctx, const LgGrid &g, const double *xb,
                                const double *axb, double *xa, double *axa, bool keep_trans);
cudaError_t lg_launch_core_mixed(letkf_ctx *ctx, const LgGrid &g, const double *xb,
                                 const double *axb, double *xa, double *axa, bool keep_trans);
// the mixed core for k = 96, 128 (letkf_mixed_wide.cu) and the work queue
// both mixed kernels take (letkf_mixed.cu)
cudaError_t lg_launch_core_mixed_wide(letkf_ctx *ctx, const LgGrid &g, const double *xb, const double *axb,
                                      double *xa, double *axa, double *trans_out, double *w_out);
cudaError_t lg_build_chunk_queue(letkf_ctx *ctx, int &chunk, int &nchunks);
int lg_run_chunk(const letkf_ctx *ctx);
cudaError_t lg_launch_core_batch_fp64(letkf_ctx *ctx, int64_t nb, const int64_t *d_off,
                                      const double *d_hx, const float *d_rdi,
                                      const double *d_dep, const double *d_rloc,
                                      double *d_trans, double *d_w);

LgGrid lg_grid(letkf_ctx *ctx);
LgParams lg_params(letkf_ctx *ctx);
