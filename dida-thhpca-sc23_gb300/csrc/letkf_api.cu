// letkf_api.cu -- C-ABI host side of the GB300 LETKF analysis.
//
// The reference runs letkf_run (code/x86/TradDA/DA/LETKF/src/letkf.F90:157-257)
// once per DA cycle: gen_obs_struct, the MPI obs halo exchange, then the column
// loop.  Here one call does H, the bucket grid, the local search and the fused
// core + update on one GPU; the halo exchange has no counterpart because all
// observations live in one device array.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "letkf_internal.cuh"

bool lg_core_supports(int k);
bool lg_mixed_supports(int k);
int lg_search_cap(int max_obs);

cudaError_t lg_issue_copy(const LgCopyJob &j)
{
    cudaError_t e = cudaSuccess;
    if (j.after) e = cudaStreamWaitEvent(j.stream, j.after, 0);
    for (const LgCopyJob::Part &p : j.part) {
        if (e != cudaSuccess || !p.width || !p.height) continue;
        e = p.height == 1 ? cudaMemcpyAsync(p.dst, p.src, p.width, j.kind, j.stream)
                          : cudaMemcpy2DAsync(p.dst, p.dpitch, p.src, p.spitch, p.width, p.height, j.kind, j.stream);
    }
    if (e == cudaSuccess && j.done) e = cudaEventRecord(j.done, j.stream);
    return e;
}

LgCopyAgent::LgCopyAgent(int device) : device_(device) { thread_ = std::thread(&LgCopyAgent::loop, this); }

LgCopyAgent::~LgCopyAgent()
{
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    work_.notify_all();
    thread_.join();
}

uint64_t LgCopyAgent::push(const LgCopyJob &job)
{
    uint64_t seq;
    {
        std::lock_guard<std::mutex> lk(mu_);
        queue_.push_back(job);
        seq = ++pushed_;
    }
    work_.notify_one();
    return seq;
}

void LgCopyAgent::wait_issued(uint64_t seq)
{
    std::unique_lock<std::mutex> lk(mu_);
    idle_.wait(lk, [&] { return issued_ >= seq; });
}

cudaError_t LgCopyAgent::drain()
{
    std::unique_lock<std::mutex> lk(mu_);
    idle_.wait(lk, [this] { return issued_ == pushed_; });
    const cudaError_t e = err_;
    err_ = cudaSuccess;
    return e;
}

void LgCopyAgent::loop()
{
    const cudaError_t dev = cudaSetDevice(device_);
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        work_.wait(lk, [this] { return stop_ || !queue_.empty(); });
        if (queue_.empty()) return;
        const LgCopyJob j = queue_.front();
        queue_.pop_front();
        lk.unlock();
        // after a failed job the rest of the run's jobs are dropped: the run
        // reports the error, and its outputs are not meaningful
        cudaError_t e = dev;
        if (e == cudaSuccess) {
            lk.lock();
            const bool failed = err_ != cudaSuccess;
            lk.unlock();
            if (!failed) e = lg_issue_copy(j);
        }
        lk.lock();
        issued_++;
        if (e != cudaSuccess && err_ == cudaSuccess) err_ = e;
        idle_.notify_all();
    }
}

namespace {

std::atomic<int64_t> g_launches{0};

int set_err(letkf_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->last_error = msg;
    return code;
}

#define LG_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return set_err(ctx, e_ == cudaErrorMemoryAllocation ? LETKF_ERR_ALLOC : LETKF_ERR_CUDA, \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

template <typename T>
cudaError_t h2d(DevBuf<T> &buf, const T *src, size_t count, cudaStream_t s)
{
    cudaError_t e = buf.reserve(count);
    if (e != cudaSuccess || count == 0) return e;
    return cudaMemcpyAsync(buf.p, src, sizeof(T) * count, cudaMemcpyHostToDevice, s);
}

// The copy streams and their events (created on first use).
cudaError_t copy_streams(letkf_ctx *ctx)
{
    for (int i = 0; i < letkf_ctx::kCopyStreams; i++) {
        if (ctx->cstream[i]) continue;
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->cstream[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->cev[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->sev[i], cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    for (int i = 0; i < letkf_ctx::kPieces; i++) {
        if (ctx->pev[i]) continue;
        cudaError_t e = cudaEventCreateWithFlags(&ctx->pev[i], cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// True where p is ordinary pageable host memory (neither page-locked nor
// registered with the runtime, nor device or managed memory).
bool pageable(const void *p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

// A copy job of this run: issued here, or by the copy agent when a host
// buffer is pageable.  `after` is an event the caller records on the main
// stream next (copy_event hands out one per agent job, since the agent may
// issue the wait after the main stream's next record of a shared event).
cudaError_t copy_job(letkf_ctx *ctx, const LgCopyJob &j, uint64_t *seq = nullptr)
{
    if (seq) *seq = 0;
    if (!ctx->agent_on) return lg_issue_copy(j);
    const uint64_t q = ctx->agent->push(j);
    if (seq) *seq = q;
    return cudaSuccess;
}

cudaError_t copy_event(letkf_ctx *ctx, int stream, cudaEvent_t &ev)
{
    if (!ctx->agent_on) {
        ev = ctx->sev[stream];
        return cudaSuccess;
    }
    if (ctx->agent_ev_next == ctx->agent_ev.size()) {
        cudaEvent_t e = nullptr;
        cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        if (r != cudaSuccess) return r;
        ctx->agent_ev.push_back(e);
    }
    ev = ctx->agent_ev[ctx->agent_ev_next++];
    return cudaSuccess;
}

// The copies of columns [c0, c1) of an array of `per` doubles per column
// between the device (columns contiguous) and the host array in the run's
// layout (ctx->host_ld, host_off): one copy without a halo, else the partial
// longitude lines at either end as plain copies and the whole lines between
// as one strided copy.
void column_parts(const letkf_ctx *ctx, std::vector<LgCopyJob::Part> &out, bool to_host, const void *host,
                  const void *dev, size_t per, int64_t c0, int64_t c1)
{
    const int64_t nlat = ctx->nlat, ld = ctx->host_ld, off = ctx->host_off;
    const size_t cb = per * sizeof(double);
    auto hp = [&](int64_t c) { return (char *)host + (size_t)(off + c % nlat + ld * (c / nlat)) * cb; };
    auto dp = [&](int64_t c) { return (char *)dev + (size_t)c * cb; };
    auto add = [&](int64_t c, size_t width, size_t lines) {
        LgCopyJob::Part p;
        p.width = width;
        p.height = lines;
        p.dst = to_host ? hp(c) : dp(c);
        p.src = to_host ? (const void *)dp(c) : (const void *)hp(c);
        p.dpitch = to_host ? (size_t)ld * cb : (size_t)nlat * cb;
        p.spitch = to_host ? (size_t)nlat * cb : (size_t)ld * cb;
        out.push_back(p);
    };
    if (ld == nlat && off == 0) {
        if (c1 > c0) add(c0, (size_t)(c1 - c0) * cb, 1);
        return;
    }
    // strided copies take pitches below 2^31 bytes; wider lines go one by one
    const bool strided = (size_t)ld * cb < ((size_t)1 << 31);
    for (int64_t c = c0; c < c1;) {
        const int64_t line_end = (c / nlat + 1) * nlat;
        if (c % nlat != 0 || c1 < line_end || !strided) {
            const int64_t e = std::min(c1, line_end);
            add(c, (size_t)(e - c) * cb, 1);
            c = e;
        } else {
            const int64_t lines = (c1 - c) / nlat;
            add(c, (size_t)nlat * cb, (size_t)lines);
            c += lines * nlat;
        }
    }
}

// The state in for a run with host buffers: kPieces equal column ranges of
// the members and the mean, in column order, dealt in turn to the copy
// streams; each piece's stream records its event pev[i] when it is in.  The
// launches that read the state wait for the pieces they need (lg_state_wait).
cudaError_t state_in(letkf_ctx *ctx, const double *xb, const double *axb, cudaEvent_t after = nullptr)
{
    const size_t per_s = (size_t)ctx->n * ctx->k, per_m = (size_t)ctx->n;
    cudaError_t e = ctx->d_xb.reserve((size_t)ctx->ncol * per_s);
    if (e == cudaSuccess) e = ctx->d_axb.reserve((size_t)ctx->ncol * per_m);
    constexpr int NS = letkf_ctx::kCopyStreams, P = letkf_ctx::kPieces;
    // the pieces start after the main stream's work so far, or after `after`
    cudaEvent_t start = after;
    if (!start && e == cudaSuccess) e = copy_event(ctx, 0, start);
    if (!after && e == cudaSuccess) e = cudaEventRecord(start, ctx->stream);
    const int64_t part = (ctx->ncol + P - 1) / P;
    ctx->npieces = 0;
    for (int i = 0; i < P && e == cudaSuccess; i++) {
        const int64_t a = std::min<int64_t>(ctx->ncol, i * part), b = std::min<int64_t>(ctx->ncol, a + part);
        if (b <= a) break;
        LgCopyJob j;
        j.stream = ctx->cstream[i % NS];
        j.after = i < NS ? start : nullptr;
        j.done = ctx->pev[i];
        j.kind = cudaMemcpyHostToDevice;
        column_parts(ctx, j.part, false, xb, ctx->d_xb.p, per_s, a, b);
        column_parts(ctx, j.part, false, axb, ctx->d_axb.p, per_m, a, b);
        ctx->piece_c0[i] = a;
        ctx->piece_c1[i] = b;
        ctx->piece_waited[i] = false;
        e = copy_job(ctx, j, &ctx->piece_seq[i]);
        if (e == cudaSuccess) ctx->npieces = i + 1;
    }
    return e;
}

// A device address of host array p for the kernels (mapped page-locked
// memory, or pageable memory on a device that uses the host's page tables);
// null where the device cannot read it.
const void *host_view(letkf_ctx *ctx, const void *p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    if (a.type != cudaMemoryTypeUnregistered) return nullptr;
    int pma = 0;
    if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, ctx->device) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return pma ? p : nullptr;
}

// Wait for the copy agent's jobs (none without a pageable buffer).
cudaError_t drain_copies(letkf_ctx *ctx) { return ctx->agent_on ? ctx->agent->drain() : cudaSuccess; }

float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return 0.f;
    return ms;
}

int check_obs(letkf_ctx *ctx, const letkf_obs *obs)
{
    if (!obs) return set_err(ctx, LETKF_ERR_INVALID, "obs is NULL");
    if (obs->nobs < 0 || obs->nobs >= (int64_t)INT32_MAX)
        return set_err(ctx, LETKF_ERR_INVALID, "nobs out of range");
    if (obs->nobs == 0) return LETKF_OK;
    if (!obs->lat || !obs->lon || !obs->var || !obs->yo || !obs->rinv)
        return set_err(ctx, LETKF_ERR_INVALID, "obs lat/lon/var/yo/rinv must be set");
    const bool need_ph = ctx->params.h_mode == 0 || ctx->params.vert_dist > 0.0;
    if (need_ph && !obs->ph) return set_err(ctx, LETKF_ERR_INVALID, "obs ph required");
    if (ctx->params.h_mode == 1 && ctx->nvar3d > 0 && !obs->lev)
        return set_err(ctx, LETKF_ERR_INVALID, "obs lev required for level select");
    return LETKF_OK;
}

// Stage observation arrays on the device (copies for host pointers).
struct ObsDev {
    const double *lat, *lon, *ph, *yo, *rinv;
    const int32_t *lev, *var;
};

int stage_obs(letkf_ctx *ctx, const letkf_obs *obs, bool host, ObsDev &d)
{
    const int64_t no = obs->nobs;
    if (host) {
        LG_CUDA(h2d(ctx->d_olat, obs->lat, no, ctx->stream));
        LG_CUDA(h2d(ctx->d_olon, obs->lon, no, ctx->stream));
        LG_CUDA(h2d(ctx->d_oyo, obs->yo, no, ctx->stream));
        LG_CUDA(h2d(ctx->d_orinv, obs->rinv, no, ctx->stream));
        LG_CUDA(h2d(ctx->d_ovar, obs->var, no, ctx->stream));
        if (obs->ph) LG_CUDA(h2d(ctx->d_oph, obs->ph, no, ctx->stream));
        else LG_CUDA(ctx->d_oph.reserve(1));
        if (obs->lev) LG_CUDA(h2d(ctx->d_olev, obs->lev, no, ctx->stream));
        else LG_CUDA(ctx->d_olev.reserve(1));
        d = {ctx->d_olat.p, ctx->d_olon.p, ctx->d_oph.p, ctx->d_oyo.p, ctx->d_orinv.p,
             ctx->d_olev.p, ctx->d_ovar.p};
    } else {
        LG_CUDA(ctx->d_oph.reserve(1));
        LG_CUDA(ctx->d_olev.reserve(1));
        d = {obs->lat, obs->lon, obs->ph ? obs->ph : ctx->d_oph.p, obs->yo, obs->rinv,
             obs->lev ? obs->lev : ctx->d_olev.p, obs->var};
    }
    return LETKF_OK;
}

int reserve_obs_work(letkf_ctx *ctx, int64_t no)
{
    const size_t n = (size_t)std::max<int64_t>(no, 1);
    LG_CUDA(ctx->d_yb.reserve(n * ctx->k));
    if (lg_is_mixed(ctx->params.precision)) {
        LG_CUDA(ctx->d_ys32.reserve((n > 0 ? n : 1) * ctx->k));
        LG_CUDA(ctx->d_oef.reserve(n));
    }
    LG_CUDA(ctx->d_dep.reserve(n));
    LG_CUDA(ctx->d_rinvf.reserve(n));
    LG_CUDA(ctx->d_os.reserve(n));
    LG_CUDA(ctx->d_oc.reserve(n));
    LG_CUDA(ctx->d_oyr.reserve(n));
    LG_CUDA(ctx->d_oxyz.reserve(n));
    LG_CUDA(ctx->d_obucket.reserve(n));
    LG_CUDA(ctx->d_bidx.reserve(n));
    LG_CUDA(ctx->d_bxyz.reserve(n));
    return LETKF_OK;
}

int read_status(letkf_ctx *ctx, unsigned &status, unsigned long long *cnt)
{
    LG_CUDA(cudaMemcpyAsync(&status, ctx->d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            ctx->stream));
    LG_CUDA(cudaMemcpyAsync(cnt, ctx->d_counters.p, sizeof(unsigned long long) * LG_CNT_N,
                            cudaMemcpyDeviceToHost, ctx->stream));
    LG_CUDA(cudaStreamSynchronize(ctx->stream));
    return LETKF_OK;
}

int reset_status(letkf_ctx *ctx)
{
    LG_CUDA(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
    LG_CUDA(cudaMemsetAsync(ctx->d_counters.p, 0, sizeof(unsigned long long) * LG_CNT_N, ctx->stream));
    return LETKF_OK;
}

// H and the observation buckets for the staged observations.
// H, the buckets and the per-observation terms of the search.  With
// defer_members the state is still being copied in: only the geometry pass
// runs now, and the members pass waits for the copy in lg_members_if_pending.
int obs_prepare(letkf_ctx *ctx, const double *xb, const double *axb, const ObsDev &od, int64_t no,
                bool defer_members = false)
{
    const LgGrid g = lg_grid(ctx);
    int rc = reserve_obs_work(ctx, no);
    if (rc) return rc;
    LG_CUDA(lg_launch_obs_prepare(ctx, g, xb, axb, no, od.lat, od.lon, od.ph, od.lev, od.var, od.yo,
                                  od.rinv, defer_members ? 1 : 0));
    if (defer_members) {
        ctx->members_pending = true;
        ctx->pend_xb = xb;
        ctx->pend_axb = axb;
        ctx->pend_lat = od.lat;
        ctx->pend_lon = od.lon;
        ctx->pend_ph = od.ph;
        ctx->pend_lev = od.lev;
        ctx->pend_var = od.var;
        ctx->pend_yo = od.yo;
        ctx->pend_rinv = od.rinv;
        ctx->pend_no = no;
    }
    LG_CUDA(lg_launch_buckets(ctx, no));
    if (ctx->dec_nx > 0) LG_CUDA(lg_launch_block_members(ctx, no, od.lat, od.lon));
    if (ctx->params.overlap == 0 && ctx->params.vert_dist > 0.0) {
        LG_CUDA(ctx->d_olnp.reserve((size_t)std::max<int64_t>(no, 1)));
        LG_CUDA(lg_launch_obs_lnp(ctx, no, od.ph));
    }
    return LETKF_OK;
}

size_t list_entry_bytes(const letkf_ctx *ctx)
{
    return sizeof(int32_t) + sizeof(double) + (lg_is_mixed(ctx->params.precision) ? sizeof(float2) : 0);
}

// Entries the list pool may hold: the caller's limit, else the device's free
// memory plus the pool's own, less 1 GiB for the rest of the run.
int64_t pool_limit(letkf_ctx *ctx)
{
    if (ctx->list_limit > 0) return ctx->list_limit;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return std::max<int64_t>(ctx->list_cap, 1);
    const size_t held = ctx->d_lidx.n * sizeof(int32_t) + ctx->d_lrloc.n * sizeof(double) +
                        ctx->d_lmeta.n * sizeof(float2);
    const size_t keep = (size_t)1 << 30;
    const size_t avail = fr + held > keep ? fr + held - keep : 0;
    return std::max<int64_t>((int64_t)(avail / list_entry_bytes(ctx)), 1);
}

void release_pool(letkf_ctx *ctx)
{
    ctx->d_lidx.release();
    ctx->d_lrloc.release();
    ctx->d_lmeta.release();
    ctx->list_cap = 0;
}

// A list pool of at least cap entries (a larger one that is held is kept).
int size_pool(letkf_ctx *ctx, int64_t cap)
{
    if (cap <= ctx->list_cap && ctx->d_lidx.p) return LETKF_OK;
    release_pool(ctx);
    LG_CUDA(ctx->d_lidx.reserve((size_t)cap));
    LG_CUDA(ctx->d_lrloc.reserve((size_t)cap));
    if (lg_is_mixed(ctx->params.precision)) LG_CUDA(ctx->d_lmeta.reserve((size_t)cap));
    ctx->list_cap = cap;
    return LETKF_OK;
}

cudaError_t launch_search(letkf_ctx *ctx, const ObsDev &od, int64_t no)
{
    const LgGrid g = lg_grid(ctx);
    // before the departures (H's members pass deferred) the entries get
    // their second factor at the core launch
    ctx->lists_need_ef = ctx->members_pending && lg_is_mixed(ctx->params.precision);
    return ctx->dec_nx > 0 ? lg_launch_search_dec(ctx, g, od.lat) : lg_launch_search(ctx, g, no);
}

cudaError_t launch_core(letkf_ctx *ctx, const double *xb, const double *axb, double *xa, double *axa)
{
    cudaError_t e = lg_members_if_pending(ctx);
    if (e != cudaSuccess) return e;
    if (ctx->lists_need_ef && (e = lg_launch_list_efactor(ctx)) != cudaSuccess) return e;
    // the cores read the state: its copy first (the staged k = 64 core waits
    // before each block's update for the block's columns)
    const bool staged = lg_is_mixed(ctx->params.precision) && ctx->k == 64 && ctx->params.overlap == 0;
    if (!staged && (e = lg_state_wait(ctx, 0, ctx->ncol)) != cudaSuccess) return e;
    const LgGrid g = lg_grid(ctx);
    // overlapped cubes: each cube's trans now, the columns' averages after
    // the last window (lg_launch_overlap_update)
    if (ctx->params.overlap > 0) return lg_launch_core_fp64(ctx, g, nullptr, nullptr, nullptr, nullptr, true);
    const bool keep = ctx->d_trans.p != nullptr;
    return lg_is_mixed(ctx->params.precision) ? lg_launch_core_mixed(ctx, g, xb, axb, xa, axa, keep)
                                                     : lg_launch_core_fp64(ctx, g, xb, axb, xa, axa, keep);
}

// Zero the list cursor and the work-queue cursor (the counters that restart
// with every window; the others sum over the windows).
int restart_cursors(letkf_ctx *ctx)
{
    LG_CUDA(cudaMemsetAsync(ctx->d_counters.p + LG_CNT_CURSOR, 0, sizeof(unsigned long long), ctx->stream));
    LG_CUDA(cudaMemsetAsync(ctx->d_counters.p + LG_CNT_QUEUE, 0, sizeof(unsigned long long), ctx->stream));
    return LETKF_OK;
}

// The list length of every cube of the run's range from the last search.
int read_need(letkf_ctx *ctx, std::vector<int32_t> &need)
{
    need.resize((size_t)(ctx->range1 - ctx->range0));
    LG_CUDA(cudaMemcpyAsync(need.data(), ctx->d_lneed.p + ctx->range0, sizeof(int32_t) * need.size(),
                            cudaMemcpyDeviceToHost, ctx->stream));
    LG_CUDA(cudaStreamSynchronize(ctx->stream));
    return LETKF_OK;
}

// Local lists and the analysis of cubes range0 .. range1-1.  One search over
// the range gives every cube's list length; when the lists fit the pool (grown
// up to the limit if needed) one core launch follows, else the range is cut
// into consecutive windows whose lists fit and each window is searched again
// and analysed.  ev[3] is recorded after the first search (or count).
int search_and_core(letkf_ctx *ctx, const double *xb, const double *axb, double *xa, double *axa,
                    const ObsDev &od, int64_t no, unsigned long long *cnt)
{
    const int64_t c0 = ctx->range0, c1 = ctx->range1;
    int rc = LETKF_OK;
    // a pool from before a smaller limit was set is given back
    if (ctx->list_limit > 0 && ctx->list_cap > ctx->list_limit) release_pool(ctx);
    const int64_t limit = pool_limit(ctx);
    if (ctx->list_cap == 0) {
        const int64_t guess = (c1 - c0) * (int64_t)std::min(ctx->params.max_obs, 512);
        rc = size_pool(ctx, std::max<int64_t>(std::min(guess, limit), 1));
        if (rc) return rc;
    }
    ctx->lists_whole = false;
    ctx->win0 = c0;
    ctx->win1 = c1;
    // a run after one that needed windows counts first: one pass that only
    // counts gives every list length, so no full search fills a pool that is
    // too small
    const bool count_first = ctx->last_windows > 1;
    std::vector<int32_t> need;
    bool fits = false;
    for (int attempt = 0; attempt < 2; attempt++) {
        ctx->count_pass = count_first && attempt == 0;
        const cudaError_t e = launch_search(ctx, od, no);
        const bool counted = ctx->count_pass;
        ctx->count_pass = false;
        LG_CUDA(e);
        unsigned st = 0;
        rc = read_status(ctx, st, cnt);
        if (rc) return rc;
        if (st & LG_ST_SEGMENTS)
            return set_err(ctx, LETKF_ERR_UNSUPPORTED, "localization cap spans too many buckets");
        if (st & LG_ST_BAD_OBS)
            return set_err(ctx, LETKF_ERR_INVALID,
                           "observation outside the grid or with a bad variable/level/pressure");
        fits = !counted && !(st & LG_ST_LIST_FULL);
        if (fits) break;
        // every cube's length is known now: restart the counters and either
        // grow the pool to hold all lists or go through windows
        rc = reset_status(ctx);
        if (rc) return rc;
        int64_t total = (int64_t)cnt[LG_CNT_CURSOR];
        if (counted) {
            rc = read_need(ctx, need);
            if (rc) return rc;
            total = 0;
            for (int32_t v : need) total += v;
        }
        if (attempt > 0 || total > limit) break;
        rc = size_pool(ctx, std::min(limit, total + total / 16 + 1024));
        if (rc) return rc;
        need.clear();
    }
    LG_CUDA(cudaEventRecord(ctx->ev[3], ctx->stream));
    if (fits) {
        LG_CUDA(launch_core(ctx, xb, axb, xa, axa));
        ctx->last_windows = 1;
        ctx->lists_whole = c0 == 0 && c1 == ctx->ncubes;
        return LETKF_OK;
    }
    if (need.empty()) {
        rc = read_need(ctx, need);
        if (rc) return rc;
    }
    // windows end on multiples of the mixed core's chunk size (so that every
    // cube keeps its chunk); the pool holds at least the heaviest chunk
    const int64_t align = lg_is_mixed(ctx->params.precision) ? lg_run_chunk(ctx) : 1;
    std::vector<int64_t> unit;   // list entries of each aligned group of cubes
    for (int64_t c = c0; c < c1;) {
        const int64_t e = std::min(c1, (c / align + 1) * align);
        int64_t s = 0;
        for (int64_t i = c; i < e; i++) s += need[(size_t)(i - c0)];
        unit.push_back(s);
        c = e;
    }
    int64_t heaviest = 1;
    for (int64_t s : unit) heaviest = std::max(heaviest, s);
    rc = size_pool(ctx, std::max(limit, heaviest));
    if (rc) return rc;
    std::vector<int64_t> bounds{c0};
    int64_t acc = 0, at = c0;
    for (int64_t s : unit) {
        if (acc + s > ctx->list_cap) {
            bounds.push_back(at);
            acc = 0;
        }
        acc += s;
        at = std::min(c1, (at / align + 1) * align);
    }
    bounds.push_back(c1);
    for (size_t w = 0; w + 1 < bounds.size(); w++) {
        rc = restart_cursors(ctx);
        if (rc) return rc;
        ctx->win0 = bounds[w];
        ctx->win1 = bounds[w + 1];
        LG_CUDA(launch_search(ctx, od, no));
        LG_CUDA(launch_core(ctx, xb, axb, xa, axa));
    }
    ctx->win0 = c0;
    ctx->win1 = c1;
    ctx->last_windows = (int)(bounds.size() - 1);
    return LETKF_OK;
}

// The whole analysis on device pointers with no host synchronization, for
// capture into a CUDA graph.  Every buffer must already be sized for these
// inputs by an earlier run (the list pool cannot grow here: a list pool that
// is too small shows as LETKF_ERR_ALLOC when the status is read).
int enqueue_run(letkf_ctx *ctx, const double *xb, const double *axb, const letkf_obs *obs, double *xa,
                double *axa)
{
    if (ctx->dec_nx > 0)
        return set_err(ctx, LETKF_ERR_UNSUPPORTED, "decomposed observation sets are not captured in graphs");
    if (ctx->params.overlap > 0 || ctx->params.vert_dist > 0.0)
        return set_err(ctx, LETKF_ERR_UNSUPPORTED, "overlapped cubes and vertical localization are not captured in graphs");
    int rc = reset_status(ctx);
    if (rc) return rc;
    ObsDev od;
    rc = stage_obs(ctx, obs, false, od);
    if (rc) return rc;
    const int64_t no = obs->nobs;
    rc = obs_prepare(ctx, xb, axb, od, no);
    if (rc) return rc;
    ctx->win0 = ctx->range0;
    ctx->win1 = ctx->range1;
    LG_CUDA(launch_search(ctx, od, no));
    LG_CUDA(launch_core(ctx, xb, axb, xa, axa));
    return LETKF_OK;
}

void fill_stats(letkf_ctx *ctx, const unsigned long long *cnt)
{
    letkf_stats &s = ctx->stats;
    s.ncubes = ctx->range1 - ctx->range0;
    s.sum_p = (int64_t)cnt[LG_CNT_SUMP];
    s.max_p = (int64_t)cnt[LG_CNT_MAXP];
    s.n_truncated = (int64_t)cnt[LG_CNT_TRUNC];
    s.n_borderline = (int64_t)cnt[LG_CNT_BORDER];
    s.n_not_converged = (int64_t)cnt[LG_CNT_NOTCONV];
    s.max_sweeps = (int32_t)cnt[LG_CNT_MAXSWEEP];
    s.sum_sweeps = (int64_t)cnt[LG_CNT_SUMSWEEP];
    s.n_ill_conditioned = (int64_t)cnt[LG_CNT_ILLCOND];
    s.sched_chunk = ctx->sched_chunk;
    s.n_windows = ctx->last_windows;
    s.precision = ctx->params.precision;
}

}  // namespace

void lg_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void lg_stage_mark(letkf_ctx *ctx, int s, bool end)
{
    if (s < 0 || s >= letkf_ctx::kStages) return;
    const int i = ctx->stg_n[s];
    if (i >= letkf_ctx::kStageMarks) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    cudaEvent_t &e = ctx->stg_ev[s][end ? 1 : 0][i];
    if (!e && cudaEventCreate(&e) != cudaSuccess) {
        e = nullptr;
        return;
    }
    if (cudaEventRecord(e, ctx->stream) != cudaSuccess) return;
    if (end) ctx->stg_n[s] = i + 1;
}

LgGrid lg_grid(letkf_ctx *ctx)
{
    LgGrid g;
    g.nlat = ctx->nlat;
    g.nlon = ctx->nlon;
    g.nz = ctx->nz;
    g.nvar2d = ctx->nvar2d;
    g.nvar3d = ctx->nvar3d;
    g.k = ctx->k;
    g.n = ctx->n;
    g.ps_row = ctx->ps_row;
    g.p0 = ctx->p0;
    g.ptop = ctx->ptop;
    g.glat = ctx->d_glat.p;
    g.glon = ctx->d_glon.p;
    g.hyai = ctx->d_hyai.p;
    g.hybi = ctx->d_hybi.p;
    return g;
}

LgParams lg_params(letkf_ctx *ctx)
{
    LgParams p;
    const letkf_params &q = ctx->params;
    p.local_dist = q.loc_dist_km;
    p.vert_dist = q.vert_dist;
    p.inflation = q.inflation;
    p.obs_polar = q.obs_polar_deg;
    p.gc_filter = q.gc_filter;
    p.gc_filter_vertical = q.gc_filter_vertical;
    p.max_obs = q.max_obs;
    p.cube_n = q.cube_n;
    p.cube_nz = q.cube_nz;
    p.overlap = q.overlap;
    p.h_mode = q.h_mode;
    p.precision = q.precision;
    p.nbj = ctx->nbj;
    p.nbi = ctx->nbi;
    p.cube_step = q.cube_n - q.overlap;
    p.cube0 = ctx->win0;
    p.count_only = ctx->count_pass ? 1 : 0;
    p.spin_limit = ctx->wait_limit < 0 ? LG_MBAR_SPIN_LIMIT
                   : (uint32_t)(ctx->wait_limit < (int64_t)LG_MBAR_SPIN_LIMIT ? ctx->wait_limit
                                                                              : (int64_t)LG_MBAR_SPIN_LIMIT);
    p.members = ctx->members_on ? 1 : 0;
    p.gamma1 = ctx->members_g1;
    p.gamma2 = ctx->members_g2;
    p.polar = ctx->members_polar;
    p.spb = ctx->members_spb;
    p.spa = ctx->members_spa;
    return p;
}

extern "C" {

int64_t letkf_gpu_launch_count(void) { return g_launches.load(); }

int letkf_decomp_dims(int nranks, int *lat_blocks, int *lon_blocks)
{
    if (!lat_blocks || !lon_blocks) return LETKF_ERR_INVALID;
    int a = 0, b = 0;
    if (lg_decomp_dims(nranks, a, b) != 0) return LETKF_ERR_INVALID;
    *lat_blocks = a;
    *lon_blocks = b;
    return LETKF_OK;
}

int letkf_gpu_create(letkf_ctx **out, const letkf_grid *grid, const letkf_params *params, int device)
{
    letkf_ctx *ctx = nullptr;
    if (!out || !grid || !params) return LETKF_ERR_INVALID;
    *out = nullptr;
    const letkf_grid &G = *grid;
    const letkf_params &P = *params;
    if (G.nlat < 2 || G.nlon < 2 || G.nz < 1 || G.nvar2d < 0 || G.nvar3d < 0 ||
        G.nvar2d + G.nvar3d < 1 || !G.lat || !G.lon)
        return LETKF_ERR_INVALID;
    if (!lg_core_supports(G.ens)) return LETKF_ERR_UNSUPPORTED;
    for (int i = 0; i < G.nlat; i++)
        if (!(G.lat[i] > -90.0f && G.lat[i] < 90.0f) || (i > 0 && !(G.lat[i] > G.lat[i - 1])))
            return LETKF_ERR_INVALID;
    for (int i = 0; i < G.nlon; i++)
        if (!(G.lon[i] >= 0.0f && G.lon[i] < 360.0f) || (i > 0 && !(G.lon[i] > G.lon[i - 1])))
            return LETKF_ERR_INVALID;
    const int n = G.nvar2d + G.nvar3d * G.nz;
    if (!(P.loc_dist_km > 0.0 && P.loc_dist_km <= 4000.0) || !(P.inflation > 0.0) ||
        P.max_obs < 1 || P.cube_n < 1 || P.cube_nz < 1 || P.overlap < 0 ||
        P.overlap >= P.cube_n || (P.h_mode != 0 && P.h_mode != 1) ||
        (P.precision != LETKF_PREC_FP64 && !lg_is_mixed(P.precision)) ||
        !(P.obs_polar_deg >= 0.0))
        return LETKF_ERR_INVALID;
    const bool need_hybrid = P.h_mode == 0 || P.vert_dist > 0.0;
    if (need_hybrid && (!G.hyai || !G.hybi || G.ps_row < 0 || G.ps_row >= n))
        return LETKF_ERR_INVALID;
    const bool decomposed = P.decomp_lat_blocks != 0 || P.decomp_lon_blocks != 0;
    if (decomposed && (P.decomp_lat_blocks < 1 || P.decomp_lon_blocks < 1 || P.decomp_lat_blocks > G.nlat ||
                       P.decomp_lon_blocks > G.nlon ||
                       (int64_t)P.decomp_lat_blocks * P.decomp_lon_blocks > 65535))
        return LETKF_ERR_INVALID;
    if (decomposed && P.cube_n != 1) return LETKF_ERR_UNSUPPORTED;
    // the overlapped-cube and vertical-localization modes run in the FP64 form
    if ((P.overlap != 0 || P.vert_dist > 0.0) && P.precision != LETKF_PREC_FP64) return LETKF_ERR_UNSUPPORTED;
    if (P.precision == LETKF_PREC_MIXED && !lg_mixed_supports(G.ens)) return LETKF_ERR_UNSUPPORTED;
    // the FP64 eigenpair refinement is a stage of the staged (k = 64) core
    if (P.precision == LETKF_PREC_MIXED_F64EIG && G.ens != 64) return LETKF_ERR_UNSUPPORTED;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return LETKF_ERR_CUDA;
    if (device >= ndev) return LETKF_ERR_INVALID;
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return LETKF_ERR_CUDA;

    ctx = new letkf_ctx();
    cudaGetDevice(&ctx->device);
    ctx->params = P;
    ctx->nlat = G.nlat;
    ctx->nlon = G.nlon;
    ctx->nz = G.nz;
    ctx->nvar2d = G.nvar2d;
    ctx->nvar3d = G.nvar3d;
    ctx->k = G.ens;
    ctx->n = n;
    ctx->ps_row = G.ps_row;
    ctx->p0 = G.p0;
    ctx->ptop = G.ptop;
    ctx->ncol = (int64_t)G.nlat * G.nlon;
    // cubes start every cube_n - overlap points (letkf_compute.F90:150-160)
    const int step = P.cube_n - P.overlap;
    ctx->nbj = (G.nlat + step - 1) / step;
    ctx->nbi = (G.nlon + step - 1) / step;
    ctx->ncubes = (int64_t)ctx->nbj * ctx->nbi;
    ctx->range0 = ctx->win0 = 0;
    ctx->range1 = ctx->win1 = ctx->ncubes;
    ctx->have_hybrid = G.hyai && G.hybi;

    int rc = LETKF_OK;
    auto setup = [&]() -> int {
        LG_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
        ctx->stream = ctx->own_stream;
        for (int i = 0; i < 8; i++) LG_CUDA(cudaEventCreate(&ctx->ev[i]));
        std::vector<float> glat(G.lat, G.lat + G.nlat), glon(G.lon, G.lon + G.nlon);
        glat.push_back(90.0f);      // grid_lat(nx+1) = 90 (pro_info.F90:77,82)
        glon.push_back(360.0f);     // grid_lon(ny+1) = 360 (pro_info.F90:78,83)
        LG_CUDA(h2d(ctx->d_glat, glat.data(), glat.size(), ctx->stream));
        LG_CUDA(h2d(ctx->d_glon, glon.data(), glon.size(), ctx->stream));
        if (decomposed) LG_CUDA(lg_decomp_setup(ctx, glat, glon));
        LG_CUDA(lg_launch_geo_tables(ctx));
        std::vector<double> zero(G.nz + 1, 0.0);
        LG_CUDA(h2d(ctx->d_hyai, G.hyai ? G.hyai : zero.data(), (size_t)G.nz + 1, ctx->stream));
        LG_CUDA(h2d(ctx->d_hybi, G.hybi ? G.hybi : zero.data(), (size_t)G.nz + 1, ctx->stream));
        // bucket cells about a third of the cut-off radius 2c; the cell sizes
        // divide 180 and 360 degrees exactly so that cell index j + nblon is
        // longitude + 360 (the longitude ranges of a cap wrap around)
        const double radius_deg = 2.0 * P.loc_dist_km / LG_EARTH_A * 180.0 / M_PI;
        const double cell = std::min(10.0, std::max(0.25, radius_deg / 3.0));
        ctx->nblat = (int)std::ceil(180.0 / cell);
        ctx->nblon = (int)std::ceil(360.0 / cell);
        ctx->cell_lat = 180.0 / ctx->nblat;
        ctx->cell_lon = 360.0 / ctx->nblon;
        const size_t nb = (size_t)ctx->nblat * ctx->nblon;
        LG_CUDA(ctx->d_bcount.reserve(nb));
        LG_CUDA(ctx->d_bstart.reserve(nb + 1));
        LG_CUDA(ctx->d_loff.reserve((size_t)ctx->ncubes));
        LG_CUDA(ctx->d_lcnt.reserve((size_t)ctx->ncubes));
        LG_CUDA(ctx->d_lneed.reserve((size_t)ctx->ncubes));
        LG_CUDA(ctx->d_status.reserve(1));
        LG_CUDA(ctx->d_counters.reserve(LG_CNT_N));
        LG_CUDA(ctx->d_ymax.reserve(1));
        LG_CUDA(cudaMemsetAsync(ctx->d_ymax.p, 0, sizeof(unsigned), ctx->stream));
        LG_CUDA(cudaStreamSynchronize(ctx->stream));
        return LETKF_OK;
    };
    rc = setup();
    if (rc != LETKF_OK) {
        letkf_gpu_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return LETKF_OK;
}

int letkf_gpu_set_stream(letkf_ctx *ctx, void *stream)
{
    if (!ctx) return LETKF_ERR_INVALID;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return LETKF_OK;
}

int letkf_gpu_set_wait_limit(letkf_ctx *ctx, int64_t polls)
{
    if (!ctx) return LETKF_ERR_INVALID;
    ctx->wait_limit = polls < 0 ? -1 : polls;
    return LETKF_OK;
}

int letkf_gpu_set_keep_trans(letkf_ctx *ctx, int keep)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (keep && ctx->params.overlap == 0 && ctx->params.vert_dist > 0.0)
        return set_err(ctx, LETKF_ERR_UNSUPPORTED, "vertical localization solves one problem per level block");
    if (keep) {
        LG_CUDA(ctx->d_trans.reserve((size_t)ctx->ncubes * ctx->k * ctx->k));
        LG_CUDA(ctx->d_w.reserve((size_t)ctx->ncubes * ctx->k));
    } else {
        ctx->d_trans.release();
        ctx->d_w.release();
    }
    return LETKF_OK;
}

int letkf_gpu_set_list_limit(letkf_ctx *ctx, int64_t max_entries)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (max_entries < 0) return set_err(ctx, LETKF_ERR_INVALID, "negative list limit");
    ctx->list_limit = max_entries;
    return LETKF_OK;
}

int letkf_gpu_set_cube_range(letkf_ctx *ctx, int64_t first, int64_t count)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (count < 0) {
        ctx->range0 = 0;
        ctx->range1 = ctx->ncubes;
        return LETKF_OK;
    }
    if (first < 0 || count < 1 || first > ctx->ncubes - count)
        return set_err(ctx, LETKF_ERR_INVALID, "cube range outside the grid");
    if (ctx->params.cube_n > 1 && (first % ctx->nbj != 0 || count % ctx->nbj != 0))
        return set_err(ctx, LETKF_ERR_INVALID, "with cube_n > 1 the range must be whole longitude strips");
    ctx->range0 = first;
    ctx->range1 = first + count;
    return LETKF_OK;
}

}  // extern "C"

int lg_set_err(letkf_ctx *ctx, int code, const char *msg) { return set_err(ctx, code, msg); }

cudaError_t lg_members_if_pending(letkf_ctx *ctx)
{
    if (!ctx->members_pending) return cudaSuccess;
    ctx->members_pending = false;
    // H's rows: gathered from the host arrays, else the whole state copy
    cudaError_t e = ctx->gathered ? cudaStreamWaitEvent(ctx->stream, ctx->gev, 0) : lg_state_wait(ctx, 0, ctx->ncol);
    if (e != cudaSuccess) return e;
    return lg_launch_obs_prepare(ctx, lg_grid(ctx), ctx->pend_xb, ctx->pend_axb, ctx->pend_no, ctx->pend_lat,
                                 ctx->pend_lon, ctx->pend_ph, ctx->pend_lev, ctx->pend_var, ctx->pend_yo,
                                 ctx->pend_rinv, 2);
}

cudaError_t lg_state_wait(letkf_ctx *ctx, int64_t c0, int64_t c1)
{
    for (int i = 0; i < ctx->npieces; i++) {
        if (ctx->piece_waited[i] || ctx->piece_c1[i] <= c0 || ctx->piece_c0[i] >= c1) continue;
        // a piece of the copy thread: its event is recorded once the job is issued
        if (ctx->piece_seq[i]) ctx->agent->wait_issued(ctx->piece_seq[i]);
        const cudaError_t e = cudaStreamWaitEvent(ctx->stream, ctx->pev[i], 0);
        if (e != cudaSuccess) return e;
        ctx->piece_waited[i] = true;
    }
    return cudaSuccess;
}

cudaError_t lg_sink_columns(letkf_ctx *ctx, int64_t c0, int64_t c1)
{
    if (!ctx->sink_xa || c1 <= c0) return cudaSuccess;
    const int i = ctx->sink_next++ % letkf_ctx::kCopyStreams;
    LgCopyJob j;
    cudaError_t e = copy_event(ctx, i, j.after);
    if (e == cudaSuccess) e = cudaEventRecord(j.after, ctx->stream);
    const size_t per_s = (size_t)ctx->n * ctx->k, per_m = (size_t)ctx->n;
    j.stream = ctx->cstream[i];
    j.kind = cudaMemcpyDeviceToHost;
    column_parts(ctx, j.part, true, ctx->sink_xa, ctx->sink_dxa, per_s, c0, c1);
    column_parts(ctx, j.part, true, ctx->sink_axa, ctx->sink_daxa, per_m, c0, c1);
    if (e == cudaSuccess) e = copy_job(ctx, j);
    if (e == cudaSuccess) ctx->sink_cols += c1 - c0;
    return e;
}
int lg_reset_status(letkf_ctx *ctx) { return reset_status(ctx); }
int lg_read_status(letkf_ctx *ctx, unsigned &status, unsigned long long *cnt)
{
    return read_status(ctx, status, cnt);
}

int lg_check_run(letkf_ctx *ctx, const letkf_obs *obs)
{
    int rc = check_obs(ctx, obs);
    if (rc) return rc;
    if (ctx->params.overlap > 0 && (ctx->range0 != 0 || ctx->range1 != ctx->ncubes))
        return set_err(ctx, LETKF_ERR_UNSUPPORTED, "overlapped cubes average over neighbouring cubes: no cube range");
    return LETKF_OK;
}

int lg_run_analysis(letkf_ctx *ctx, const letkf_obs *obs, bool host_obs, const double *dxb,
                    const double *daxb, double *dxa, double *daxa, unsigned long long *cnt, bool state_in_flight)
{
    ObsDev od;
    for (int s = 0; s < letkf_ctx::kStages; s++) ctx->stg_n[s] = 0;
    int rc = stage_obs(ctx, obs, host_obs, od);
    if (rc) return rc;
    LG_CUDA(cudaEventRecord(ctx->ev[1], ctx->stream));
    ctx->gathered = false;
    if (ctx->copy_xb) {
        // The state copy, behind the observations (small copies that would
        // wait behind it on the copy engines).  Where the device can read the
        // host arrays, the rows H reads go first, by a kernel on the first
        // copy stream, and the bulk copy follows: H's members pass then waits
        // for those rows only, the geometry and the search run meanwhile.
        cudaEvent_t after = nullptr;
        if (ctx->gather_xb && dxb == ctx->d_xb.p && daxb == ctx->d_axb.p) {
            if (!ctx->gev) LG_CUDA(cudaEventCreateWithFlags(&ctx->gev, cudaEventDisableTiming));
            LG_CUDA(cudaEventRecord(ctx->sev[0], ctx->stream));
            LG_CUDA(cudaStreamWaitEvent(ctx->cstream[0], ctx->sev[0], 0));
            LG_CUDA(lg_launch_gather_rows(ctx, ctx->cstream[0], lg_grid(ctx), obs->nobs, od.lat, od.lon, od.ph,
                                          od.lev, od.var, ctx->gather_xb, ctx->gather_axb, ctx->d_xb.p,
                                          ctx->d_axb.p));
            LG_CUDA(cudaEventRecord(ctx->gev, ctx->cstream[0]));
            after = ctx->gev;
            ctx->gathered = true;
        }
        const cudaError_t e = state_in(ctx, ctx->copy_xb, ctx->copy_axb, after);
        ctx->copy_xb = ctx->copy_axb = nullptr;
        if (e != cudaSuccess) return set_err(ctx, LETKF_ERR_CUDA, cudaGetErrorString(e));
    }
    rc = obs_prepare(ctx, dxb, daxb, od, obs->nobs, state_in_flight);
    if (rc) return rc;
    LG_CUDA(cudaEventRecord(ctx->ev[2], ctx->stream));
    if (ctx->params.overlap > 0) {
        LG_CUDA(ctx->d_trans.reserve((size_t)ctx->ncubes * ctx->k * ctx->k));
        LG_CUDA(ctx->d_w.reserve((size_t)ctx->ncubes * ctx->k));
    }
    rc = search_and_core(ctx, dxb, daxb, dxa, daxa, od, obs->nobs, cnt);
    if (rc) return rc;
    if (ctx->params.overlap > 0) LG_CUDA(lg_launch_overlap_update(ctx, lg_grid(ctx), dxb, daxb, dxa, daxa));
    LG_CUDA(cudaEventRecord(ctx->ev[4], ctx->stream));
    return LETKF_OK;
}

int lg_finish_run(letkf_ctx *ctx, const letkf_obs *obs, unsigned long long *cnt)
{
    LG_CUDA(cudaEventRecord(ctx->ev[5], ctx->stream));
    unsigned st = 0;
    int rc = read_status(ctx, st, cnt);
    if (rc) return rc;
    if (st & LG_ST_LIST_FULL) return set_err(ctx, LETKF_ERR_ALLOC, "local observation lists did not fit");
    // a fused members run found a NaN background member
    if (st & LG_ST_BAD_STATE) return set_err(ctx, LETKF_ERR_INVALID, "a background member is NaN");
    fill_stats(ctx, cnt);
    ctx->stats.ms_h2d = elapsed(ctx->ev[0], ctx->ev[1]);
    ctx->stats.ms_obs = elapsed(ctx->ev[1], ctx->ev[2]);
    ctx->stats.ms_search = elapsed(ctx->ev[2], ctx->ev[3]);
    ctx->stats.ms_core = elapsed(ctx->ev[3], ctx->ev[4]);
    ctx->stats.ms_d2h = elapsed(ctx->ev[4], ctx->ev[5]);
    ctx->stats.ms_total = elapsed(ctx->ev[0], ctx->ev[5]);
    for (int s = 0; s < letkf_ctx::kStages; s++) {
        double t = 0.0;
        for (int i = 0; i < ctx->stg_n[s]; i++) t += elapsed(ctx->stg_ev[s][0][i], ctx->stg_ev[s][1][i]);
        ctx->stats.ms_stage[s] = t;
    }
    ctx->have_run = true;
    ctx->last_nobs = obs->nobs;
    if (st & LG_ST_TIMEOUT)
        return set_err(ctx, LETKF_ERR_TIMEOUT, "a bounded wait on the tensor cores ran out");
    if (st & LG_ST_NOT_CONV)
        return set_err(ctx, LETKF_ERR_NOT_CONVERGED, "an eigensolve reached its sweep limit");
    return LETKF_OK;
}

namespace {

// letkf_gpu_run and letkf_gpu_run_halo: with host buffers the state goes in
// on the copy streams while the geometry, buckets and search run, and the
// staged core's finished blocks go out while later blocks run; the host
// arrays hold the columns in the layout of ctx->host_ld / host_off.
int run_impl(letkf_ctx *ctx, const double *xb, const double *axb, const letkf_obs *obs, double *xa, double *axa,
             bool host, int halo)
{
    int rc = lg_check_run(ctx, obs);
    if (rc) return rc;
    LG_CUDA(cudaSetDevice(ctx->device));
    const size_t nstate = (size_t)ctx->ncol * ctx->n * ctx->k, nmean = (size_t)ctx->ncol * ctx->n;
    ctx->host_ld = ctx->nlat + 2 * (int64_t)halo;
    ctx->host_off = halo + ctx->host_ld * halo;
    LG_CUDA(cudaEventRecord(ctx->ev[0], ctx->stream));
    rc = reset_status(ctx);
    if (rc) return rc;
    const double *dxb = xb, *daxb = axb;
    double *dxa = xa, *daxa = axa;
    if (host) {
        LG_CUDA(copy_streams(ctx));
        LG_CUDA(ctx->d_xa.reserve(nstate));
        LG_CUDA(ctx->d_axa.reserve(nmean));
        // device views of the input arrays for H's rows (null: H waits)
        ctx->gather_xb = ctx->gather_axb = nullptr;
        if (ctx->host_read) {
            const void *vx = host_view(ctx, xb), *va = host_view(ctx, axb);
            if (vx && va) {
                ctx->gather_xb = static_cast<const double *>(vx);
                ctx->gather_axb = static_cast<const double *>(va);
            }
        }
        // from the state copy on, every return passes the join below: no
        // copy may still use the caller's buffers after the call
        ctx->agent_on = pageable(xb) || pageable(axb) || pageable(xa) || pageable(axa);
        ctx->agent_ev_next = 0;
        if (ctx->agent_on && !ctx->agent) {
            try {
                ctx->agent.reset(new LgCopyAgent(ctx->device));
            } catch (const std::exception &) {
                ctx->agent_on = false;
                return set_err(ctx, LETKF_ERR_ALLOC, "cannot start the host copy thread");
            }
        }
        // the state goes in once the observations are staged (lg_run_analysis)
        LG_CUDA(ctx->d_xb.reserve(nstate));
        LG_CUDA(ctx->d_axb.reserve(nmean));
        ctx->copy_xb = xb;
        ctx->copy_axb = axb;
        dxb = ctx->d_xb.p;
        daxb = ctx->d_axb.p;
        dxa = ctx->d_xa.p;
        daxa = ctx->d_axa.p;
        // one column per cube and no averaging over cubes: the core can hand
        // out finished columns (the staged k = 64 core does)
        if (ctx->params.cube_n == 1 && ctx->params.overlap == 0) {
            ctx->sink_xa = xa;
            ctx->sink_axa = axa;
            ctx->sink_dxa = dxa;
            ctx->sink_daxa = daxa;
        }
        ctx->sink_cols = 0;
    }
    unsigned long long cnt[LG_CNT_N] = {};
    // with host buffers the state is still on the copy streams: the H
    // geometry, the buckets and the search run meanwhile
    rc = lg_run_analysis(ctx, obs, host, dxb, daxb, dxa, daxa, cnt, host);
    ctx->sink_xa = nullptr;
    ctx->sink_axa = nullptr;
    if (host) {
        // every copy of the copy streams (the state in, finished blocks out)
        // before the main stream goes on, also when the analysis stopped
        // early; then nothing is left writing into the caller's buffers
        ctx->members_pending = false;
        ctx->lists_need_ef = false;
        const cudaError_t ae = drain_copies(ctx);
        ctx->agent_on = false;
        ctx->npieces = 0;
        ctx->gather_xb = ctx->gather_axb = nullptr;
        ctx->gathered = false;
        ctx->copy_xb = ctx->copy_axb = nullptr;
        for (int i = 0; i < letkf_ctx::kCopyStreams; i++) {
            LG_CUDA(cudaEventRecord(ctx->cev[i], ctx->cstream[i]));
            LG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->cev[i], 0));
        }
        if (!rc && ae != cudaSuccess) rc = set_err(ctx, LETKF_ERR_CUDA, cudaGetErrorString(ae));
        if (rc) cudaStreamSynchronize(ctx->stream);
    }
    if (rc) return rc;
    if (host && ctx->sink_cols != ctx->range1 - ctx->range0) {
        // the columns of the analysed cubes: with cube_n 1 the cubes
        // themselves, else whole longitude strips of them
        int64_t col0 = ctx->range0, col1 = ctx->range1;
        if (ctx->params.cube_n > 1) {
            col0 = ctx->range0 / ctx->nbj * ctx->params.cube_n * ctx->nlat;
            col1 = std::min<int64_t>(ctx->range1 / ctx->nbj * ctx->params.cube_n, ctx->nlon) * ctx->nlat;
        }
        LgCopyJob j;
        j.stream = ctx->stream;
        j.kind = cudaMemcpyDeviceToHost;
        column_parts(ctx, j.part, true, xa, dxa, (size_t)ctx->n * ctx->k, col0, col1);
        column_parts(ctx, j.part, true, axa, daxa, (size_t)ctx->n, col0, col1);
        LG_CUDA(lg_issue_copy(j));
    }
    return lg_finish_run(ctx, obs, cnt);
}

}  // namespace

extern "C" {

int letkf_gpu_run(letkf_ctx *ctx, const double *xb, const double *axb, const letkf_obs *obs,
                  double *xa, double *axa, int flags)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (!xb || !axb || !xa || !axa) return set_err(ctx, LETKF_ERR_INVALID, "NULL state pointer");
    if (flags != LETKF_HOST_PTRS && flags != LETKF_DEVICE_PTRS)
        return set_err(ctx, LETKF_ERR_INVALID, "bad flags");
    return run_impl(ctx, xb, axb, obs, xa, axa, flags == LETKF_HOST_PTRS, 0);
}

int letkf_gpu_run_halo(letkf_ctx *ctx, int halo, const double *xb, const double *axb, const letkf_obs *obs,
                       double *xa, double *axa)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (!xb || !axb || !xa || !axa) return set_err(ctx, LETKF_ERR_INVALID, "NULL state pointer");
    if (halo < 0 || halo > 1 << 16) return set_err(ctx, LETKF_ERR_INVALID, "bad halo width");
    return run_impl(ctx, xb, axb, obs, xa, axa, true, halo);
}

int letkf_gpu_synchronize(letkf_ctx *ctx)
{
    if (!ctx) return LETKF_ERR_INVALID;
    LG_CUDA(cudaStreamSynchronize(ctx->stream));
    return LETKF_OK;
}

int letkf_gpu_obs_operator(letkf_ctx *ctx, const double *xb, const double *axb,
                           const letkf_obs *obs, double *yb, double *dep)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (!xb || !axb || !yb || !dep) return set_err(ctx, LETKF_ERR_INVALID, "NULL pointer");
    int rc = check_obs(ctx, obs);
    if (rc) return rc;
    LG_CUDA(cudaSetDevice(ctx->device));
    const size_t nstate = (size_t)ctx->ncol * ctx->n * ctx->k, nmean = (size_t)ctx->ncol * ctx->n;
    rc = reset_status(ctx);
    if (rc) return rc;
    LG_CUDA(h2d(ctx->d_xb, xb, nstate, ctx->stream));
    LG_CUDA(h2d(ctx->d_axb, axb, nmean, ctx->stream));
    ObsDev od;
    rc = stage_obs(ctx, obs, true, od);
    if (rc) return rc;
    rc = reserve_obs_work(ctx, obs->nobs);
    if (rc) return rc;
    LG_CUDA(lg_launch_obs_prepare(ctx, lg_grid(ctx), ctx->d_xb.p, ctx->d_axb.p, obs->nobs, od.lat,
                                  od.lon, od.ph, od.lev, od.var, od.yo, od.rinv));
    if (obs->nobs > 0) {
        LG_CUDA(cudaMemcpyAsync(yb, ctx->d_yb.p, sizeof(double) * obs->nobs * ctx->k,
                                cudaMemcpyDeviceToHost, ctx->stream));
        LG_CUDA(cudaMemcpyAsync(dep, ctx->d_dep.p, sizeof(double) * obs->nobs,
                                cudaMemcpyDeviceToHost, ctx->stream));
    }
    unsigned st = 0;
    unsigned long long cnt[LG_CNT_N];
    rc = read_status(ctx, st, cnt);
    if (rc) return rc;
    if (st & LG_ST_BAD_OBS)
        return set_err(ctx, LETKF_ERR_INVALID,
                       "observation outside the grid or with a bad variable/level/pressure");
    return LETKF_OK;
}

int letkf_gpu_local_obs_cubes(letkf_ctx *ctx, const int64_t *cubes, int64_t n, int64_t *offsets,
                              int32_t *idx, double *rloc)
{
    if (!ctx || n < 0 || (n > 0 && !cubes) || !offsets) return LETKF_ERR_INVALID;
    if (!ctx->have_run) return set_err(ctx, LETKF_ERR_STATE, "no run yet");
    if (!ctx->lists_whole)
        return set_err(ctx, LETKF_ERR_STATE, "the last run kept no complete lists (cube windows or a cube range)");
    for (int64_t i = 0; i < n; i++)
        if (cubes[i] < 0 || cubes[i] >= ctx->ncubes) return set_err(ctx, LETKF_ERR_INVALID, "cube out of range");
    LG_CUDA(cudaSetDevice(ctx->device));
    LG_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<int64_t> off((size_t)n);
    std::vector<int32_t> cnt((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        LG_CUDA(cudaMemcpy(&off[i], ctx->d_loff.p + cubes[i], sizeof(int64_t), cudaMemcpyDeviceToHost));
        LG_CUDA(cudaMemcpy(&cnt[i], ctx->d_lcnt.p + cubes[i], sizeof(int32_t), cudaMemcpyDeviceToHost));
    }
    offsets[0] = 0;
    for (int64_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + cnt[i];
    for (int64_t i = 0; i < n; i++) {
        if (cnt[i] == 0) continue;
        if (idx)
            LG_CUDA(cudaMemcpy(idx + offsets[i], ctx->d_lidx.p + off[i], sizeof(int32_t) * cnt[i],
                               cudaMemcpyDeviceToHost));
        if (rloc)
            LG_CUDA(cudaMemcpy(rloc + offsets[i], ctx->d_lrloc.p + off[i], sizeof(double) * cnt[i],
                               cudaMemcpyDeviceToHost));
    }
    return LETKF_OK;
}

int letkf_gpu_local_obs(letkf_ctx *ctx, int64_t *offsets, int32_t *idx, double *rloc)
{
    if (!ctx || !offsets) return LETKF_ERR_INVALID;
    if (!ctx->have_run) return set_err(ctx, LETKF_ERR_STATE, "no run yet");
    if (!ctx->lists_whole)
        return set_err(ctx, LETKF_ERR_STATE, "the last run kept no complete lists (cube windows or a cube range)");
    const int64_t nc = ctx->ncubes;
    std::vector<int64_t> off(nc);
    std::vector<int32_t> cnt(nc);
    LG_CUDA(cudaMemcpy(off.data(), ctx->d_loff.p, sizeof(int64_t) * nc, cudaMemcpyDeviceToHost));
    LG_CUDA(cudaMemcpy(cnt.data(), ctx->d_lcnt.p, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost));
    offsets[0] = 0;
    for (int64_t c = 0; c < nc; c++) offsets[c + 1] = offsets[c] + cnt[c];
    if (idx || rloc) {
        const int64_t total = offsets[nc];
        int64_t hi = 0;
        for (int64_t c = 0; c < nc; c++) hi = std::max<int64_t>(hi, off[c] + cnt[c]);
        std::vector<int32_t> li((size_t)std::max<int64_t>(hi, 1));
        std::vector<double> lr((size_t)std::max<int64_t>(hi, 1));
        if (hi > 0) {
            LG_CUDA(cudaMemcpy(li.data(), ctx->d_lidx.p, sizeof(int32_t) * hi, cudaMemcpyDeviceToHost));
            LG_CUDA(cudaMemcpy(lr.data(), ctx->d_lrloc.p, sizeof(double) * hi, cudaMemcpyDeviceToHost));
        }
        for (int64_t c = 0; c < nc; c++) {
            if (idx) std::memcpy(idx + offsets[c], li.data() + off[c], sizeof(int32_t) * cnt[c]);
            if (rloc) std::memcpy(rloc + offsets[c], lr.data() + off[c], sizeof(double) * cnt[c]);
        }
        (void)total;
    }
    return LETKF_OK;
}

int letkf_gpu_last_trans(letkf_ctx *ctx, const int64_t *cubes, int64_t ncubes, double *trans, double *w)
{
    if (!ctx || (!cubes && ncubes > 0)) return LETKF_ERR_INVALID;
    if (!ctx->have_run || !ctx->d_trans.p)
        return set_err(ctx, LETKF_ERR_STATE, "no run with kept transforms (letkf_gpu_set_keep_trans)");
    const int k = ctx->k;
    for (int64_t i = 0; i < ncubes; i++) {
        if (cubes[i] < 0 || cubes[i] >= ctx->ncubes) return set_err(ctx, LETKF_ERR_INVALID, "cube index");
        if (trans)
            LG_CUDA(cudaMemcpy(trans + i * k * k, ctx->d_trans.p + cubes[i] * k * k,
                               sizeof(double) * k * k, cudaMemcpyDeviceToHost));
        if (w)
            LG_CUDA(cudaMemcpy(w + i * k, ctx->d_w.p + cubes[i] * k, sizeof(double) * k,
                               cudaMemcpyDeviceToHost));
    }
    return LETKF_OK;
}

int letkf_gpu_core_batch(letkf_ctx *ctx, int64_t nb, const int64_t *offsets, const double *hxens,
                         const float *rdiaginv, const double *dep, const double *rloc,
                         double *trans, double *w)
{
    if (!ctx || nb < 0 || !offsets || !trans || !w) return LETKF_ERR_INVALID;
    if (nb == 0) return LETKF_OK;
    const int k = ctx->k;
    const int64_t total = offsets[nb];
    if (offsets[0] != 0 || total < 0) return set_err(ctx, LETKF_ERR_INVALID, "offsets");
    std::vector<int32_t> cnt(nb);
    for (int64_t b = 0; b < nb; b++) {
        const int64_t c = offsets[b + 1] - offsets[b];
        if (c < 0 || c > INT32_MAX) return set_err(ctx, LETKF_ERR_INVALID, "offsets not ascending");
        cnt[b] = (int32_t)c;
    }
    if (total > 0 && (!hxens || !rdiaginv || !dep || !rloc))
        return set_err(ctx, LETKF_ERR_INVALID, "NULL obs arrays");
    LG_CUDA(cudaSetDevice(ctx->device));
    int rc = reset_status(ctx);
    if (rc) return rc;
    LG_CUDA(h2d(ctx->d_boff, offsets, (size_t)nb, ctx->stream));
    LG_CUDA(ctx->d_lcnt.reserve((size_t)std::max<int64_t>(nb, ctx->ncubes)));
    LG_CUDA(cudaMemcpyAsync(ctx->d_lcnt.p, cnt.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice,
                            ctx->stream));
    LG_CUDA(h2d(ctx->d_bhx, hxens, (size_t)std::max<int64_t>(total, 1) * k * (total > 0), ctx->stream));
    LG_CUDA(h2d(ctx->d_brdi, rdiaginv, (size_t)total, ctx->stream));
    LG_CUDA(h2d(ctx->d_bdep, dep, (size_t)total, ctx->stream));
    LG_CUDA(h2d(ctx->d_brloc, rloc, (size_t)total, ctx->stream));
    DevBuf<double> dt, dw;
    LG_CUDA(dt.reserve((size_t)nb * k * k));
    LG_CUDA(dw.reserve((size_t)nb * k));
    cudaError_t e = lg_launch_core_batch_fp64(ctx, nb, ctx->d_boff.p, ctx->d_bhx.p, ctx->d_brdi.p,
                                              ctx->d_bdep.p, ctx->d_brloc.p, dt.p, dw.p);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(trans, dt.p, sizeof(double) * nb * k * k, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w, dw.p, sizeof(double) * nb * k, cudaMemcpyDeviceToHost, ctx->stream);
    unsigned st = 0;
    unsigned long long cnt2[LG_CNT_N];
    rc = (e == cudaSuccess) ? read_status(ctx, st, cnt2) : LETKF_ERR_CUDA;
    cudaStreamSynchronize(ctx->stream);
    dt.release();
    dw.release();
    // the per-cube counts of the last run were overwritten
    ctx->have_run = false;
    if (e != cudaSuccess) return set_err(ctx, LETKF_ERR_CUDA, cudaGetErrorString(e));
    if (rc) return rc;
    if (st & LG_ST_NOT_CONV)
        return set_err(ctx, LETKF_ERR_NOT_CONVERGED, "an eigensolve reached its sweep limit");
    return LETKF_OK;
}

int letkf_gpu_get_stats(letkf_ctx *ctx, letkf_stats *stats)
{
    if (!ctx || !stats) return LETKF_ERR_INVALID;
    *stats = ctx->stats;
    return LETKF_OK;
}

const char *letkf_gpu_last_error(letkf_ctx *ctx)
{
    return ctx ? ctx->last_error.c_str() : "no context";
}

int letkf_gpu_destroy(letkf_ctx *ctx)
{
    if (!ctx) return LETKF_OK;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    DevBuf<float> *fb[] = {&ctx->d_glat, &ctx->d_glon, &ctx->d_rinvf, &ctx->d_brdi};
    for (auto *b : fb) b->release();
    DevBuf<double> *db[] = {&ctx->d_hyai, &ctx->d_hybi, &ctx->d_xb, &ctx->d_axb, &ctx->d_xa,
                            &ctx->d_axa, &ctx->d_olat, &ctx->d_olon, &ctx->d_oph, &ctx->d_oyo,
                            &ctx->d_orinv, &ctx->d_yb, &ctx->d_dep, &ctx->d_os, &ctx->d_oc,
                            &ctx->d_oyr, &ctx->d_lrloc, &ctx->d_trans, &ctx->d_w, &ctx->d_bhx,
                            &ctx->d_bdep, &ctx->d_brloc};
    for (auto *b : db) b->release();
    ctx->d_olev.release();
    ctx->d_ovar.release();
    ctx->d_lcnt.release();
    ctx->d_lidx.release();
    ctx->d_loff.release();
    ctx->d_boff.release();
    ctx->d_oxyz.release();
    ctx->d_bxyz.release();
    ctx->d_obucket.release();
    ctx->d_bcount.release();
    ctx->d_bstart.release();
    ctx->d_bidx.release();
    ctx->d_status.release();
    ctx->d_counters.release();
    ctx->d_ymax.release();
    for (int i = 0; i < 8; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    for (int s = 0; s < letkf_ctx::kStages; s++)
        for (int h = 0; h < 2; h++)
            for (int i = 0; i < letkf_ctx::kStageMarks; i++)
                if (ctx->stg_ev[s][h][i]) cudaEventDestroy(ctx->stg_ev[s][h][i]);
    ctx->agent.reset();
    for (cudaEvent_t e : ctx->agent_ev) cudaEventDestroy(e);
    for (int i = 0; i < letkf_ctx::kPieces; i++)
        if (ctx->pev[i]) cudaEventDestroy(ctx->pev[i]);
    if (ctx->gev) cudaEventDestroy(ctx->gev);
    for (int i = 0; i < letkf_ctx::kCopyStreams; i++) {
        if (ctx->cev[i]) cudaEventDestroy(ctx->cev[i]);
        if (ctx->sev[i]) cudaEventDestroy(ctx->sev[i]);
        if (ctx->cstream[i]) cudaStreamDestroy(ctx->cstream[i]);
    }
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return LETKF_OK;
}

// ---------------------------------------------------------------------------
// Fortran-callable shims (one context per process).

static letkf_ctx *g_fctx = nullptr;
static std::vector<double> g_olat, g_olon, g_oph, g_oyo, g_orinv;
static std::vector<int32_t> g_olev, g_ovar;

void letkf_init_gpu_(const int *nlat, const int *nlon, const int *nz, const int *nvar2d,
                     const int *nvar3d, const int *ens, const float *lat, const float *lon,
                     const double *hyai, const double *hybi, const double *p0,
                     const double *ptop, const int *ps_row, const double *loc_dist_km,
                     const double *vert_dist, const double *inflation,
                     const double *obs_polar_deg, const int *gc_filter,
                     const int *gc_filter_vertical, const int *cube_n, const int *cube_nz,
                     const int *overlap, const int *h_mode, const int *precision, int *ierr)
{
    if (g_fctx) {
        letkf_gpu_destroy(g_fctx);
        g_fctx = nullptr;
    }
    letkf_grid g{};
    g.nlat = *nlat;
    g.nlon = *nlon;
    g.nz = *nz;
    g.nvar2d = *nvar2d;
    g.nvar3d = *nvar3d;
    g.ens = *ens;
    g.lat = lat;
    g.lon = lon;
    g.hyai = hyai;
    g.hybi = hybi;
    g.p0 = *p0;
    g.ptop = *ptop;
    g.ps_row = *ps_row - 1;   // Fortran ps_indx is 1-based
    letkf_params p{};
    p.loc_dist_km = *loc_dist_km;
    p.vert_dist = *vert_dist;
    p.inflation = *inflation;
    p.obs_polar_deg = *obs_polar_deg;
    p.gc_filter = *gc_filter;
    p.gc_filter_vertical = *gc_filter_vertical;
    p.max_obs = 10000;
    p.cube_n = *cube_n;
    p.cube_nz = *cube_nz;
    p.overlap = *overlap;
    p.h_mode = *h_mode;
    p.precision = *precision;
    *ierr = letkf_gpu_create(&g_fctx, &g, &p, -1);
}

void letkf_set_obs_gpu_(const int64_t *nobs, const double *lat, const double *lon, const double *ph,
                        const int *lev, const int *var, const double *yo, const double *rinv,
                        int *ierr)
{
    const int64_t n = *nobs;
    if (n < 0) {
        *ierr = LETKF_ERR_INVALID;
        return;
    }
    g_olat.assign(lat, lat + n);
    g_olon.assign(lon, lon + n);
    g_oph.assign(ph, ph + n);
    g_oyo.assign(yo, yo + n);
    g_orinv.assign(rinv, rinv + n);
    g_olev.assign(lev, lev + n);
    g_ovar.resize(n);
    for (int64_t i = 0; i < n; i++) g_ovar[i] = var[i] - 1;
    *ierr = LETKF_OK;
}

void letkf_run_gpu_(const int *ntimes, const int *halo, const double *xb, const double *axb,
                    double *xa, double *axa, int *ierr)
{
    (void)ntimes;
    if (!g_fctx) {
        *ierr = LETKF_ERR_STATE;
        return;
    }
    letkf_obs o{};
    o.nobs = (int64_t)g_olat.size();
    o.lat = g_olat.data();
    o.lon = g_olon.data();
    o.ph = g_oph.data();
    o.lev = g_olev.data();
    o.var = g_ovar.data();
    o.yo = g_oyo.data();
    o.rinv = g_orinv.data();
    // xb(ens, n, 1-halo:nlat+halo, 1-halo:nlon+halo): the copies skip the
    // halo, which xa and axa keep as they were
    *ierr = letkf_gpu_run_halo(g_fctx, *halo, xb, axb, &o, xa, axa);
}

void letkf_final_gpu_(int *ierr)
{
    *ierr = letkf_gpu_destroy(g_fctx);
    g_fctx = nullptr;
}

int letkf_gpu_set_host_read(letkf_ctx *ctx, int on)
{
    if (!ctx) return LETKF_ERR_INVALID;
    ctx->host_read = on ? 1 : 0;
    return LETKF_OK;
}

int letkf_gpu_set_schedule(letkf_ctx *ctx, int chunk)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (chunk != 0 && (chunk < 8 || chunk > 1024 || (chunk & (chunk - 1)) != 0))
        return set_err(ctx, LETKF_ERR_INVALID, "the chunk must be 0 or a power of two from 8 to 1024");
    ctx->sched_chunk = chunk;
    return LETKF_OK;
}

int letkf_gpu_autotune(letkf_ctx *ctx, const double *xb, const double *axb, const letkf_obs *obs,
                       double *xa, double *axa, int flags)
{
    if (!ctx) return LETKF_ERR_INVALID;
    if (!lg_is_mixed(ctx->params.precision))
        return letkf_gpu_run(ctx, xb, axb, obs, xa, axa, flags);
    // chunk sizes of the mixed core's work queue: small chunks balance the
    // load, large ones cost fewer queue fetches; the fastest core wins (the
    // one-launch cores take chunks of whole warm-start runs)
    static const int cand64[] = {8, 16, 32, 64}, cand[] = {16, 32, 64, 128};
    int best = 0;
    double best_ms = 1e300;
    for (int c : (ctx->k == 64 ? cand64 : cand)) {
        ctx->sched_chunk = c;
        const int rc = letkf_gpu_run(ctx, xb, axb, obs, xa, axa, flags);
        if (rc != LETKF_OK && rc != LETKF_ERR_NOT_CONVERGED) return rc;
        if (flags == LETKF_DEVICE_PTRS) LG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (ctx->stats.ms_core < best_ms) {
            best_ms = ctx->stats.ms_core;
            best = c;
        }
    }
    ctx->sched_chunk = best;
    ctx->stats.sched_chunk = best;
    return LETKF_OK;
}

}  // extern "C"

struct letkf_batch {
    int n = 0;
    std::vector<letkf_ctx *> ctx;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> joins;
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
    std::string last_error;
};

namespace {

void batch_release(letkf_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto e : b->joins)
        if (e) cudaEventDestroy(e);
    for (auto s : b->streams)
        if (s) cudaStreamDestroy(s);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
}

}  // namespace

extern "C" {

int letkf_batch_create(letkf_batch **out, int n, letkf_ctx *const *ctxs, const double *const *xb,
                       const double *const *axb, const letkf_obs *obs, double *const *xa, double *const *axa)
{
    if (!out || n < 1 || !ctxs || !xb || !axb || !obs || !xa || !axa) return LETKF_ERR_INVALID;
    *out = nullptr;
    for (int i = 0; i < n; i++)
        if (!ctxs[i] || ctxs[i]->device != ctxs[0]->device) return LETKF_ERR_INVALID;
    for (int i = 0; i < n; i++)
        if (ctxs[i]->dec_nx > 0)
            return set_err(ctxs[i], LETKF_ERR_UNSUPPORTED,
                           "decomposed observation sets are not captured in graphs");
    // one analysis of each instance outside the graph sizes every buffer
    for (int i = 0; i < n; i++) {
        const int rc = letkf_gpu_run(ctxs[i], xb[i], axb[i], &obs[i], xa[i], axa[i], LETKF_DEVICE_PTRS);
        if (rc != LETKF_OK && rc != LETKF_ERR_NOT_CONVERGED) return rc;
        if (letkf_gpu_synchronize(ctxs[i]) != LETKF_OK) return LETKF_ERR_CUDA;
    }
    letkf_batch *b = new letkf_batch();
    b->n = n;
    b->ctx.assign(ctxs, ctxs + n);
    b->streams.assign(n, nullptr);
    b->joins.assign(n, nullptr);
    std::vector<cudaStream_t> saved(n, nullptr);
    auto fail = [&](int rc) {
        for (int i = 0; i < n; i++)
            if (saved[i]) ctxs[i]->stream = saved[i];
        batch_release(b);
        return rc;
    };
    if (cudaSetDevice(ctxs[0]->device) != cudaSuccess) return fail(LETKF_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
        return fail(LETKF_ERR_CUDA);
    for (int i = 0; i < n; i++)
        if (cudaStreamCreateWithFlags(&b->streams[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming) != cudaSuccess)
            return fail(LETKF_ERR_CUDA);
    // every instance on its own stream, forked from and joined to the origin
    const int64_t l0 = g_launches.load();
    if (cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        return fail(LETKF_ERR_CUDA);
    int rc = LETKF_OK;
    if (cudaEventRecord(b->fork, b->origin) != cudaSuccess) rc = LETKF_ERR_CUDA;
    for (int i = 0; i < n && rc == LETKF_OK; i++) {
        saved[i] = ctxs[i]->stream;
        ctxs[i]->stream = b->streams[i];
        if (cudaStreamWaitEvent(b->streams[i], b->fork, 0) != cudaSuccess) rc = LETKF_ERR_CUDA;
        if (rc == LETKF_OK) rc = enqueue_run(ctxs[i], xb[i], axb[i], &obs[i], xa[i], axa[i]);
        if (rc == LETKF_OK && (cudaEventRecord(b->joins[i], b->streams[i]) != cudaSuccess ||
                               cudaStreamWaitEvent(b->origin, b->joins[i], 0) != cudaSuccess))
            rc = LETKF_ERR_CUDA;
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->origin, &graph);
    for (int i = 0; i < n; i++)
        if (saved[i]) {
            ctxs[i]->stream = saved[i];
            saved[i] = nullptr;
        }
    if (rc != LETKF_OK) {
        if (graph) cudaGraphDestroy(graph);
        return fail(rc);
    }
    if (ec != cudaSuccess || !graph) return fail(LETKF_ERR_CUDA);
    b->graph = graph;
    if (cudaGraphInstantiate(&b->exec, graph, 0) != cudaSuccess) return fail(LETKF_ERR_CUDA);
    b->launches = g_launches.load() - l0;
    *out = b;
    return LETKF_OK;
}

int letkf_batch_launch(letkf_batch *b, void *stream)
{
    if (!b || !b->exec) return LETKF_ERR_INVALID;
    const cudaError_t e = cudaGraphLaunch(b->exec, stream ? (cudaStream_t)stream : b->origin);
    if (e != cudaSuccess) {
        b->last_error = cudaGetErrorString(e);
        return LETKF_ERR_CUDA;
    }
    g_launches.fetch_add(b->launches, std::memory_order_relaxed);
    return LETKF_OK;
}

int letkf_batch_sync(letkf_batch *b, void *stream)
{
    if (!b) return LETKF_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(stream ? (cudaStream_t)stream : b->origin);
    if (e != cudaSuccess) {
        b->last_error = cudaGetErrorString(e);
        return LETKF_ERR_CUDA;
    }
    int worst = LETKF_OK;
    for (letkf_ctx *ctx : b->ctx) {
        unsigned st = 0;
        unsigned long long cnt[LG_CNT_N] = {};
        const int rc = read_status(ctx, st, cnt);
        if (rc) return rc;
        fill_stats(ctx, cnt);
        int r = LETKF_OK;
        if (st & LG_ST_LIST_FULL) r = set_err(ctx, LETKF_ERR_ALLOC, "local observation lists did not fit");
        else if (st & LG_ST_BAD_OBS) r = set_err(ctx, LETKF_ERR_INVALID, "bad observation");
        else if (st & LG_ST_TIMEOUT) r = set_err(ctx, LETKF_ERR_TIMEOUT, "a bounded wait on the tensor cores ran out");
        else if (st & LG_ST_SEGMENTS) r = set_err(ctx, LETKF_ERR_UNSUPPORTED, "localization cap spans too many buckets");
        else if (st & LG_ST_NOT_CONV) r = set_err(ctx, LETKF_ERR_NOT_CONVERGED, "eigensolve did not converge");
        if (worst == LETKF_OK) worst = r;
    }
    return worst;
}

int64_t letkf_batch_launches(letkf_batch *b) { return b ? b->launches : 0; }

int letkf_batch_destroy(letkf_batch *b)
{
    if (!b) return LETKF_OK;
    cudaSetDevice(b->ctx.empty() ? 0 : b->ctx[0]->device);
    if (b->origin) cudaStreamSynchronize(b->origin);
    batch_release(b);
    return LETKF_OK;
}

}  // extern "C"
