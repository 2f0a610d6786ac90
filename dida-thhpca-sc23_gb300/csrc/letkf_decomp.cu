// letkf_decomp.cu -- observation sets of a decomposed DA group.
//
// The reference runs the DA on P MPI ranks, each owning one lat x lon block
// of the grid.  A rank reads the observations inside its block's box, swaps
// them with the ranks of its neighbour set, and a column's local list scans
// those blocks in a fixed order (code/x86/TradDA/DA/LETKF/src/letkf_yb.F90:
// 71-133).  Which blocks a rank scans, and which obs a block holds, decide
// the lists, so a P-rank run's analysis differs from a one-block run's.  This
// file reproduces them on one GPU:
//   * host, once per context: the block ranges (pro_info_get_indx,
//     DA/utils/pro_info.F90:96-125), the boxes the obs store is queried with
//     (read_obs_mod.F90:73-165; bounds printed "%.5f" by the store client,
//     LIB/REDIS/src/redis_wrapper.c:4097-4117) and every block's neighbour
//     list (comm_info_init and nearest_dist, letkf_init.F90:100-341);
//   * device, once per run: the obs of every block in ascending index order
//     (a count pass and an ordered fill pass over (block, obs chunk) tiles).
// The per-column scan is k_search_dec in letkf_search.cu.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "letkf_internal.cuh"

namespace {

constexpr int kMemThreads = 256;
constexpr int kMemChunk = 8 * kMemThreads;     // obs per (block, chunk) tile

// pro_info_get_indx along one axis: 1-based inclusive range of block b
// (1-based) of n points in nb blocks, the first n mod nb blocks one longer.
void block_range(int n, int nb, int b, int &s, int &e)
{
    const int sec = n / nb, res = n % nb;
    if (b - 1 < res) {
        s = (b - 1) * (sec + 1) + 1;
        e = s + sec;
    } else {
        s = (b - 1) * sec + res + 1;
        e = s + sec - 1;
    }
}

struct HostGrid {
    const std::vector<float> &lat, &lon;   // with grid_lat(nlat+1) = 90, grid_lon(nlon+1) = 360
    int nlat, nlon;
    float glat(int i) const { return lat[i - 1]; }   // 1-based
    float glon(int j) const { return lon[j - 1]; }
};

// latlon_dist_r8 (pro_info.F90:149-161): double evaluation with the float pi
// and Earth radius.
double dist_r8(double x1, double y1, double x2, double y2)
{
    const double pi = (double)(atanf(1.0f) * 4.0f), a = (double)6371.393f;
    double v = std::cos(x1 / 180.0 * pi) * std::cos(x2 / 180.0 * pi) * std::cos(y1 / 180.0 * pi - y2 / 180.0 * pi) +
               std::sin(x1 / 180.0 * pi) * std::sin(x2 / 180.0 * pi);
    if (v > 1.0) v = 1.0;
    return a * std::acos(v);
}

// latlon_dist_r4 (pro_info.F90:163-175): the same in single precision.
float dist_r4(float x1, float y1, float x2, float y2)
{
    const float pi = atanf(1.0f) * 4.0f, a = 6371.393f;
    float v = cosf(x1 / 180.0f * pi) * cosf(x2 / 180.0f * pi) * cosf(y1 / 180.0f * pi - y2 / 180.0f * pi) +
              sinf(x1 / 180.0f * pi) * sinf(x2 / 180.0f * pi);
    if (v > 1.0f) v = 1.0f;
    return a * acosf(v);
}

// nearest_dist (letkf_init.F90:293-341), blocks 1-based.
double nearest_dist(const HostGrid &G, int NX, int NY, double polar, int bx1, int by1, int bx2, int by2)
{
    int xs1, xe1, ys1, ye1, xs2, xe2, ys2, ye2, tx1, tx2;
    block_range(G.nlat, NX, bx1, xs1, xe1);
    block_range(G.nlon, NY, by1, ys1, ye1);
    block_range(G.nlat, NX, bx2, xs2, xe2);
    block_range(G.nlon, NY, by2, ys2, ye2);
    if (bx1 > bx2) {
        tx1 = xs1;
        tx2 = xe2 + 1;
    } else if (bx1 < bx2) {
        tx1 = xe1 + 1;
        tx2 = xs2;
    } else if (bx1 > NX / 2) {
        tx1 = xe1 + 1;
        tx2 = xe2 + 1;
    } else {
        tx1 = xs1;
        tx2 = xs2;
    }
    float lat1 = G.glat(tx1), lat2 = G.glat(tx2);
    if (std::fabs((double)lat1) > polar) lat1 = (float)(lat1 < 0.0f ? -polar : polar);
    if (std::fabs((double)lat2) > polar) lat2 = (float)(lat2 < 0.0f ? -polar : polar);
    if (by1 == by2) return (double)dist_r4(lat1, G.glon(ys1), lat2, G.glon(ys2));
    const float d1 = dist_r4(lat1, G.glon(ys1), lat2, G.glon(ye2 % G.nlon + 1));
    const float d2 = dist_r4(lat1, G.glon(ye1 % G.nlon + 1), lat2, G.glon(ys2));
    return (double)std::min(d1, d2);
}

// comm_info_init (letkf_init.F90:100-177): the blocks block (bx, by) (1-based)
// scans, as 0-based ids bx' * NY + by', in scan order.  Blocks are compared
// with local_dist itself although obs are kept out to 2 local_dist.
void block_slots(const HostGrid &G, int NX, int NY, double c, double polar, int bx, int by,
                 std::vector<int> &out)
{
    int s_lat, e_lat, s_lon, e_lon, ts, te;
    block_range(G.nlat, NX, bx, s_lat, e_lat);
    block_range(G.nlon, NY, by, s_lon, e_lon);
    const double y1 = G.glon(s_lon);
    int north = 0, south = 0;
    for (int t = bx - 1; t > 0; t--) {
        block_range(G.nlat, NX, t, ts, te);
        if (dist_r8(G.glat(s_lat), y1, G.glat(te + 1), y1) > c) break;
        north++;
    }
    for (int t = bx + 1; t <= NX; t++) {
        block_range(G.nlat, NX, t, ts, te);
        if (dist_r8(G.glat(e_lat + 1), y1, G.glat(ts), y1) > c) break;
        south++;
    }
    for (int i = -north; i <= south; i++) {
        const int tbx = bx + i;
        int west = 0, east = 0, tby = by;
        while (west <= (NY - 1) / 2) {
            tby = (tby + NY - 2) % NY + 1;
            if (nearest_dist(G, NX, NY, polar, bx, by, tbx, tby) > c) break;
            west++;
        }
        tby = by;
        while (east <= (NY - 1) / 2) {
            tby = tby % NY + 1;
            if (nearest_dist(G, NX, NY, polar, bx, by, tbx, tby) > c) break;
            east++;
        }
        if (west + east > NY - 1) east--;
        for (int j = -west; j <= east; j++) out.push_back((tbx - 1) * NY + ((by - 1 + j) % NY + NY) % NY);
    }
}

// The store's range query sees a box bound as the float printed "%.5f".
double box_bound(float v)
{
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.5f", (double)v);
    return std::strtod(buf, nullptr);
}

// Block membership of the obs of one (block, chunk) tile.
//   mode 0: cnt[b * nchunk + c] = number of obs of the chunk inside block b
//   mode 1: write them, in index order, from pos[b * nchunk + c]
__global__ void __launch_bounds__(kMemThreads)
k_block_members(int mode, int64_t nobs, const double *__restrict__ olat, const double *__restrict__ olon,
                const double *__restrict__ box, int NX, int NY, int nchunk, int *__restrict__ cnt,
                const int *__restrict__ pos, int *__restrict__ out)
{
    __shared__ int s_warp[kMemThreads / 32];
    const int c = blockIdx.x, b = blockIdx.y;
    const int bx = b / NY, by = b % NY;
    const double la0 = box[bx], la1 = box[NX + bx], lo0 = box[2 * NX + by], lo1 = box[2 * NX + NY + by];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int run = mode == 1 ? pos[(int64_t)b * nchunk + c] : 0;
    int total = 0;
    for (int step = 0; step < kMemChunk / kMemThreads; step++) {
        const int64_t o = (int64_t)c * kMemChunk + step * kMemThreads + threadIdx.x;
        bool in = false;
        if (o < nobs) {
            const double la = olat[o], lo = olon[o];
            in = la >= la0 && la <= la1 && lo >= lo0 && lo <= lo1;
        }
        if (mode == 0) {
            total += __syncthreads_count(in);
            continue;
        }
        const unsigned ball = __ballot_sync(0xffffffffu, in);
        if (lane == 0) s_warp[warp] = __popc(ball);
        __syncthreads();
        int before = 0, all = 0;
#pragma unroll
        for (int w = 0; w < kMemThreads / 32; w++) {
            before += (w < warp) ? s_warp[w] : 0;
            all += s_warp[w];
        }
        if (in) out[run + before + __popc(ball & ((1u << lane) - 1u))] = (int)o;
        run += all;
        __syncthreads();
    }
    if (mode == 0 && threadIdx.x == 0) cnt[(int64_t)b * nchunk + c] = total;
}

}  // namespace

int lg_decomp_dims(int nranks, int &lat_blocks, int &lon_blocks)
{
    if (nranks < 1) return -1;
    int best = 1;
    for (int b = 1; (int64_t)b * b <= nranks; b++)
        if (nranks % b == 0) best = b;
    lon_blocks = nranks / best;      // dims(1) >= dims(2); dims(1) splits longitude
    lat_blocks = best;
    return 0;
}

cudaError_t lg_decomp_setup(letkf_ctx *ctx, const std::vector<float> &glat_ext,
                            const std::vector<float> &glon_ext)
{
    const int NX = ctx->params.decomp_lat_blocks, NY = ctx->params.decomp_lon_blocks;
    ctx->dec_nx = NX;
    ctx->dec_ny = NY;
    const HostGrid G{glat_ext, glon_ext, ctx->nlat, ctx->nlon};
    std::vector<double> box(2 * NX + 2 * NY);
    std::vector<int> row_blk(ctx->nlat), col_blk(ctx->nlon);
    for (int b = 1; b <= NX; b++) {
        int s, e;
        block_range(ctx->nlat, NX, b, s, e);
        box[b - 1] = box_bound(G.glat(s));
        box[NX + b - 1] = box_bound(G.glat(e + 1));
        for (int i = s; i <= e; i++) row_blk[i - 1] = b - 1;
    }
    for (int b = 1; b <= NY; b++) {
        int s, e;
        block_range(ctx->nlon, NY, b, s, e);
        box[2 * NX + b - 1] = box_bound(G.glon(s));
        box[2 * NX + NY + b - 1] = box_bound(G.glon(e + 1));
        for (int i = s; i <= e; i++) col_blk[i - 1] = b - 1;
    }
    std::vector<int> slot_off(1, 0), slot_blk;
    for (int bx = 1; bx <= NX; bx++)
        for (int by = 1; by <= NY; by++) {
            block_slots(G, NX, NY, ctx->params.loc_dist_km, ctx->params.obs_polar_deg, bx, by, slot_blk);
            slot_off.push_back((int)slot_blk.size());
        }
    if (slot_blk.empty()) slot_blk.push_back(0);
    cudaError_t e;
    if ((e = ctx->d_dec_box.reserve(box.size())) != cudaSuccess) return e;
    if ((e = ctx->d_dec_row_blk.reserve(row_blk.size())) != cudaSuccess) return e;
    if ((e = ctx->d_dec_col_blk.reserve(col_blk.size())) != cudaSuccess) return e;
    if ((e = ctx->d_dec_slot_off.reserve(slot_off.size())) != cudaSuccess) return e;
    if ((e = ctx->d_dec_slot_blk.reserve(slot_blk.size())) != cudaSuccess) return e;
    if ((e = cudaMemcpy(ctx->d_dec_box.p, box.data(), sizeof(double) * box.size(), cudaMemcpyHostToDevice)))
        return e;
    if ((e = cudaMemcpy(ctx->d_dec_row_blk.p, row_blk.data(), sizeof(int) * row_blk.size(),
                        cudaMemcpyHostToDevice)))
        return e;
    if ((e = cudaMemcpy(ctx->d_dec_col_blk.p, col_blk.data(), sizeof(int) * col_blk.size(),
                        cudaMemcpyHostToDevice)))
        return e;
    if ((e = cudaMemcpy(ctx->d_dec_slot_off.p, slot_off.data(), sizeof(int) * slot_off.size(),
                        cudaMemcpyHostToDevice)))
        return e;
    return cudaMemcpy(ctx->d_dec_slot_blk.p, slot_blk.data(), sizeof(int) * slot_blk.size(),
                      cudaMemcpyHostToDevice);
}

cudaError_t lg_launch_block_members(letkf_ctx *ctx, int64_t nobs, const double *olat, const double *olon)
{
    const int NX = ctx->dec_nx, NY = ctx->dec_ny, nb = NX * NY;
    const int nchunk = (int)std::max<int64_t>(1, (nobs + kMemChunk - 1) / kMemChunk);
    ctx->dec_nchunk = nchunk;
    const size_t ntile = (size_t)nb * nchunk;
    cudaError_t e;
    if ((e = ctx->d_dec_cnt.reserve(ntile + 1)) != cudaSuccess) return e;
    if ((e = ctx->d_dec_pos.reserve(ntile + 1)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(ctx->d_dec_cnt.p, 0, sizeof(int) * (ntile + 1), ctx->stream)) != cudaSuccess)
        return e;
    const dim3 grid((unsigned)nchunk, (unsigned)nb);
    lg_count_launch();
    k_block_members<<<grid, kMemThreads, 0, ctx->stream>>>(0, nobs, olat, olon, ctx->d_dec_box.p, NX, NY,
                                                            nchunk, ctx->d_dec_cnt.p, nullptr, nullptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    lg_launch_scan_exclusive(ctx->d_dec_cnt.p, ctx->d_dec_pos.p, (int)ntile, ctx->stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int total = 0;
    if ((e = cudaMemcpyAsync(&total, ctx->d_dec_pos.p + ntile, sizeof(int), cudaMemcpyDeviceToHost,
                             ctx->stream)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return e;
    if ((e = ctx->d_dec_obs.reserve((size_t)std::max(total, 1))) != cudaSuccess) return e;
    if (total == 0) return cudaSuccess;
    lg_count_launch();
    k_block_members<<<grid, kMemThreads, 0, ctx->stream>>>(1, nobs, olat, olon, ctx->d_dec_box.p, NX, NY,
                                                            nchunk, nullptr, ctx->d_dec_pos.p,
                                                            ctx->d_dec_obs.p);
    return cudaGetLastError();
}
