/*
 * letkf_oracle.c -- CPU restatement of the reference LETKF analysis path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path.  See letkf_oracle.h
 * for the data layout.  Compiled with -ffp-contract=off so that no multiply-add
 * is fused: every expression rounds exactly as its Fortran source does when
 * evaluated left to right in IEEE double.
 *
 * Reference paths below are relative to code/x86/TradDA/.
 */
#include "letkf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* pi = atan(1.0) * 4 in default (single) precision, promoted to real(8):
 * DA/utils/pro_info.F90:156.  Earth radius `a` is the default-real literal
 * 6371.393 promoted to real(8): DA/utils/pro_info.F90:148.                  */
#define ORC_PI_F32 3.1415927410125732421875
#define ORC_EARTH_A 6371.39306640625

/* Default-real literals 1.666667 and 0.6666667 of schr2, promoted to real(8):
 * DA/LETKF/src/letkf_yb.F90:256-261.                                        */
#define ORC_GC_C1 1.66666698455810546875
#define ORC_GC_C2 0.666666686534881591796875

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* schr2: Gaspari-Cohn 5th-order piecewise rational function.
 * DA/LETKF/src/letkf_yb.F90:245-269.  A NaN argument fails every `>` test and
 * returns 1.0, as the Fortran does.                                          */
double orc_schr2(double ri)
{
    double rci, rj, rk;
    if (ri > 2.0) {
        rci = 0.0;
    } else if (ri > 1.0) {
        rj = ri / 12.0 - 0.5;
        rj = rj * ri + 0.625;
        rj = rj * ri + ORC_GC_C1;
        rci = (rj * ri - 5.0) * ri + 4.0 - ORC_GC_C2 / ri;
    } else if (ri > 0.0) {
        rk = ri * ri;
        rj = (-0.25 * ri + 0.5) * ri + 0.625;
        rci = (rj * ri - ORC_GC_C1) * rk + 1.0;
    } else {
        rci = 1.0;
    }
    return rci;
}

/* schr: box-car.  DA/LETKF/src/letkf_yb.F90:270-285. */
double orc_schr(double ri)
{
    return (ri > 2.0) ? 0.0 : 1.0;
}

/* latlon_dist_r8: great-circle distance in km.  DA/utils/pro_info.F90:149-161.
 * x = latitude, y = longitude, degrees.                                      */
double orc_latlon_dist(double x1, double y1, double x2, double y2)
{
    const double pi = ORC_PI_F32;
    double x1r = x1 / 180.0 * pi, x2r = x2 / 180.0 * pi;
    double y1r = y1 / 180.0 * pi, y2r = y2 / 180.0 * pi;
    double v = cos(x1r) * cos(x2r) * cos(y1r - y2r) + sin(x1r) * sin(x2r);
    /* Fortran min(v, 1.0) */
    if (v > 1.0) v = 1.0;
    return ORC_EARTH_A * acos(v);
}

/* Same distance with the sin/cos of both latitudes and the longitudes in
 * radians precomputed; bitwise identical to orc_latlon_dist.                 */
static inline double dist_pre(double s1, double c1, double y1r,
                              double s2, double c2, double y2r)
{
    double v = c1 * c2 * cos(y1r - y2r) + s1 * s2;
    if (v > 1.0) v = 1.0;
    return ORC_EARTH_A * acos(v);
}

static inline double lat_rad(double x) { return x / 180.0 * ORC_PI_F32; }

/* Extended float grid: grid_lat(nx+1) = 90 and grid_lon(ny+1) = 360 for the
 * last block (DA/utils/pro_info.F90:77-83).                                  */
static inline float glat_ext(const orc_config *cfg, int i /* 1-based */)
{
    return (i <= cfg->nlat) ? cfg->glat[i - 1] : 90.0f;
}
static inline float glon_ext(const orc_config *cfg, int j /* 1-based */)
{
    return (j <= cfg->nlon) ? cfg->glon[j - 1] : 360.0f;
}

/* find_obs_grid: first grid index with grid >= obs coordinate, and the weight
 * of the point before it.  DA/LETKF/src/letkf_obs.F90:187-243.  The grid
 * spacing is a real(4) difference (grid_lat is real(4)).                     */
int orc_find_obs_grid(const orc_config *cfg, double lat, double lon,
                      int *tx, int *ty, double *ax, double *ay)
{
    int i;
    *tx = 0;
    for (i = 1; i <= cfg->nlat + 1; i++) {
        if ((double)glat_ext(cfg, i) >= lat) { *tx = i; break; }
    }
    *ty = 0;
    for (i = 1; i <= cfg->nlon + 1; i++) {
        if ((double)glon_ext(cfg, i) >= lon) { *ty = i; break; }
    }
    if (*tx == 0 || *ty == 0) return -1;
    if (*tx > 1) {
        float dlf = glat_ext(cfg, *tx) - glat_ext(cfg, *tx - 1);
        double dlat = (double)dlf;
        *ax = (dlat - lat + (double)glat_ext(cfg, *tx - 1)) / dlat;
    } else {
        *ax = 0.0;
    }
    if (*ty > 1) {
        float dlf = glon_ext(cfg, *ty) - glon_ext(cfg, *ty - 1);
        double dlon = (double)dlf;
        *ay = (dlon - lon + (double)glon_ext(cfg, *ty - 1)) / dlon;
    } else {
        *ay = 0.0;
    }
    return 0;
}

/* Grid row / column of a 1-based extended index.  Rows beyond the poles clamp
 * to the nearest row; columns wrap around the periodic longitude circle.    */
static inline int lat_row(const orc_config *cfg, int i1)
{
    int r = i1 - 1;
    if (r < 0) r = 0;
    if (r > cfg->nlat - 1) r = cfg->nlat - 1;
    return r;
}
static inline int lon_col(const orc_config *cfg, int j1)
{
    int c = (j1 - 1) % cfg->nlon;
    if (c < 0) c += cfg->nlon;
    return c;
}

static inline int state_rows(const orc_config *cfg)
{
    return cfg->nvar2d + cfg->nvar3d * cfg->nz;
}
static inline int var_start(const orc_config *cfg, int v)
{
    return (v < cfg->nvar2d) ? v : cfg->nvar2d + (v - cfg->nvar2d) * cfg->nz;
}

typedef struct {
    int64_t c11, c21, c12, c22;  /* column indices of (lat tx-1, lon ty-1) ... */
    double t1, t2;
} corners;

/* Bilinear value of member e at state row r:
 * DA/LETKF/src/obs_make.F90:285-294 (r1/r2 then r1*t2 + r2*(1-t2)).          */
static inline double bilin(const orc_config *cfg, const double *xb, const double *axb,
                           const corners *q, int r, int e)
{
    int n = state_rows(cfg), k = cfg->k;
#define V(c) (xb[((c) * n + r) * (int64_t)k + e] + axb[(c) * n + r])
    double r1 = V(q->c11) * q->t1 + V(q->c21) * (1 - q->t1);
    double r2 = V(q->c12) * q->t1 + V(q->c22) * (1 - q->t1);
#undef V
    return r1 * q->t2 + r2 * (1 - q->t2);
}

/* Interface pressure of level i (0-based, i = 0..nz):
 * da_hybrid_coord_calc_ph_lev, DA/utils/vert_coord_mod.F90:556-563.          */
static inline double ph_lev(const orc_config *cfg, int i, double ps)
{
    return cfg->hyai[i] * (cfg->p0 - cfg->ptop) + cfg->hybi[i] * (ps - cfg->ptop) + cfg->ptop;
}

/* gen_obs_struct after the read: H for every obs and member
 * (DA/LETKF/src/letkf_obs.F90:120-154, obs_make.F90:233-381), then the
 * ensemble-mean removal (letkf_obs.F90:156-178).  With h_mode 1 the obs level
 * is a model level index and H is bilinear at that level.                    */
int orc_obs_operator(const orc_config *cfg, const double *xb, const double *axb,
                     const orc_obs *obs, double *yb, double *dep)
{
    const int k = cfg->k, nz = cfg->nz;
    int64_t o;
    int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (o = 0; o < obs->nobs; o++) {
        int tx, ty, e, v = obs->var[o];
        double ax, ay;
        corners q;
        double *y = yb + o * (int64_t)k;
        if (orc_find_obs_grid(cfg, obs->lat[o], obs->lon[o], &tx, &ty, &ax, &ay) != 0) {
            err |= 1;
            continue;
        }
        {
            int la0 = lat_row(cfg, tx - 1), la1 = lat_row(cfg, tx);
            int lo0 = lon_col(cfg, ty - 1), lo1 = lon_col(cfg, ty);
            q.c11 = la0 + (int64_t)cfg->nlat * lo0;
            q.c21 = la1 + (int64_t)cfg->nlat * lo0;
            q.c12 = la0 + (int64_t)cfg->nlat * lo1;
            q.c22 = la1 + (int64_t)cfg->nlat * lo1;
            q.t1 = ax;
            q.t2 = ay;
        }
        if (v < cfg->nvar2d) {
            for (e = 0; e < k; e++) y[e] = bilin(cfg, xb, axb, &q, var_start(cfg, v), e);
        } else if (cfg->h_mode == 1) {
            int row = var_start(cfg, v) + obs->lev[o] - 1;
            for (e = 0; e < k; e++) y[e] = bilin(cfg, xb, axb, &q, row, e);
        } else {
            /* ps2ph_3d_interp (obs_make.F90:345-381) then the level search and
             * log-p interpolation of obs_interpolation_3d_2 (:252-321).      */
            double oph = obs->ph[o];
            double *ph = (double *)malloc(sizeof(double) * (nz + 1));
            for (e = 0; e < k; e++) {
                double ps = bilin(cfg, xb, axb, &q, cfg->ps_row, e);
                int i, j, pos, start = var_start(cfg, v);
                for (i = 0; i < nz; i++)
                    ph[i] = 0.5 * (ph_lev(cfg, i, ps) + ph_lev(cfg, i + 1, ps));
                ph[nz] = ph[nz - 1];
                j = 1;
                while (j <= nz && oph > ph[j - 1]) j++;
                pos = j - 1;
                if (pos >= 1 && pos < nz) {
                    int tl = start + pos - 1;
                    double t3 = (log(ph[pos]) - log(oph)) / (log(ph[pos]) - log(ph[pos - 1]));
                    double r1 = bilin(cfg, xb, axb, &q, tl, e);
                    double r3 = bilin(cfg, xb, axb, &q, tl + 1, e);
                    y[e] = r1 * t3 + r3 * (1 - t3);
                } else {
                    int tl = (pos == 0) ? start : start + nz - 1;
                    y[e] = bilin(cfg, xb, axb, &q, tl, e);
                }
            }
            free(ph);
        }
        {
            double sum_y = 0.0;
            for (e = 0; e < k; e++) sum_y = sum_y + y[e];
            sum_y = sum_y / k;
            dep[o] = obs->yo[o] - sum_y;
            for (e = 0; e < k; e++) y[e] = y[e] - sum_y;
        }
    }
    return err ? -1 : 0;
}

/* Column loop bounds: letkf_compute_nooverlap, DA/LETKF/src/letkf_compute.F90:53-65.
 * Cubes are numbered lon-block-major, as the loops run.  Bounds are 0-based
 * and inclusive.                                                             */
int64_t orc_num_cubes(const orc_config *cfg)
{
    int64_t nbj = (cfg->nlat + cfg->cube_n - 1) / cfg->cube_n;
    int64_t nbi = (cfg->nlon + cfg->cube_n - 1) / cfg->cube_n;
    return nbj * nbi;
}

void orc_cube_bounds(const orc_config *cfg, int64_t cube, int *sj, int *ej, int *si, int *ei)
{
    int64_t nbj = (cfg->nlat + cfg->cube_n - 1) / cfg->cube_n;
    int bj = (int)(cube % nbj), bi = (int)(cube / nbj);
    *sj = bj * cfg->cube_n;
    *ej = *sj + cfg->cube_n - 1;
    if (*ej > cfg->nlat - 1) *ej = cfg->nlat - 1;
    *si = bi * cfg->cube_n;
    *ei = *si + cfg->cube_n - 1;
    if (*ei > cfg->nlon - 1) *ei = cfg->nlon - 1;
}

/* Cube centre: grid_lat((sj+ej)/2), grid_lon((si+ei)/2) with 1-based Fortran
 * integer division (letkf_yb.F90:19-20).                                     */
void orc_cube_center(const orc_config *cfg, int sj, int ej, int si, int ei,
                     double *clat, double *clon)
{
    int cj = ((sj + 1) + (ej + 1)) / 2, ci = ((si + 1) + (ei + 1)) / 2;
    *clat = (double)cfg->glat[cj - 1];
    *clon = (double)cfg->glon[ci - 1];
}

/* ---- local observation search ------------------------------------------ */

typedef struct {
    double lat;
    int32_t idx;
} lat_key;

static int cmp_lat(const void *a, const void *b)
{
    const lat_key *x = (const lat_key *)a, *y = (const lat_key *)b;
    if (x->lat < y->lat) return -1;
    if (x->lat > y->lat) return 1;
    return (x->idx < y->idx) ? -1 : (x->idx > y->idx);
}
static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x < y) ? -1 : (x > y);
}

typedef struct {
    lat_key *keys;        /* obs sorted by latitude */
    double *s, *c, *yr;   /* sin/cos of obs latitude, obs longitude in radians */
    int64_t n;
    /* decomposed mode: obs of each block (ascending), neighbour slots */
    int nbx, nby;
    int *bx_of_row, *by_of_col;        /* block of each lat row / lon column */
    int64_t *blk_off;
    int32_t *blk_obs;
    int *slot_off;
    int32_t *slot_blk;
} obs_index;

static void decomp_build(const orc_config *cfg, const orc_obs *obs, obs_index *ix);

static void obs_index_build(const orc_config *cfg, const orc_obs *obs, obs_index *ix)
{
    int64_t o;
    ix->n = obs->nobs;
    ix->keys = (lat_key *)malloc(sizeof(lat_key) * (obs->nobs > 0 ? obs->nobs : 1));
    ix->s = (double *)malloc(sizeof(double) * (obs->nobs > 0 ? obs->nobs : 1));
    ix->c = (double *)malloc(sizeof(double) * (obs->nobs > 0 ? obs->nobs : 1));
    ix->yr = (double *)malloc(sizeof(double) * (obs->nobs > 0 ? obs->nobs : 1));
    for (o = 0; o < obs->nobs; o++) {
        double xr = lat_rad(obs->lat[o]);
        ix->keys[o].lat = obs->lat[o];
        ix->keys[o].idx = (int32_t)o;
        ix->s[o] = sin(xr);
        ix->c[o] = cos(xr);
        ix->yr[o] = lat_rad(obs->lon[o]);
    }
    qsort(ix->keys, (size_t)obs->nobs, sizeof(lat_key), cmp_lat);
    ix->nbx = ix->nby = 0;
    ix->bx_of_row = ix->by_of_col = NULL;
    ix->blk_off = NULL;
    ix->blk_obs = NULL;
    ix->slot_off = NULL;
    ix->slot_blk = NULL;
    if (cfg->dec_lat_blocks > 0 && cfg->dec_lon_blocks > 0) decomp_build(cfg, obs, ix);
}

static void obs_index_free(obs_index *ix)
{
    free(ix->keys);
    free(ix->s);
    free(ix->c);
    free(ix->yr);
    free(ix->bx_of_row);
    free(ix->by_of_col);
    free(ix->blk_off);
    free(ix->blk_obs);
    free(ix->slot_off);
    free(ix->slot_blk);
}

static int64_t lower_bound_lat(const obs_index *ix, double lat)
{
    int64_t lo = 0, hi = ix->n;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (ix->keys[mid].lat < lat) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* gen_yb_dis selection (DA/LETKF/src/letkf_yb.F90:71-133), for one logical
 * block that holds every obs once: scan obs in index order, keep those with
 * |lat| <= obs_polar and gc > 0, stop at MAX_OBS.
 *
 * The scan visits only a superset of the obs that can pass: those within the
 * latitude band |lat - clat| <= 2c/a (+1e-6 rad) and, where the cap holds no
 * pole, the longitude band |dlon| <= asin(sin(2c/a)/cos(clat)) (+1e-6 rad); and
 * those within 1e-6 rad of the antipode's latitude, where rounding can push
 * the cosine below -1 so that acos returns NaN and schr2(NaN) = 1 keeps the
 * obs.  Every other obs has a computed distance well above 2c.              */
static int local_point(const orc_config *cfg, const orc_obs *obs, const obs_index *ix,
                       double clat, double clon, int32_t *idx, double *rloc,
                       int32_t *cand_buf)
{
    const double deg = 180.0 / M_PI;
    double theta = 2.0 * cfg->local_dist / ORC_EARTH_A;
    double band = (theta + 1e-6) * deg;
    double s2 = sin(lat_rad(clat)), c2 = cos(lat_rad(clat)), y2r = lat_rad(clon);
    double clat_r = clat / deg;
    int use_lon = 0;
    double dlon_max = 0.0;
    int64_t a, b, m;
    int ncand = 0, nobsl = 0, i;

    if (fabs(clat_r) + theta + 1e-6 < M_PI / 2 - 1e-6) {
        double sv = sin(theta) / cos(fabs(clat_r) + 0.0);
        if (sv < 1.0) {
            use_lon = 1;
            dlon_max = (asin(sv) + 1e-6) * deg;
        }
    }
    a = lower_bound_lat(ix, clat - band);
    b = lower_bound_lat(ix, clat + band + 1e-12);
    for (m = a; m < b && m < ix->n; m++) {
        int32_t o = ix->keys[m].idx;
        if (ix->keys[m].lat > clat + band) break;
        if (use_lon) {
            double d = fabs(obs->lon[o] - clon);
            if (d > 180.0) d = 360.0 - d;
            if (d > dlon_max) continue;
        }
        cand_buf[ncand++] = o;
    }
    /* antipodal latitude band */
    {
        double alat = -clat, aband = 1e-6 * deg;
        int64_t a2 = lower_bound_lat(ix, alat - aband);
        for (m = a2; m < ix->n && ix->keys[m].lat <= alat + aband; m++) {
            cand_buf[ncand++] = ix->keys[m].idx;
        }
    }
    qsort(cand_buf, (size_t)ncand, sizeof(int32_t), cmp_i32);
    /* drop duplicates (an obs seen from both bands) */
    {
        int w = 0;
        for (i = 0; i < ncand; i++)
            if (w == 0 || cand_buf[i] != cand_buf[w - 1]) cand_buf[w++] = cand_buf[i];
        ncand = w;
    }
    for (i = 0; i < ncand; i++) {
        int32_t o = cand_buf[i];
        double dist, gc;
        if (!(fabs(obs->lat[o]) <= cfg->obs_polar)) continue;
        dist = dist_pre(ix->s[o], ix->c[o], ix->yr[o], s2, c2, y2r);
        gc = cfg->gc_filter ? orc_schr2(dist * 1.0 / cfg->local_dist)
                            : orc_schr(dist * 1.0 / cfg->local_dist);
        if (gc > 0 || gc != gc) {
            if (idx) idx[nobsl] = o;
            if (rloc) rloc[nobsl] = gc;
            nobsl++;
            if (nobsl >= cfg->max_obs) break;
        }
    }
    return nobsl;
}


/* ---- decomposed observation sets --------------------------------------- */

int orc_decomp_dims(int nranks, int *lat_blocks, int *lon_blocks)
{
    int b, best = 1;
    if (nranks < 1) return -1;
    for (b = 1; (int64_t)b * b <= nranks; b++)
        if (nranks % b == 0) best = b;
    *lon_blocks = nranks / best;     /* dims(1) >= dims(2) */
    *lat_blocks = best;
    return 0;
}

/* pro_info_get_indx (DA/utils/pro_info.F90:96-125) along one axis: 1-based
 * inclusive index range of block b (1-based) of n points in nb blocks, the
 * first n mod nb blocks one point longer.                                   */
static void block_range(int n, int nb, int b, int *s, int *e)
{
    int sec = n / nb, res = n % nb;
    if (b - 1 < res) {
        *s = (b - 1) * (sec + 1) + 1;
        *e = *s + sec;
    } else {
        *s = (b - 1) * sec + res + 1;
        *e = *s + sec - 1;
    }
}

/* latlon_dist_r4, DA/utils/pro_info.F90:163-175: the distance in default
 * (single) precision, with float pi and Earth radius.                       */
static float latlon_dist_f32(float x1, float y1, float x2, float y2)
{
    const float pi = atanf(1.0f) * 4.0f, a = 6371.393f;
    float v = cosf(x1 / 180.0f * pi) * cosf(x2 / 180.0f * pi) * cosf(y1 / 180.0f * pi - y2 / 180.0f * pi) +
              sinf(x1 / 180.0f * pi) * sinf(x2 / 180.0f * pi);
    if (v > 1.0f) v = 1.0f;
    return a * acosf(v);
}

/* nearest_dist, DA/LETKF/src/letkf_init.F90:293-341 (1-based blocks). */
static double nearest_dist(const orc_config *cfg, int bx1, int by1, int bx2, int by2)
{
    const int NX = cfg->dec_lat_blocks, NY = cfg->dec_lon_blocks;
    int xs1, xe1, ys1, ye1, xs2, xe2, ys2, ye2, tx1, tx2;
    float lat1, lat2;
    block_range(cfg->nlat, NX, bx1, &xs1, &xe1);
    block_range(cfg->nlon, NY, by1, &ys1, &ye1);
    block_range(cfg->nlat, NX, bx2, &xs2, &xe2);
    block_range(cfg->nlon, NY, by2, &ys2, &ye2);
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
    lat1 = glat_ext(cfg, tx1);
    lat2 = glat_ext(cfg, tx2);
    if (fabs((double)lat1) > cfg->obs_polar) lat1 = (float)(lat1 < 0 ? -cfg->obs_polar : cfg->obs_polar);
    if (fabs((double)lat2) > cfg->obs_polar) lat2 = (float)(lat2 < 0 ? -cfg->obs_polar : cfg->obs_polar);
    if (by1 == by2)
        return (double)latlon_dist_f32(lat1, glon_ext(cfg, ys1), lat2, glon_ext(cfg, ys2));
    {
        float d1 = latlon_dist_f32(lat1, glon_ext(cfg, ys1), lat2, glon_ext(cfg, ye2 % cfg->nlon + 1));
        float d2 = latlon_dist_f32(lat1, glon_ext(cfg, ye1 % cfg->nlon + 1), lat2, glon_ext(cfg, ys2));
        return (double)(d1 < d2 ? d1 : d2);
    }
}

/* comm_info_init, DA/LETKF/src/letkf_init.F90:100-291: the blocks whose obs
 * a block's columns scan, in the order gen_yb_dis visits them (lat offsets
 * -north_n..south_n, then lon offsets -west_n..east_n, wrapping in longitude).
 * Blocks are compared against local_dist itself (the cut-off is 2 local_dist),
 * as the reference does.                                                    */
int orc_block_slots(const orc_config *cfg, int bx0, int by0, int32_t *blocks, int cap)
{
    const int NX = cfg->dec_lat_blocks, NY = cfg->dec_lon_blocks;
    const int bx = bx0 + 1, by = by0 + 1;
    int s_lat, e_lat, s_lon, e_lon, tx_s, tx_e, north_n = 0, south_n = 0, i, n = 0;
    double x1, y1, x2, y2;
    block_range(cfg->nlat, NX, bx, &s_lat, &e_lat);
    block_range(cfg->nlon, NY, by, &s_lon, &e_lon);
    x1 = glat_ext(cfg, s_lat);
    y1 = glon_ext(cfg, s_lon);
    y2 = y1;
    for (i = bx - 1; i > 0; i--) {
        block_range(cfg->nlat, NX, i, &tx_s, &tx_e);
        x2 = glat_ext(cfg, tx_e + 1);
        if (orc_latlon_dist(x1, y1, x2, y2) > cfg->local_dist) break;
        north_n++;
    }
    x1 = glat_ext(cfg, e_lat + 1);
    for (i = bx + 1; i <= NX; i++) {
        block_range(cfg->nlat, NX, i, &tx_s, &tx_e);
        x2 = glat_ext(cfg, tx_s);
        if (orc_latlon_dist(x1, y1, x2, y2) > cfg->local_dist) break;
        south_n++;
    }
    for (i = -north_n; i <= south_n; i++) {
        const int tbx = bx + i;
        int west = 0, east = 0, tby, j;
        tby = by;
        while (west <= (NY - 1) / 2) {
            tby = (tby + NY - 2) % NY + 1;
            if (nearest_dist(cfg, bx, by, tbx, tby) > cfg->local_dist) break;
            west++;
        }
        tby = by;
        while (east <= (NY - 1) / 2) {
            tby = tby % NY + 1;
            if (nearest_dist(cfg, bx, by, tbx, tby) > cfg->local_dist) break;
            east++;
        }
        if (west + east > NY - 1) east--;
        for (j = -west; j <= east; j++) {
            const int lb = ((by - 1 + j) % NY + NY) % NY;
            if (n < cap) blocks[n] = (int32_t)((tbx - 1) * NY + lb);
            n++;
        }
    }
    return n;
}

/* A block's box bound as the obs store's range query sees it: the float grid
 * coordinate printed with five decimals ("%.5f", LIB/REDIS/src/
 * redis_wrapper.c:4097-4117) and read back.                                 */
static double box_bound(float v)
{
    char buf[64];
    snprintf(buf, sizeof buf, "%.5f", (double)v);
    return strtod(buf, NULL);
}

/* Obs of each block: inside the closed box [grid_lat(s), grid_lat(e+1)] x
 * [grid_lon(s), grid_lon(e+1)] of the block (allocate_obslist / read_obs,
 * DA/LETKF/src/read_obs_mod.F90:73-165,338-449, called from
 * letkf_obs.F90:45-90), in ascending index order (the store's range query
 * returns sorted ids).  An obs on a shared edge belongs to both blocks; one
 * outside every box (south of the first row or west of the first column of
 * centres) to none.                                                          */
static void decomp_build(const orc_config *cfg, const orc_obs *obs, obs_index *ix)
{
    const int NX = cfg->dec_lat_blocks, NY = cfg->dec_lon_blocks, nb = NX * NY;
    double *la0 = (double *)malloc(sizeof(double) * NX), *la1 = (double *)malloc(sizeof(double) * NX);
    double *lo0 = (double *)malloc(sizeof(double) * NY), *lo1 = (double *)malloc(sizeof(double) * NY);
    int64_t *cnt = (int64_t *)calloc((size_t)nb + 1, sizeof(int64_t));
    int b, s, e, i, cap;
    int64_t o;
    ix->nbx = NX;
    ix->nby = NY;
    ix->bx_of_row = (int *)malloc(sizeof(int) * cfg->nlat);
    ix->by_of_col = (int *)malloc(sizeof(int) * cfg->nlon);
    for (b = 0; b < NX; b++) {
        block_range(cfg->nlat, NX, b + 1, &s, &e);
        la0[b] = box_bound(glat_ext(cfg, s));
        la1[b] = box_bound(glat_ext(cfg, e + 1));
        for (i = s; i <= e; i++) ix->bx_of_row[i - 1] = b;
    }
    for (b = 0; b < NY; b++) {
        block_range(cfg->nlon, NY, b + 1, &s, &e);
        lo0[b] = box_bound(glon_ext(cfg, s));
        lo1[b] = box_bound(glon_ext(cfg, e + 1));
        for (i = s; i <= e; i++) ix->by_of_col[i - 1] = b;
    }
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            ix->blk_off = (int64_t *)malloc(sizeof(int64_t) * (nb + 1));
            ix->blk_off[0] = 0;
            for (b = 0; b < nb; b++) ix->blk_off[b + 1] = ix->blk_off[b] + cnt[b];
            ix->blk_obs = (int32_t *)malloc(sizeof(int32_t) * (ix->blk_off[nb] + 1));
            memset(cnt, 0, sizeof(int64_t) * (nb + 1));
        }
        for (o = 0; o < obs->nobs; o++) {
            int bxa, bya;
            for (bxa = 0; bxa < NX; bxa++) {
                if (!(obs->lat[o] >= la0[bxa] && obs->lat[o] <= la1[bxa])) continue;
                for (bya = 0; bya < NY; bya++) {
                    if (!(obs->lon[o] >= lo0[bya] && obs->lon[o] <= lo1[bya])) continue;
                    b = bxa * NY + bya;
                    if (pass == 1) ix->blk_obs[ix->blk_off[b] + cnt[b]] = (int32_t)o;
                    cnt[b]++;
                }
            }
        }
    }
    cap = 2 * nb + 2;
    ix->slot_off = (int *)malloc(sizeof(int) * (nb + 1));
    ix->slot_blk = (int32_t *)malloc(sizeof(int32_t) * (size_t)nb * cap);
    ix->slot_off[0] = 0;
    for (b = 0; b < nb; b++) {
        int ns = orc_block_slots(cfg, b / NY, b % NY, ix->slot_blk + ix->slot_off[b], cap);
        if (ns > cap) ns = cap;
        ix->slot_off[b + 1] = ix->slot_off[b] + ns;
    }
    free(la0); free(la1); free(lo0); free(lo1); free(cnt);
}

/* gen_yb_dis over the neighbour blocks of block b (letkf_yb.F90:71-133). */
static int local_point_dec(const orc_config *cfg, const orc_obs *obs, const obs_index *ix, int b,
                           double clat, double clon, int32_t *idx, double *rloc)
{
    double s2 = sin(lat_rad(clat)), c2 = cos(lat_rad(clat)), y2r = lat_rad(clon);
    int nobsl = 0, sl;
    for (sl = ix->slot_off[b]; sl < ix->slot_off[b + 1]; sl++) {
        const int32_t blk = ix->slot_blk[sl];
        int64_t m;
        for (m = ix->blk_off[blk]; m < ix->blk_off[blk + 1]; m++) {
            const int32_t o = ix->blk_obs[m];
            double dist, gc;
            if (!(fabs(obs->lat[o]) <= cfg->obs_polar)) continue;
            dist = dist_pre(ix->s[o], ix->c[o], ix->yr[o], s2, c2, y2r);
            gc = cfg->gc_filter ? orc_schr2(dist * 1.0 / cfg->local_dist)
                                : orc_schr(dist * 1.0 / cfg->local_dist);
            if (gc > 0 || gc != gc) {
                if (idx) idx[nobsl] = o;
                if (rloc) rloc[nobsl] = gc;
                nobsl++;
                if (nobsl >= cfg->max_obs) return nobsl;
            }
        }
    }
    return nobsl;
}

/* Local list of the cube (sj..ej, si..ei) in either obs-set mode. */
static int cube_list(const orc_config *cfg, const orc_obs *obs, const obs_index *ix,
                     int sj, int ej, int si, int ei, int32_t *idx, double *rloc, int32_t *buf)
{
    double clat, clon;
    orc_cube_center(cfg, sj, ej, si, ei, &clat, &clon);
    if (ix->nbx > 0)
        return local_point_dec(cfg, obs, ix, ix->bx_of_row[sj] * ix->nby + ix->by_of_col[si], clat,
                               clon, idx, rloc);
    return local_point(cfg, obs, ix, clat, clon, idx, rloc, buf);
}

int orc_local_obs_point(const orc_config *cfg, const orc_obs *obs, double clat, double clon,
                        int32_t *idx, double *rloc)
{
    obs_index ix;
    int32_t *buf;
    int n;
    obs_index_build(cfg, obs, &ix);
    buf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
    n = local_point(cfg, obs, &ix, clat, clon, idx, rloc, buf);
    free(buf);
    obs_index_free(&ix);
    return n;
}

int64_t orc_local_obs(const orc_config *cfg, const orc_obs *obs,
                      int64_t *offsets, int32_t *idx, double *rloc, int64_t cap)
{
    int64_t nc = orc_num_cubes(cfg), c, total;
    obs_index ix;
    obs_index_build(cfg, obs, &ix);
#pragma omp parallel
    {
        int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
#pragma omp for schedule(dynamic, 16)
        for (c = 0; c < nc; c++) {
            int sj, ej, si, ei;
            orc_cube_bounds(cfg, c, &sj, &ej, &si, &ei);
            offsets[c + 1] = cube_list(cfg, obs, &ix, sj, ej, si, ei, NULL, NULL, buf);
        }
        free(buf);
    }
    offsets[0] = 0;
    for (c = 0; c < nc; c++) offsets[c + 1] += offsets[c];
    total = offsets[nc];
    if (idx != NULL) {
        if (total > cap) {
            obs_index_free(&ix);
            return -1;
        }
#pragma omp parallel
        {
            int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
#pragma omp for schedule(dynamic, 16)
            for (c = 0; c < nc; c++) {
                int sj, ej, si, ei;
                orc_cube_bounds(cfg, c, &sj, &ej, &si, &ei);
                cube_list(cfg, obs, &ix, sj, ej, si, ei, idx + offsets[c],
                          rloc ? rloc + offsets[c] : NULL, buf);
            }
            free(buf);
        }
    }
    obs_index_free(&ix);
    return total;
}

/* The lists of the selected cubes only (same selection and order as
 * orc_local_obs, letkf_yb.F90:3-133), packed in the order of `cubes`:
 * offsets[n + 1]; idx/rloc may be NULL for counts only.  The observation
 * index is built once for all of them.  Returns the total, or -1 when it
 * exceeds cap.                                                              */
int64_t orc_local_obs_cubes(const orc_config *cfg, const orc_obs *obs, int64_t n, const int64_t *cubes,
                            int64_t *offsets, int32_t *idx, double *rloc, int64_t cap)
{
    int64_t i, total;
    obs_index ix;
    obs_index_build(cfg, obs, &ix);
#pragma omp parallel
    {
        int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
#pragma omp for schedule(dynamic, 4)
        for (i = 0; i < n; i++) {
            int sj, ej, si, ei;
            orc_cube_bounds(cfg, cubes[i], &sj, &ej, &si, &ei);
            offsets[i + 1] = cube_list(cfg, obs, &ix, sj, ej, si, ei, NULL, NULL, buf);
        }
        free(buf);
    }
    offsets[0] = 0;
    for (i = 0; i < n; i++) offsets[i + 1] += offsets[i];
    total = offsets[n];
    if (idx != NULL) {
        if (total > cap) {
            obs_index_free(&ix);
            return -1;
        }
#pragma omp parallel
        {
            int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
#pragma omp for schedule(dynamic, 4)
            for (i = 0; i < n; i++) {
                int sj, ej, si, ei;
                orc_cube_bounds(cfg, cubes[i], &sj, &ej, &si, &ei);
                cube_list(cfg, obs, &ix, sj, ej, si, ei, idx + offsets[i], rloc ? rloc + offsets[i] : NULL,
                          buf);
            }
            free(buf);
        }
    }
    obs_index_free(&ix);
    return total;
}

/* ---- eigensolver --------------------------------------------------------- */

/* Cyclic Jacobi for a symmetric matrix (Golub & Van Loan, Alg. 8.5.3, with
 * the rotation of sym.schur2).  a is column-major k x k.  Stops after a sweep
 * in which every off-diagonal element was below 1e-18*sqrt(|a_pp a_qq|) or an
 * absolute floor of 1e-300.  Eigenvalues are returned ascending (the order of
 * dsyevd), with the vectors permuted alike.                                  */
int orc_jacobi_eig(int k, double *a, double *lam, double *v, int max_sweeps)
{
    int sweep, p, q, r, i;
#define A(i, j) a[(i) + (int64_t)k * (j)]
#define VV(i, j) v[(i) + (int64_t)k * (j)]
    for (i = 0; i < k * k; i++) v[i] = 0.0;
    for (i = 0; i < k; i++) VV(i, i) = 1.0;
    for (sweep = 1; sweep <= max_sweeps; sweep++) {
        int rotated = 0;
        for (p = 0; p < k - 1; p++) {
            for (q = p + 1; q < k; q++) {
                double apq = A(p, q), app = A(p, p), aqq = A(q, q);
                double tau, t, c, s;
                if (fabs(apq) <= 1e-18 * sqrt(fabs(app * aqq)) || fabs(apq) < 1e-300) {
                    A(p, q) = 0.0;
                    A(q, p) = 0.0;
                    continue;
                }
                rotated = 1;
                tau = (aqq - app) / (2.0 * apq);
                if (tau >= 0)
                    t = 1.0 / (tau + sqrt(1.0 + tau * tau));
                else
                    t = -1.0 / (-tau + sqrt(1.0 + tau * tau));
                c = 1.0 / sqrt(1.0 + t * t);
                s = t * c;
                for (r = 0; r < k; r++) {
                    double arp = A(r, p), arq = A(r, q);
                    A(r, p) = c * arp - s * arq;
                    A(r, q) = s * arp + c * arq;
                }
                for (r = 0; r < k; r++) {
                    double apr = A(p, r), aqr = A(q, r);
                    A(p, r) = c * apr - s * aqr;
                    A(q, r) = s * apr + c * aqr;
                }
                A(p, q) = 0.0;
                A(q, p) = 0.0;
                for (r = 0; r < k; r++) {
                    double vrp = VV(r, p), vrq = VV(r, q);
                    VV(r, p) = c * vrp - s * vrq;
                    VV(r, q) = s * vrp + c * vrq;
                }
            }
        }
        if (!rotated) break;
    }
    for (i = 0; i < k; i++) lam[i] = A(i, i);
    /* insertion sort, ascending */
    for (i = 1; i < k; i++) {
        int j = i;
        while (j > 0 && lam[j - 1] > lam[j]) {
            double t = lam[j]; lam[j] = lam[j - 1]; lam[j - 1] = t;
            for (r = 0; r < k; r++) {
                double tv = VV(r, j); VV(r, j) = VV(r, j - 1); VV(r, j - 1) = tv;
            }
            j--;
        }
    }
#undef A
#undef VV
    return (sweep > max_sweeps) ? -1 : sweep;
}

/* ---- letkf_core ---------------------------------------------------------- */

/* letkf_core, DA/LETKF/src/letkf_core.F90:14-233, step by step:
 *   hxens * sqrt(rdiaginv*rloc)                                   (:58-69)
 *   work1 = hxens hxens^T  (full k x k, as the dgemm)             (:74)
 *   eig(work1), eival += (k-1)/inflation                          (:98-113)
 *   pa = V diag(1/eival) V^T                                      (:129-143)
 *   hxens * sqrt(rdiaginv*rloc) once more                         (:146-148)
 *   work2 = pa hxens;  w = work2 dep                              (:164-195)
 *   trans = V diag(sqrt((k-1)/eival)) V^T + w 1^T                 (:198-225)
 * hxens is [obs][k] (member fastest), trans column-major.                    */
int orc_letkf_core(int k, int p, const double *hxens, const float *rdiaginv,
                   const double *dep, const double *rloc, double inflation,
                   double *trans, double *w)
{
    int i, j, l, o, sweeps;
    double *hx = (double *)malloc(sizeof(double) * ((int64_t)p * k + 1));
    double *rr = (double *)malloc(sizeof(double) * (p + 1));
    double *work1 = (double *)malloc(sizeof(double) * k * k);
    double *eivec = (double *)malloc(sizeof(double) * k * k);
    double *pa = (double *)malloc(sizeof(double) * k * k);
    double *eival = (double *)malloc(sizeof(double) * k);
    double *v = (double *)malloc(sizeof(double) * k * k);
    double *work2 = (double *)malloc(sizeof(double) * ((int64_t)p * k + 1));

    for (o = 0; o < p; o++) {
        rr[o] = (double)rdiaginv[o] * rloc[o];
        rr[o] = sqrt(rr[o]);
        for (i = 0; i < k; i++) hx[(int64_t)o * k + i] = hxens[(int64_t)o * k + i] * rr[o];
    }
    for (j = 0; j < k; j++)
        for (i = 0; i < k; i++) {
            double s = 0.0;
            for (o = 0; o < p; o++) s = s + hx[(int64_t)o * k + i] * hx[(int64_t)o * k + j];
            work1[i + k * j] = s;
        }
    sweeps = orc_jacobi_eig(k, work1, eival, v, 100);
    for (i = 0; i < k * k; i++) work1[i] = v[i];
    for (j = 0; j < k; j++) eival[j] = eival[j] * 1.0 + (double)(k - 1) / inflation;

    for (j = 0; j < k; j++)
        for (i = 0; i < k; i++) {
            eivec[i + k * j] = work1[i + k * j];
            work1[i + k * j] = work1[i + k * j] / eival[j];
        }
    for (j = 0; j < k; j++)
        for (i = 0; i < k; i++) {
            double s = 0.0;
            for (l = 0; l < k; l++) s = s + work1[i + k * l] * eivec[j + k * l];
            pa[i + k * j] = s;
        }
    for (o = 0; o < p; o++)
        for (i = 0; i < k; i++) hx[(int64_t)o * k + i] = hx[(int64_t)o * k + i] * rr[o];
    for (o = 0; o < p; o++)
        for (i = 0; i < k; i++) {
            double s = 0.0;
            for (l = 0; l < k; l++) s = s + pa[i + k * l] * hx[(int64_t)o * k + l];
            work2[i + (int64_t)k * o] = s;
        }
    for (i = 0; i < k; i++) w[i] = 0.0;
    for (o = 0; o < p; o++)
        for (i = 0; i < k; i++) w[i] = w[i] + work2[i + (int64_t)k * o] * dep[o];
    for (j = 0; j < k; j++) {
        double rho = sqrt((double)(k - 1) / eival[j]);
        for (i = 0; i < k; i++) work1[i + k * j] = eivec[i + k * j] * rho;
    }
    for (j = 0; j < k; j++)
        for (i = 0; i < k; i++) {
            double s = 0.0;
            for (l = 0; l < k; l++) s = s + work1[i + k * l] * eivec[j + k * l];
            trans[i + k * j] = s;
        }
    for (j = 0; j < k; j++)
        for (i = 0; i < k; i++) trans[i + k * j] = trans[i + k * j] + w[i];

    free(hx); free(rr); free(work1); free(eivec); free(pa); free(eival); free(v); free(work2);
    return sweeps < 0 ? -1 : 0;
}

/* ---- update -------------------------------------------------------------- */

/* xb_2_xa for one column, DA/LETKF/src/letkf_compute.F90:231-301:
 * xa = trans^T xb (+ axb), then the analysis mean is recomputed and removed. */
static void xb_2_xa_col(int k, int n, const double *trans, const double *xb,
                        const double *axb, double *xa, double *axa)
{
    int r, e, i;
    for (r = 0; r < n; r++) {
        const double *x = xb + (int64_t)r * k;
        double *y = xa + (int64_t)r * k;
        double m = 0.0;
        for (e = 0; e < k; e++) {
            double s = 0.0;
            for (i = 0; i < k; i++) s = s + trans[i + k * e] * x[i];
            y[e] = s;
        }
        for (e = 0; e < k; e++) y[e] = y[e] + axb[r];
        for (e = 0; e < k; e++) m = m + y[e];
        m = m / k;
        axa[r] = m;
        for (e = 0; e < k; e++) y[e] = y[e] - m;
    }
}

/* Gather of gen_yb_dis (letkf_yb.F90:98-106): yb, dis, rdiaginv (real(4)), rloc. */
static void gather_local(int k, int p, const int32_t *idx, const double *yb, const double *dep,
                         const orc_obs *obs, double *hx, float *rdi, double *dis)
{
    int o;
    for (o = 0; o < p; o++) {
        int32_t g = idx[o];
        memcpy(hx + (int64_t)o * k, yb + (int64_t)g * k, sizeof(double) * k);
        dis[o] = dep[g];
        rdi[o] = (float)obs->rinv[g];
    }
}

static void cube_core(const orc_config *cfg, const orc_obs *obs, const obs_index *ix,
                      const double *yb, const double *dep, int64_t cube,
                      int32_t *cbuf, int32_t *idx, double *rl, double *hx, float *rdi,
                      double *dis, double *trans, double *w, int *fail)
{
    int sj, ej, si, ei, p;
    orc_cube_bounds(cfg, cube, &sj, &ej, &si, &ei);
    p = cube_list(cfg, obs, ix, sj, ej, si, ei, idx, rl, cbuf);
    gather_local(cfg->k, p, idx, yb, dep, obs, hx, rdi, dis);
    if (orc_letkf_core(cfg->k, p, hx, rdi, dis, rl, cfg->inflation, trans, w) != 0) *fail = 1;
}

int orc_letkf_cubes(const orc_config *cfg, const orc_obs *obs, const double *yb,
                    const double *dep, const double *xb, const double *axb,
                    double *xa, double *axa, const int64_t *cubes, int64_t ncubes)
{
    const int k = cfg->k, n = state_rows(cfg);
    int64_t t;
    int fail = 0;
    obs_index ix;
    obs_index_build(cfg, obs, &ix);
#pragma omp parallel reduction(| : fail)
    {
        int mo = cfg->max_obs;
        int32_t *cbuf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
        int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * mo);
        double *rl = (double *)malloc(sizeof(double) * mo);
        double *hx = (double *)malloc(sizeof(double) * (int64_t)mo * k);
        float *rdi = (float *)malloc(sizeof(float) * mo);
        double *dis = (double *)malloc(sizeof(double) * mo);
        double *trans = (double *)malloc(sizeof(double) * k * k);
        double *w = (double *)malloc(sizeof(double) * k);
#pragma omp for schedule(dynamic, 4)
        for (t = 0; t < ncubes; t++) {
            int sj, ej, si, ei, jj, ii;
            int64_t cube = cubes ? cubes[t] : t;
            cube_core(cfg, obs, &ix, yb, dep, cube, cbuf, idx, rl, hx, rdi, dis, trans, w, &fail);
            orc_cube_bounds(cfg, cube, &sj, &ej, &si, &ei);
            for (ii = si; ii <= ei; ii++)
                for (jj = sj; jj <= ej; jj++) {
                    int64_t c = jj + (int64_t)cfg->nlat * ii;
                    xb_2_xa_col(k, n, trans, xb + c * n * k, axb + c * n, xa + c * n * k, axa + c * n);
                }
        }
        free(cbuf); free(idx); free(rl); free(hx); free(rdi); free(dis); free(trans); free(w);
    }
    obs_index_free(&ix);
    return fail ? -1 : 0;
}

/* Vertical-localization column loop: letkf_compute_nooverlap_vertical,
 * DA/LETKF/src/letkf_compute.F90:358-526, with gen_yb_dis_vertical
 * (letkf_yb.F90:137-221), vertical_localization (:223-243) and ps2alnp
 * (obs_make.F90:418-437).  ps2alnp reads interface pressure nz+1 without
 * setting it; here it is the surface interface hyai(nz+1), hybi(nz+1).       */
static int run_vertical(const orc_config *cfg, const orc_obs *obs, const double *yb,
                        const double *dep, const double *xb, const double *axb,
                        double *xa, double *axa)
{
    const int k = cfg->k, n = state_rows(cfg), nz = cfg->nz;
    int64_t nc = orc_num_cubes(cfg), cube, c;
    int fail = 0;
    obs_index ix;
    obs_index_build(cfg, obs, &ix);
#pragma omp parallel reduction(| : fail)
    {
        int mo = cfg->max_obs;
        int32_t *cbuf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
        int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * mo);
        double *rlh = (double *)malloc(sizeof(double) * mo);
        double *rl = (double *)malloc(sizeof(double) * mo);
        double *lnp = (double *)malloc(sizeof(double) * mo);
        double *hx = (double *)malloc(sizeof(double) * (int64_t)mo * k);
        float *rdi = (float *)malloc(sizeof(float) * mo);
        double *dis = (double *)malloc(sizeof(double) * mo);
        double *trans = (double *)malloc(sizeof(double) * k * k);
        double *w = (double *)malloc(sizeof(double) * k);
        double *alnp = (double *)malloc(sizeof(double) * nz);
#pragma omp for schedule(dynamic, 4)
        for (cube = 0; cube < nc; cube++) {
            int sj, ej, si, ei, p, o, kk, v, ii, jj;
            double ps;
            orc_cube_bounds(cfg, cube, &sj, &ej, &si, &ei);
            p = cube_list(cfg, obs, &ix, sj, ej, si, ei, idx, rlh, cbuf);
            gather_local(k, p, idx, yb, dep, obs, hx, rdi, dis);
            for (o = 0; o < p; o++) lnp[o] = log(obs->ph[idx[o]]);
            {
                int cj = ((sj + 1) + (ej + 1)) / 2 - 1, ci = ((si + 1) + (ei + 1)) / 2 - 1;
                int64_t cc = cj + (int64_t)cfg->nlat * ci;
                ps = axb[cc * n + cfg->ps_row];
            }
            for (kk = 0; kk < nz; kk++)
                alnp[kk] = log(0.5 * (ph_lev(cfg, kk, ps) + ph_lev(cfg, kk + 1, ps)));
            for (kk = 0; kk < nz; kk += cfg->cube_nz) {
                int sk = kk, ek = kk + cfg->cube_nz - 1, ck;
                if (ek > nz - 1) ek = nz - 1;
                ck = ((sk + 1) + (ek + 1)) / 2 - 1;
                for (o = 0; o < p; o++) {
                    double z = fabs(alnp[ck] - lnp[o]) / cfg->vert_dist;
                    rl[o] = rlh[o] * (cfg->gc_filter_vertical ? orc_schr2(z) : orc_schr(z));
                }
                if (orc_letkf_core(k, p, hx, rdi, dis, rl, cfg->inflation, trans, w) != 0) fail = 1;
                for (v = 0; v < cfg->nvar2d + cfg->nvar3d; v++) {
                    int r0, r1, r, e, i;
                    if (v < cfg->nvar2d) {
                        if (ek != nz - 1) continue;
                        r0 = r1 = var_start(cfg, v);
                    } else {
                        r0 = var_start(cfg, v) + sk;
                        r1 = var_start(cfg, v) + ek;
                    }
                    for (ii = si; ii <= ei; ii++)
                        for (jj = sj; jj <= ej; jj++) {
                            int64_t cc = jj + (int64_t)cfg->nlat * ii;
                            for (r = r0; r <= r1; r++) {
                                const double *x = xb + (cc * n + r) * k;
                                for (e = 0; e < k; e++) {
                                    double s = 0.0;
                                    for (i = 0; i < k; i++) s = s + x[i] * trans[i + k * e];
                                    xa[(cc * n + r) * k + e] = axb[cc * n + r] + s;
                                }
                            }
                        }
                }
            }
        }
        free(cbuf); free(idx); free(rlh); free(rl); free(lnp); free(hx); free(rdi);
        free(dis); free(trans); free(w); free(alnp);
    }
    obs_index_free(&ix);
    /* mean recompute over every column (letkf_compute.F90:511-524) */
    nc = (int64_t)cfg->nlat * cfg->nlon;
#pragma omp parallel for schedule(static)
    for (c = 0; c < nc; c++) {
        int r, e;
        for (r = 0; r < n; r++) {
            double *y = xa + (c * n + r) * k, m = 0.0;
            for (e = 0; e < k; e++) m = m + y[e];
            m = m / k;
            axa[c * n + r] = m;
            for (e = 0; e < k; e++) y[e] = y[e] - m;
        }
    }
    return fail ? -1 : 0;
}

/* Overlapped cubes: letkf_compute + xb_add2_xa, DA/LETKF/src/letkf_compute.F90:128-228
 * and :304-354.  Cubes start every cube_n - overlap points; each column's
 * analysis is the average over the cubes that cover it.                     */
static int run_overlap(const orc_config *cfg, const orc_obs *obs, const double *yb,
                       const double *dep, const double *xb, const double *axb,
                       double *xa, double *axa)
{
    const int k = cfg->k, n = state_rows(cfg);
    const int step = cfg->cube_n - cfg->overlap;
    int64_t ncol = (int64_t)cfg->nlat * cfg->nlon, c;
    double *count;
    int mo = cfg->max_obs, fail = 0, i, j;
    int32_t *cbuf = (int32_t *)malloc(sizeof(int32_t) * (obs->nobs + 1));
    int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * mo);
    double *rl = (double *)malloc(sizeof(double) * mo);
    double *hx = (double *)malloc(sizeof(double) * (int64_t)mo * k);
    float *rdi = (float *)malloc(sizeof(float) * mo);
    double *dis = (double *)malloc(sizeof(double) * mo);
    double *trans = (double *)malloc(sizeof(double) * k * k);
    double *w = (double *)malloc(sizeof(double) * k);
    double *dist = (double *)malloc(sizeof(double) * k);
    obs_index ix;
    if (step <= 0) return -2;
    count = (double *)calloc((size_t)ncol, sizeof(double));
    obs_index_build(cfg, obs, &ix);
    memset(xa, 0, sizeof(double) * ncol * n * k);
    memset(axa, 0, sizeof(double) * ncol * n);
    for (i = 0; i < cfg->nlon; i += step) {
        int si = i, ei = i + cfg->cube_n - 1;
        if (ei > cfg->nlon - 1) ei = cfg->nlon - 1;
        for (j = 0; j < cfg->nlat; j += step) {
            int sj = j, ej = j + cfg->cube_n - 1, p, ii, jj;
            double clat, clon;
            if (ej > cfg->nlat - 1) ej = cfg->nlat - 1;
            orc_cube_center(cfg, sj, ej, si, ei, &clat, &clon);
            p = local_point(cfg, obs, &ix, clat, clon, idx, rl, cbuf);
            gather_local(k, p, idx, yb, dep, obs, hx, rdi, dis);
            if (orc_letkf_core(k, p, hx, rdi, dis, rl, cfg->inflation, trans, w) != 0) fail = 1;
            for (ii = si; ii <= ei; ii++)
                for (jj = sj; jj <= ej; jj++) {
                    int64_t cc = jj + (int64_t)cfg->nlat * ii;
                    int r, e, l;
                    for (r = 0; r < n; r++) {
                        const double *x = xb + (cc * n + r) * k;
                        double mean = 0.0;
                        for (e = 0; e < k; e++) {
                            double s = 0.0;
                            for (l = 0; l < k; l++) s = s + x[l] * trans[l + k * e];
                            dist[e] = axb[cc * n + r] + s;
                            mean = mean + dist[e];
                        }
                        mean = mean / k;
                        axa[cc * n + r] = axa[cc * n + r] + mean;
                        for (e = 0; e < k; e++)
                            xa[(cc * n + r) * k + e] = xa[(cc * n + r) * k + e] + dist[e] - mean;
                    }
                    count[cc] = count[cc] + 1;
                }
        }
    }
    for (c = 0; c < ncol; c++) {
        int r, e;
        for (r = 0; r < n; r++) {
            for (e = 0; e < k; e++) xa[(c * n + r) * k + e] = xa[(c * n + r) * k + e] / count[c];
            axa[c * n + r] = axa[c * n + r] / count[c];
        }
    }
    obs_index_free(&ix);
    free(count); free(cbuf); free(idx); free(rl); free(hx); free(rdi); free(dis);
    free(trans); free(w); free(dist);
    return fail ? -1 : 0;
}

/* letkf_run mode choice, DA/LETKF/src/letkf.F90:195-235 (the obs halo
 * exchange has no counterpart: every obs is already in one array).          */
int orc_letkf_run(const orc_config *cfg, const orc_obs *obs,
                  const double *xb, const double *axb, double *xa, double *axa)
{
    int rc;
    double *yb = (double *)malloc(sizeof(double) * (obs->nobs * (int64_t)cfg->k + 1));
    double *dep = (double *)malloc(sizeof(double) * (obs->nobs + 1));
    rc = orc_obs_operator(cfg, xb, axb, obs, yb, dep);
    if (rc == 0 && cfg->dec_lat_blocks > 0 && (cfg->cube_n != 1 || cfg->overlap != 0)) rc = -2;
    if (rc == 0) {
        if (cfg->overlap != 0)
            rc = run_overlap(cfg, obs, yb, dep, xb, axb, xa, axa);
        else if (cfg->vert_dist > 0.0)
            rc = run_vertical(cfg, obs, yb, dep, xb, axb, xa, axa);
        else
            rc = orc_letkf_cubes(cfg, obs, yb, dep, xb, axb, xa, axa, NULL, orc_num_cubes(cfg));
    }
    free(yb);
    free(dep);
    return rc;
}

/* dnn2letkf: DA/EnDNN/src/module_da_parallel.F90:184-204.  axb = sum(xin)/real(ens)
 * (the member count as a default real, exact here), xb = xin - axb.  A NaN
 * member stops the reference (:188-193); here the call returns -1.          */
int orc_members_split(const orc_config *cfg, const double *xin, double *xb, double *axb)
{
    const int k = cfg->k, n = state_rows(cfg);
    const int64_t rows = (int64_t)cfg->nlat * cfg->nlon * n;
    int64_t r;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (r = 0; r < rows; r++) {
        const double *x = xin + r * k;
        double s = 0.0;
        int e;
        for (e = 0; e < k; e++) {
            if (isnan(x[e])) bad = 1;
            s = s + x[e];
        }
        s = s / (double)(float)k;
        axb[r] = s;
        for (e = 0; e < k; e++) xb[r * k + e] = x[e] - s;
    }
    return bad ? -1 : 0;
}

/* letkf2dnn: DA/EnDNN/src/module_da_parallel.F90:214-258 (the halo branch
 * does not apply to one global block).  grid_lat is the float grid.         */
void orc_members_blend(const orc_config *cfg, double gamma1, double gamma2, double polar_lat,
                       const double *xb, const double *axb, const double *xa, const double *axa,
                       double *xout, double *spread_b, double *spread_a)
{
    const int k = cfg->k, n = state_rows(cfg);
    const int64_t ncol = (int64_t)cfg->nlat * cfg->nlon;
    int64_t c;
#pragma omp parallel for schedule(static)
    for (c = 0; c < ncol; c++) {
        const double lat = (double)cfg->glat[c % cfg->nlat];
        int r, e;
        for (r = 0; r < n; r++) {
            const int64_t row = c * n + r;
            const double *b = xb + row * k, *a = xa + row * k;
            double *o = xout + row * k;
            double sb = 0.0, sa = 0.0;
            if (fabs(lat) <= polar_lat) {
                for (e = 0; e < k; e++) o[e] = gamma1 * (axb[row] + b[e]) + gamma2 * (axa[row] + a[e]);
                for (e = 0; e < k; e++) {
                    sb = sb + b[e] * b[e];
                    sa = sa + (o[e] - axa[row]) * (o[e] - axa[row]);
                }
            } else {
                for (e = 0; e < k; e++) o[e] = b[e] + axb[row];
                for (e = 0; e < k; e++) {
                    sb = sb + b[e] * b[e];
                    sa = sa + b[e] * b[e];
                }
            }
            spread_b[row] = sqrt(sb / (double)(float)k);
            spread_a[row] = sqrt(sa / (double)(float)k);
        }
    }
}

/* struct_atm2endnn: DA/EnDNN/src/data_trans.F90:2-18, with the Fortran index
 * maps written out: xb(e, j, i, nn) is xb[e + ens*(j + ny*(i + nx*nn))] and
 * xb2(e, nn, i, j) is xb2[e + ens_max*(nn + n_max*(i + nx*j))].             */
#define XB1(e, j, i, nn) xb[(e) + (int64_t)ens * ((j) + (int64_t)ny * ((i) + (int64_t)nx * (nn)))]
#define XB2(e, nn, i, j) xb2[(e) + (int64_t)ens_max * ((nn) + (int64_t)n_max * ((i) + (int64_t)nx * (j)))]
void orc_struct_atm2endnn(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start,
                          int n_start, const double *xb, double *xb2)
{
    int nn, i, j, e;
    for (nn = n_start; nn <= n_start + n - 1; nn++)
        for (i = 1; i <= nx; i++)
            for (j = 1; j <= ny; j++)
                for (e = 1; e <= ens; e++)
                    XB2(ens_start + e - 2, nn - 1, i - 1, j - 1) = XB1(e - 1, j - 1, i - 1, nn - n_start);
}

/* struct_endnn2atm: data_trans.F90:21-38.  The first array is the
 * analysis-side one (the reference's xb), the second the model-side one.     */
void orc_struct_endnn2atm(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start,
                          int n_start, const double *xb2, double *xb)
{
    int nn, i, j, e;
    for (j = 1; j <= ny; j++)
        for (i = 1; i <= nx; i++)
            for (nn = 1; nn <= n; nn++)
                for (e = 1; e <= ens; e++)
                    XB1(e - 1, j - 1, i - 1, nn - 1) = XB2(ens_start + e - 2, nn + n_start - 2, i - 1, j - 1);
}
#undef XB1
#undef XB2

/* struct_atm2endnn_a / struct_endnn2atm_a: data_trans.F90:41-70.           */
void orc_struct_atm2endnn_a(int n, int nx, int ny, int n_max, int n_start, const double *axb, double *axb2)
{
    int nn, i, j;
    for (nn = n_start; nn <= n_start + n - 1; nn++)
        for (i = 1; i <= nx; i++)
            for (j = 1; j <= ny; j++)
                axb2[(nn - 1) + (int64_t)n_max * ((i - 1) + (int64_t)nx * (j - 1))] =
                    axb[(j - 1) + (int64_t)ny * ((i - 1) + (int64_t)nx * (nn - n_start))];
}

void orc_struct_endnn2atm_a(int n, int nx, int ny, int n_max, int n_start, const double *axb, double *axb2)
{
    int nn, i, j;
    for (j = 1; j <= ny; j++)
        for (i = 1; i <= nx; i++)
            for (nn = 1; nn <= n; nn++)
                axb2[(j - 1) + (int64_t)ny * ((i - 1) + (int64_t)nx * (nn - 1))] =
                    axb[(nn + n_start - 2) + (int64_t)n_max * ((i - 1) + (int64_t)nx * (j - 1))];
}

/* read_obs (read_obs_mod.F90:388-441): val_buf(2*nvar+1, obs_num) real(4),
 * val = val_buf(2n-1) + randn * val_buf(2n) and obs_rinv = 1.0/val_buf(2n)**2
 * in real(4); a record with lev_buf == 1 starts a profile (:401-423), whose
 * level-1 record gives lat/lon; entry (prof, lev, n) of the flat list is
 * (prof*nz + lev-1)*nvar + n.                                                */
int64_t orc_obs_from_records(int64_t nrec, int nvar, int nz, const float *lon, const float *lat,
                             const float *lev, const float *val, const float *randn, const int32_t *var_of,
                             double *olat, double *olon, double *oph, int32_t *olev, int32_t *ovar,
                             double *oyo, double *orinv)
{
    const int nv = 2 * nvar + 1;
    int64_t r, indx = -1;
    int n;
    if (nrec % nz != 0) return -1;
    for (r = 0; r < nrec; r++) {
        int level;
        if (nz == 1) {
            indx = r;
            level = 1;
        } else {
            if (lev[r] == 1.0f) indx++;
            level = (int)lev[r];
            if (indx < 0 || level != (int)(r % nz) + 1) return -1;
        }
        for (n = 0; n < nvar; n++) {
            const int64_t e = (indx * nz + (level - 1)) * nvar + n;
            const float v = val[r * nv + 2 * n], sg = val[r * nv + 2 * n + 1];
            const float z = randn ? randn[(int64_t)n * nrec + r] : 0.0f;
            const float yo = v + z * sg;
            const float ri = 1.0f / (sg * sg);
            const int64_t r1 = indx * nz;
            olat[e] = (double)lat[r1];
            olon[e] = (double)lon[r1];
            oph[e] = (double)val[r * nv + 2 * nvar];
            olev[e] = level;
            ovar[e] = var_of[n];
            oyo[e] = (double)yo;
            orinv[e] = (double)ri;
        }
    }
    return nrec * nvar;
}

/* read_obs_regular (read_obs_mod.F90:506-627): centres (latn+lats)/2.0,
 * (lonw+lone)/2.0 in real(4), lon outer and lat inner; obs_rinv =
 * 1.0/r(n,k)**2 in real(4) stored as real(8); yo_tmp = (nw+sw+ne+se)/4.0 in
 * real(4); ph = yo_tmp(1); dis_yo = yo_tmp(n+1) + randn/sqrt(obs_rinv).     */
int64_t orc_obs_regular(int nlat_o, int nlon_o, int nz, int nvar, const float *latn, const float *lats,
                        const float *lonw, const float *lone, const float *r, const float *nw,
                        const float *sw, const float *ne, const float *se, const float *randn,
                        const int32_t *var_of, double *olat, double *olon, double *oph, int32_t *olev,
                        int32_t *ovar, double *oyo, double *orinv)
{
    const int64_t nobs = (int64_t)nlat_o * nlon_o;
    int i, j, k, n;
    for (i = 0; i < nlon_o; i++)
        for (j = 0; j < nlat_o; j++) {
            const int64_t o = j + (int64_t)nlat_o * i;
            for (k = 0; k < nz; k++)
                for (n = 0; n < nvar; n++) {
                    const int64_t e = (o * nz + k) * nvar + n;
#define CORNER(f, q) f[(int64_t)(q) + (int64_t)(nvar + 1) * (k + (int64_t)nz * (j + (int64_t)nlat_o * i))]
                    const float avg_p = (((CORNER(nw, 0) + CORNER(sw, 0)) + CORNER(ne, 0)) + CORNER(se, 0)) / 4.0f;
                    const float avg_v = (((CORNER(nw, n + 1) + CORNER(sw, n + 1)) + CORNER(ne, n + 1)) +
                                         CORNER(se, n + 1)) / 4.0f;
#undef CORNER
                    const float sg = r[n + (int64_t)nvar * k];
                    const double rinv = (double)(1.0f / (sg * sg));
                    const double z = randn ? (double)randn[n + (int64_t)nvar * (k + (int64_t)nz * o)] : 0.0;
                    olat[e] = (double)((latn[j] + lats[j]) / 2.0f);
                    olon[e] = (double)((lonw[i] + lone[i]) / 2.0f);
                    oph[e] = (double)avg_p;
                    olev[e] = k + 1;
                    ovar[e] = var_of[n];
                    oyo[e] = (double)avg_v + z / sqrt(rinv);
                    orinv[e] = rinv;
                }
        }
    return nobs * nz * nvar;
}
