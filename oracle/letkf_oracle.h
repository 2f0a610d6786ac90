/*
 * letkf_oracle.h -- CPU restatement of the reference LETKF analysis path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU path is
 * compared against (tests, the smoke check and the CPU-baseline leg of the
 * benchmark).  No product code path links, loads or calls it.
 *
 * Every routine restates one routine of the x86 Fortran LETKF
 * (code/x86/TradDA/DA/LETKF/src/ and code/x86/TradDA/DA/utils/); the citation
 * is on each function in letkf_oracle.c.  The restatement keeps the
 * reference's exactness rules: float grid coordinates, float-rounded literals
 * in the distance and Gaspari-Cohn functions, R^-1 narrowed to real(4),
 * `gc > 0` selection, canonical list order and MAX_OBS truncation.
 * Its eigensolver is a self-written cyclic Jacobi method (Golub & Van Loan,
 * Matrix Computations, 4th ed., section 8.5), standing in for MKL dsyevd.
 *
 * Parity unpinned against the reference's own binaries: the Fortran LETKF
 * (MKL, MPI) cannot be built here and ships no golden vectors.  The oracle is
 * checked against closed-form known answers and against an independent
 * numpy/LAPACK restatement (tests/golden/make_golden.py and its fixtures).
 *
 * Data layout (identical to the reference's Fortran arrays):
 *   column index   c = ilat + nlat * ilon            (lat fastest)
 *   xb, xa         [c][row][member]  = xb(ens, n, lat, lon)
 *   axb, axa       [c][row]          = axb(n, lat, lon)
 *   state rows     2-D variables first, then each 3-D variable x nz levels
 *   yb             [obs][member]     = pro_yb(ens, ., ., obs)
 *   trans          column-major k x k, trans[i + k*j] = trans(i+1, j+1)
 */
#ifndef LETKF_ORACLE_H
#define LETKF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_config {
    int nlat, nlon, nz, nvar2d, nvar3d, k;
    const float *glat;          /* nlat cell-centre latitudes, degrees, ascending      */
    const float *glon;          /* nlon cell-centre longitudes, degrees, ascending     */
    const double *hyai, *hybi;  /* nz+1 hybrid interface coefficients (log-p H, vertical mode) */
    double p0, ptop;            /* hybrid reference and top pressure (Pa)              */
    int ps_row;                 /* state row holding surface pressure                  */
    double local_dist;          /* Gaspari-Cohn half-width c in km; obs kept out to 2c */
    double vert_dist;           /* vertical localization scale in ln p; <= 0 is off    */
    double inflation;           /* multiplicative inflation rho                        */
    double obs_polar;           /* obs with |lat| > obs_polar are not used             */
    int gc_filter;              /* 1: Gaspari-Cohn (schr2), 0: box-car (schr)          */
    int gc_filter_vertical;
    int max_obs;                /* MAX_OBS                                             */
    int cube_n, cube_nz, overlap;
    int h_mode;                 /* 0: hybrid log-p vertical interpolation, 1: level select */
    /* Observation-set mode.  0, 0: one logical block that holds every obs once
     * (mode "global").  Otherwise the analysis emulates a DA run decomposed
     * into dec_lat_blocks x dec_lon_blocks MPI blocks (mode "decomposed"):
     * each block holds the obs inside its lat/lon box, and a column scans the
     * blocks of its neighbour set in the reference's order.  Needs cube_n 1
     * and overlap 0.                                                        */
    int dec_lat_blocks, dec_lon_blocks;
} orc_config;

typedef struct orc_obs {
    int64_t nobs;
    const double *lat, *lon;    /* degrees; lon in [0, 360]                            */
    const double *ph;           /* obs pressure, Pa (log-p H and vertical mode)        */
    const int *lev;             /* model level 1..nz (level-select H, 3-D variables)   */
    const int *var;             /* index into the sorted variable list (2-D first)     */
    const double *yo;           /* observed value                                      */
    const double *rinv;         /* 1/sigma^2 as computed in real(4) by the reader      */
} orc_obs;

/* Scalar helpers. */
double orc_schr2(double ri);
double orc_schr(double ri);
double orc_latlon_dist(double x1, double y1, double x2, double y2);
int orc_find_obs_grid(const orc_config *cfg, double lat, double lon,
                      int *tx, int *ty, double *ax, double *ay);

/* Observation operator H on all members, then mean removal.
 * Writes yb[obs][k] (perturbations) and dep[obs] = yo - mean(H xb).  */
int orc_obs_operator(const orc_config *cfg, const double *xb, const double *axb,
                     const orc_obs *obs, double *yb, double *dep);

/* MPI_Dims_create(nranks, 2) as the DA group decomposes the globe: the most
 * balanced factor pair, larger first; dims(1) splits longitude and dims(2)
 * latitude.  Returns 0, or -1 for nranks < 1.                               */
int orc_decomp_dims(int nranks, int *lat_blocks, int *lon_blocks);

/* Neighbour set of lat/lon block (bx, by) (0-based) in scan order: writes up
 * to cap block ids (bx' * lon_blocks + by') and returns how many there are.  */
int orc_block_slots(const orc_config *cfg, int bx, int by, int32_t *blocks, int cap);

/* Cubes of the column loop (no overlap), ordered lon-block-major. */
int64_t orc_num_cubes(const orc_config *cfg);
void orc_cube_bounds(const orc_config *cfg, int64_t cube, int *sj, int *ej, int *si, int *ei);
void orc_cube_center(const orc_config *cfg, int sj, int ej, int si, int ei,
                     double *clat, double *clon);

/* Local observation lists of all cubes (one logical block covering the globe).
 * offsets has num_cubes+1 entries.  With idx == NULL only offsets is filled.
 * Returns the total list length, or a negative value if it exceeds cap.   */
int64_t orc_local_obs(const orc_config *cfg, const orc_obs *obs,
                      int64_t *offsets, int32_t *idx, double *rloc, int64_t cap);

/* Local lists of the n cubes listed in `cubes`, packed in that order
 * (offsets has n+1 entries; idx == NULL: offsets only).  Returns the total,
 * or a negative value if it exceeds cap.                                    */
int64_t orc_local_obs_cubes(const orc_config *cfg, const orc_obs *obs, int64_t n, const int64_t *cubes,
                            int64_t *offsets, int32_t *idx, double *rloc, int64_t cap);

/* Local list for one point.  Returns nobsl. */
int orc_local_obs_point(const orc_config *cfg, const orc_obs *obs, double clat, double clon,
                        int32_t *idx, double *rloc);

/* Symmetric eigensolve by cyclic Jacobi; eigenvalues ascending, vectors in
 * the columns of v (column-major).  a is overwritten.  Returns sweeps used,
 * or -1 if max_sweeps was reached.  */
int orc_jacobi_eig(int k, double *a, double *lam, double *v, int max_sweeps);

/* letkf_core: hxens[obs][k] -> trans (column-major k x k) and w (k). */
int orc_letkf_core(int k, int p, const double *hxens, const float *rdiaginv,
                   const double *dep, const double *rloc, double inflation,
                   double *trans, double *w);

/* Full analysis (H, local lists, core, update) for all columns.
 * mode is chosen as letkf_run does: overlap > 0 -> overlapped cubes,
 * else vert_dist > 0 -> vertical localization, else the plain column loop.  */
int orc_letkf_run(const orc_config *cfg, const orc_obs *obs,
                  const double *xb, const double *axb, double *xa, double *axa);

/* Plain column loop for a subset of cubes, given H outputs (yb, dep).
 * Used for bounded CPU samples.  Only the listed cubes' columns are written. */
int orc_letkf_cubes(const orc_config *cfg, const orc_obs *obs, const double *yb,
                    const double *dep, const double *xb, const double *axb,
                    double *xa, double *axa, const int64_t *cubes, int64_t ncubes);

/* Number of OpenMP threads the library will use. */
int orc_num_threads(void);

/* The caller's conversion around letkf_run (run_da_parallel,
 * DA/EnDNN/src/module_da_parallel.F90:184-258), for the members entry point.
 * members_split: full members xin [col][n][k] -> perturbations xb and mean
 * axb (sum over members / real(ens)); returns -1 if a member is NaN.
 * members_blend: xout = gamma1 (axb + xb) + gamma2 (axa + xa) where
 * |grid_lat| <= polar_lat, else xb + axb; spread_b = sqrt(sum xb^2 / ens),
 * spread_a = sqrt(sum (xout - axa)^2 / ens) (= spread_b where polar).     */
int orc_members_split(const orc_config *cfg, const double *xin, double *xb, double *axb);
/* Observations from the obs store's raw buffers (read_obs and
 * read_obs_regular, DA/LETKF/src/read_obs_mod.F90:339-651), flattened in the
 * (obs, level, variable) order of gen_yb_dis; arrays as letkf_obs.  Returns
 * the entry count, or -1 for a profile whose records are not levels 1..nz.  */
int64_t orc_obs_from_records(int64_t nrec, int nvar, int nz, const float *lon, const float *lat,
                             const float *lev, const float *val, const float *randn, const int32_t *var_of,
                             double *olat, double *olon, double *oph, int32_t *olev, int32_t *ovar,
                             double *oyo, double *orinv);
int64_t orc_obs_regular(int nlat_o, int nlon_o, int nz, int nvar, const float *latn, const float *lats,
                        const float *lonw, const float *lone, const float *r, const float *nw,
                        const float *sw, const float *ne, const float *se, const float *randn,
                        const int32_t *var_of, double *olat, double *olon, double *oph, int32_t *olev,
                        int32_t *ovar, double *oyo, double *orinv);
/* The coupler's layout transforms, EnDNN/src/data_trans.F90:1-70 (Fortran
 * arrays, 1-based ens_start / n_start).                                       */
void orc_struct_atm2endnn(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start,
                          int n_start, const double *xb, double *xb2);
void orc_struct_endnn2atm(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start,
                          int n_start, const double *xb, double *xb2);
void orc_struct_atm2endnn_a(int n, int nx, int ny, int n_max, int n_start, const double *axb, double *axb2);
void orc_struct_endnn2atm_a(int n, int nx, int ny, int n_max, int n_start, const double *axb, double *axb2);
void orc_members_blend(const orc_config *cfg, double gamma1, double gamma2, double polar_lat,
                       const double *xb, const double *axb, const double *xa, const double *axa,
                       double *xout, double *spread_b, double *spread_a);

#ifdef __cplusplus
}
#endif

#endif
