/*
 * letkf_gpu.h -- C-ABI of the GB300 LETKF analysis.
 *
 * Drop-in for the reference's analysis call
 *     letkf_init(...)                   code/x86/TradDA/DA/LETKF/src/letkf_init.F90:2-4
 *     letkf_run(ntimes, xb, axb, xa, axa)   code/x86/TradDA/DA/LETKF/src/letkf.F90:157
 * and, for callers that drive the steps themselves, for the reference's own
 * C entry points of the Sunway build
 *     letkf_core_half_c_(...)   code/sw/TradDA/DA/LETKF/src/letkf_half/letkf_core_half_master.c:24-26
 *     letkf_yb_fast_(...)       code/sw/TradDA/DA/LETKF/src/letkf_yb/letkf_yb_master.c:9-13
 *
 * All arrays are plain pointers with the reference's memory order (Fortran
 * column-major, member fastest):
 *     column index      c = ilat + nlat * ilon
 *     xb, xa            [c][row][member]     = xb(ens, n, lat, lon)
 *     axb, axa          [c][row]             = axb(n, lat, lon)
 *     state rows        2-D variables first, then each 3-D variable x nz levels
 *                       (letkf_init.F90:63-73)
 *     trans             column-major ens x ens per cube, trans[i + ens*j] = trans(i+1, j+1)
 * Observations are one flat list of scalar observations in canonical order
 * (the order in which the reference scans obs types and obs; a profile's
 * levels and variables are consecutive entries, level-major).
 *
 * Every entry point returns LETKF_OK (0) or a negative LETKF_ERR_* code and
 * never exits or prints; letkf_gpu_last_error() gives a message.  A context
 * belongs to one host thread at a time.  There is no CPU fallback: without a
 * usable CUDA device letkf_gpu_create fails with LETKF_ERR_CUDA.
 */
#ifndef LETKF_GPU_H
#define LETKF_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LETKF_OK                 0
#define LETKF_ERR_INVALID       -1   /* bad argument or input value              */
#define LETKF_ERR_CUDA          -2   /* CUDA runtime error / no device           */
#define LETKF_ERR_ALLOC         -3   /* device or pinned allocation failed       */
#define LETKF_ERR_TIMEOUT       -4   /* a bounded device wait ran out            */
#define LETKF_ERR_NOT_CONVERGED -5   /* an eigensolve hit its sweep limit        */
#define LETKF_ERR_UNSUPPORTED   -6   /* configuration not supported              */
#define LETKF_ERR_STATE         -7   /* call order (e.g. no run yet)             */

/* letkf_gpu_run flags */
#define LETKF_HOST_PTRS    0   /* xb/axb/obs/xa/axa are host memory                */
#define LETKF_DEVICE_PTRS  1   /* xb/axb/obs/xa/axa are device memory of this GPU */

/* letkf_params.precision (the reference's computing_precision knob,
 * da_namelist_mod.F90:49, selects the core's arithmetic the same way)       */
#define LETKF_PREC_FP64    0   /* FP64 throughout                                  */
#define LETKF_PREC_MIXED   1   /* FP16 hi/lo tensor-core products for A off the
                                  diagonal (FP32 accumulation, added in FP32
                                  every 16 chunks of 64 observations); g and
                                  diag(A) on the FP32 pipe; BF16 hi/lo
                                  tensor-core products for the update; FP32
                                  Jacobi eigenpairs and FP32 T; wbar in FP32
                                  with one FP64-residual refinement step; FP64
                                  mean increment                                   */
#define LETKF_PREC_MIXED_F64EIG 2 /* the same tensor-core products, with the FP32
                                  Jacobi eigenpairs refined to FP64 (one
                                  Ogita-Aishima step on FP64 residuals), FP64
                                  eigenvalues, 1/sqrt(lambda), T and wbar, and
                                  the FP64 mean increment; ensembles of 64      */

typedef struct letkf_ctx letkf_ctx;

/* Grid and state layout: the values letkf_init takes from coupler_config and
 * pro_info (letkf_init.F90:27-73, pro_info.F90:11).                          */
typedef struct letkf_grid {
    int nlat, nlon;            /* global grid (one logical block)                   */
    int nz;                    /* num_lev                                           */
    int nvar2d, nvar3d;        /* n = nvar2d + nvar3d * nz state rows               */
    int ens;                   /* atm_ensemble_total (k)                            */
    const float *lat;          /* nlat cell-centre latitudes (deg, ascending)       */
    const float *lon;          /* nlon cell-centre longitudes (deg, ascending, [0,360)) */
    const double *hyai, *hybi; /* nz+1 hybrid coefficients; NULL allowed when h_mode
                                  is level select and vertical localization is off  */
    double p0, ptop;           /* hybrid reference / top pressure (Pa)              */
    int ps_row;                /* state row of surface pressure (ps_indx)           */
} letkf_grid;

/* Namelist knobs of &namelist_da (da_namelist_mod.F90:27-49). */
typedef struct letkf_params {
    double loc_dist_km;        /* da_loc_distance: GC half-width c; obs kept to 2c  */
    double vert_dist;          /* da_vert_distance; <= 0 turns vertical loc. off    */
    double inflation;          /* da_inflation_factor                               */
    double obs_polar_deg;      /* da_polar_letkf_lat with polar_discard, else 91    */
    int gc_filter;             /* da_gc_enable: 1 Gaspari-Cohn, 0 box-car           */
    int gc_filter_vertical;    /* da_gc_enable_vertical                             */
    int max_obs;               /* MAX_OBS (letkf.F90:155): 10000                    */
    int cube_n;                /* da_block_interval                                 */
    int cube_nz;               /* da_vertical_interval                              */
    int overlap;               /* da_block_overlap                                  */
    int h_mode;                /* 0: hybrid log-p interpolation (obs_make.F90:233-381),
                                  1: level select (obs carries a model level)       */
    int precision;             /* LETKF_PREC_*                                      */
    /* Observation sets.  0, 0: one logical block holding every observation
     * once (each obs scanned once, in index order).  Otherwise the local
     * lists are those of a DA group decomposed into decomp_lat_blocks x
     * decomp_lon_blocks MPI blocks (module_da_parallel.F90:73-103, pro_info.F90:
     * 96-125): each block holds the obs inside its lat/lon box
     * (read_obs_mod.F90:73-165), and a column scans the blocks of its
     * neighbour set (letkf_init.F90:100-341) in the reference's order, which
     * reproduces a P-rank run's lists.  Needs cube_n 1 and overlap 0;
     * letkf_decomp_dims gives the blocks of P ranks.                         */
    int decomp_lat_blocks, decomp_lon_blocks;
} letkf_params;

/* Observations (the obs_list fields, read_obs_mod.F90:15-27, flattened). */
typedef struct letkf_obs {
    int64_t nobs;
    const double *lat, *lon;   /* degrees, lat in [-90,90], lon in [0,360]          */
    const double *ph;          /* pressure (Pa): h_mode 0 and vertical loc.; may be NULL otherwise */
    const int32_t *lev;        /* model level 1..nz for h_mode 1 (3-D variables)    */
    const int32_t *var;        /* variable index 0..nvar2d+nvar3d-1                 */
    const double *yo;          /* observed values                                   */
    const double *rinv;        /* 1/sigma^2; used narrowed to float as the reference */
} letkf_obs;

/* Per-run diagnostics. */
typedef struct letkf_stats {
    int64_t ncubes;            /* analysis units (cubes) of the last run            */
    int64_t sum_p;             /* total local observations over all cubes           */
    int64_t max_p;             /* largest local observation count                   */
    int64_t n_truncated;       /* cubes whose list stopped at max_obs               */
    int64_t n_borderline;      /* obs-cube pairs with |dist/c - 2| < 1e-12          */
    int64_t n_not_converged;   /* eigensolves that hit the sweep limit              */
    int32_t max_sweeps;        /* most Jacobi sweeps any cube needed                */
    int32_t precision;
    /* Device-event times between the stages of the last run.  In a run with
     * host buffers the state copies overlap the stages: ms_h2d then holds the
     * mean's and the observations' copies only, ms_core includes waiting for
     * the perturbations' copy,
     * and ms_d2h is the copy left after the analysis; ms_total is the whole. */
    double ms_h2d, ms_obs, ms_search, ms_core, ms_d2h, ms_total;
    int64_t sum_sweeps;        /* Jacobi sweeps summed over all cubes               */
    int64_t n_ill_conditioned; /* mixed form: cubes whose A' has lambda_max/lambda_min
                                  above 1e4, where the FP32 eigenpairs lose digits    */
    int32_t sched_chunk;       /* mixed form: cubes per work-queue chunk (0: default 16) */
    int32_t n_windows;         /* consecutive cube windows the run was split into
                                  (1 when every local list fit the list pool)        */
    double ms_stage[4];        /* mixed forms, k = 64 (the staged core): device-event
                                  times of the A-build, eigensolve, update and
                                  (LETKF_PREC_MIXED_F64EIG) FP64 refinement
                                  launches, each summed over the run's blocks of
                                  cubes (0 for other forms and inside a graph)       */
} letkf_stats;

/* The lat x lon blocks of a DA group of nranks MPI ranks: MPI_Dims_create(
 * nranks, 2) (the most balanced factor pair, larger first), whose first
 * dimension splits longitude and second latitude
 * (EnDNN/src/module_da_parallel.F90:73-103, 143).  No counterpart function in
 * the reference, which asks MPI.  Returns LETKF_ERR_INVALID for nranks < 1.  */
int letkf_decomp_dims(int nranks, int *lat_blocks, int *lon_blocks);

/* Create a context on CUDA device `device` (the current device if < 0).
 * Copies the grid; replaces letkf_init.                                      */
int letkf_gpu_create(letkf_ctx **ctx, const letkf_grid *grid, const letkf_params *params,
                     int device);

/* Use this CUDA stream (a cudaStream_t) for all following work; NULL = the
 * context's own stream.                                                     */
int letkf_gpu_set_stream(letkf_ctx *ctx, void *stream);

/* The analysis: letkf_run(ntimes, xb, axb, xa, axa) with the observations
 * passed in instead of read from Redis.  xb holds perturbations and axb the
 * mean, as run_da_parallel hands them over (module_da_parallel.F90:184-211);
 * xa/axa receive the analysis perturbations and mean.  With
 * LETKF_HOST_PTRS the call copies in and out and returns when xa/axa are
 * written (with page-locked buffers the state copies overlap the search and
 * the analysis: the copy-in runs beside H's geometry pass and the search, and
 * finished blocks of columns are copied out while later ones are analysed;
 * ordinary pageable buffers get the same overlap: a host thread of the
 * context issues their copies, since a copy from or to pageable memory holds
 * the thread that issues it until the bytes have moved); with
 * LETKF_DEVICE_PTRS it returns with the work queued on the stream (call
 * letkf_gpu_synchronize before reading the outputs).                        */
int letkf_gpu_run(letkf_ctx *ctx, const double *xb, const double *axb, const letkf_obs *obs,
                  double *xa, double *axa, int flags);

/* With host buffers (letkf_gpu_run, letkf_gpu_run_halo), let the kernels
 * read the state rows of the observation operator straight from the caller's
 * arrays when the device can address them (page-locked memory, or pageable
 * memory on a device that uses the host's page tables, such as a Grace
 * host): H and the local analyses then run while the bulk copy of the state
 * is still under way, and each block of the analysis waits only for its own
 * columns.  on = 0: H waits for the whole state.  The default is 1; the
 * results are the same either way.  No counterpart in the reference.        */
int letkf_gpu_set_host_read(letkf_ctx *ctx, int on);

/* letkf_gpu_run on host arrays in letkf_run's own layout with a halo
 * (letkf.F90:157-257; xb(ens, n, 1-halo:nlat+halo, 1-halo:nlon+halo), axb,
 * xa, axa alike): the copies read and write the interior columns in place
 * (strided copies of whole longitude lines), and the halo of xa/axa is left
 * as it was.  halo = 0 is letkf_gpu_run with LETKF_HOST_PTRS.               */
int letkf_gpu_run_halo(letkf_ctx *ctx, int halo, const double *xb, const double *axb,
                       const letkf_obs *obs, double *xa, double *axa);

/* The caller's conversion around letkf_run (run_da_parallel,
 * EnDNN/src/module_da_parallel.F90:163-261), for letkf_gpu_run_members.     */
typedef struct letkf_blend {
    double gamma1, gamma2;     /* gamma1, gamma2 (da_namelist_mod.F90:39-40): the
                                  analysis members are gamma1 (axb + xb) +
                                  gamma2 (axa + xa) (:230-231)                     */
    double polar_lat_deg;      /* da_polar_letkf_lat: columns with |grid_lat| above it
                                  keep the background (:222, :242-251)            */
} letkf_blend;

/* run_da_parallel's body on the device: full background members
 * xb_in [col][row][member] in; the mean and perturbations formed (dnn2letkf,
 * module_da_parallel.F90:184-204: mean = sum / real(ens); a NaN member makes
 * the call return LETKF_ERR_INVALID, and the outputs are then not meaningful),
 * the analysis of letkf_gpu_run, and the blend and spreads (letkf2dnn,
 * :214-258): xa_out [col][row][member] the analysis members, spread_b and
 * spread_a [col][row] the background and analysis spreads sqrt(sum d^2 / ens).
 * With one column per cube, no overlap and no vertical localization (and an
 * ensemble of at most 64 in the mixed forms) the split and the blend are done
 * inside the analysis (H reads the members, the update forms each row's mean
 * and writes the blended members and both spreads), so the call makes no
 * pass over the state beyond those of letkf_gpu_run; otherwise they are one
 * pass each before and after it.  Every cube is analysed (no cube range).
 * With LETKF_HOST_PTRS all arrays, observations included, are host memory;
 * with LETKF_DEVICE_PTRS all are device memory.                             */
int letkf_gpu_run_members(letkf_ctx *ctx, const double *xb_in, const letkf_obs *obs,
                          const letkf_blend *blend, double *xa_out, double *spread_b,
                          double *spread_a, int flags);

/* Observations built on the device from the obs store's raw buffers, in the
 * canonical flat order (obs, level, variable) that gen_yb_dis scans
 * (letkf_yb.F90:71-113).  Both write the context's observation buffers and
 * fill *obs with device pointers into them (valid until the next build or
 * letkf_gpu_destroy), for letkf_gpu_run with LETKF_DEVICE_PTRS.  The float
 * inputs are host (LETKF_HOST_PTRS) or device (LETKF_DEVICE_PTRS) memory;
 * var_of[nvar] (host) maps each payload variable to a state variable index.
 * randn may be NULL (no perturbation).
 *
 * Records (read_obs, read_obs_mod.F90:339-448): lon, lat, lev[nrec] and
 * val[nrec][2 nvar + 1] = value, sigma per variable, then pressure;
 * randn[nvar][nrec] the N(0,1) draws of the perturbation.  nz = 1 for
 * single-level types; for profile types (ADPUPA, GPSRO) nz levels per
 * profile, whose records hold lev = 1..nz in order (else LETKF_ERR_INVALID).
 * yo = value + randn * sigma and rinv = 1 / sigma^2 in single precision.   */
int letkf_gpu_obs_from_records(letkf_ctx *ctx, int64_t nrec, int nvar, int nz, const float *lon,
                               const float *lat, const float *lev, const float *val, const float *randn,
                               const int32_t *var_of, letkf_obs *obs, int flags);

/* Regular obs grid (read_obs_regular, read_obs_mod.F90:451-651): cell edges
 * latn, lats [nlat_o] and lonw, lone [nlon_o]; sigma r(nvar, nz); four corner
 * fields nw, sw, ne, se (nvar + 1, nz, nlat_o, nlon_o) in Fortran order
 * (pressure first, then the variables); randn(nvar, nz, nlat_o * nlon_o).
 * Obs at the cell centres, longitude outer and latitude inner; values and
 * pressure the four-corner average; yo = value + randn / sqrt(rinv).         */
int letkf_gpu_obs_regular(letkf_ctx *ctx, int nlat_o, int nlon_o, int nz, int nvar, const float *latn,
                          const float *lats, const float *lonw, const float *lone, const float *r,
                          const float *nw, const float *sw, const float *ne, const float *se,
                          const float *randn, const int32_t *var_of, letkf_obs *obs, int flags);

/* The coupler's layout transforms (EnDNN/src/data_trans.F90:1-70) on device
 * memory, so the state never goes through the host between the model and the
 * analysis.  nx = latitudes, ny = longitudes; ens_start and n_start are
 * 1-based as in the reference.  atm2endnn: xb(ens, ny, nx, n) (Fortran order)
 * into members ens_start.. and rows n_start.. of xb2(ens_max, n_max, nx, ny)
 * (the [col][row][member] layout of letkf_gpu_run); endnn2atm: back.  The _a
 * forms move the mean, axb(ny, nx, n) <-> axb2(n_max, nx, ny).  Work is
 * queued on `stream` (a cudaStream_t; NULL = the default stream).           */
int letkf_struct_atm2endnn(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start,
                           int n_start, const double *xb, double *xb2, void *stream);
int letkf_struct_endnn2atm(int ens, int n, int nx, int ny, int ens_max, int n_max, int ens_start,
                           int n_start, const double *xb, double *xb2, void *stream);
int letkf_struct_atm2endnn_a(int n, int nx, int ny, int n_max, int n_start, const double *axb,
                             double *axb2, void *stream);
int letkf_struct_endnn2atm_a(int n, int nx, int ny, int n_max, int n_start, const double *axb,
                             double *axb2, void *stream);

/* Most local-list entries (obs of one cube's list) the list pool may hold;
 * 0 (the default) sizes it from the device's free memory.  When the lists of
 * all analysed cubes do not fit, a run searches and analyses the cubes in
 * consecutive windows whose lists fit (letkf_stats.n_windows), with the same
 * results; letkf_gpu_local_obs then has no lists to return.  No counterpart
 * in the reference, whose ranks each hold their own sub-domain's lists.     */
int letkf_gpu_set_list_limit(letkf_ctx *ctx, int64_t max_entries);

/* Analyse only cubes first .. first+count-1 (count < 0: every cube), as one
 * DA rank analyses its own sub-domain (letkf_run's nx x ny arrays,
 * letkf.F90:169-176); cube = lat block + (lat blocks) * lon block, so with
 * cube_n 1 the cubes are the columns.  The observation operator still reads
 * the whole background.  Columns of other cubes are not written (host
 * pointers: not copied back).  With cube_n > 1, first and count must be
 * multiples of the number of lat blocks (whole longitude strips).  The local
 * lists of a range run are not kept for letkf_gpu_local_obs.  The mixed form
 * warm-starts each cube's eigensolve from the cube before it inside aligned
 * runs of cubes (8 cubes for k = 64, 16 otherwise), so a range whose first
 * cube is inside a run starts that cube cold (results then agree with a whole
 * run to FP32 eigensolve precision); ranges starting at multiples of 16,
 * windows and the work-queue schedule leave every result unchanged.          */
int letkf_gpu_set_cube_range(letkf_ctx *ctx, int64_t first, int64_t count);

/* Most polls of each bounded wait of the mixed cores on their own
 * tensor-core work (polls < 0: the default, 2^22; 0: every wait gives up at
 * once).  A wait that runs out makes the run return LETKF_ERR_TIMEOUT after
 * the kernel has let its committed products finish and freed its tensor
 * memory, so the context stays usable.  For tests of that path; no
 * counterpart in the reference.                                             */
int letkf_gpu_set_wait_limit(letkf_ctx *ctx, int64_t polls);

/* Keep (1) or drop (0) every cube's trans and w of the following runs in
 * device memory (ncubes * ens * (ens+1) doubles) for letkf_gpu_last_trans. */
int letkf_gpu_set_keep_trans(letkf_ctx *ctx, int keep);

/* Wait for the context's stream and report any deferred device error. */
int letkf_gpu_synchronize(letkf_ctx *ctx);

/* Observation operator H and mean removal only (gen_obs_struct,
 * letkf_obs.F90:16-182): yb[obs][ens] perturbations and dep = yo - mean(H xb).
 * Host pointers.                                                             */
int letkf_gpu_obs_operator(letkf_ctx *ctx, const double *xb, const double *axb,
                           const letkf_obs *obs, double *yb, double *dep);

/* Local observation lists of the last run (gen_yb_dis selection,
 * letkf_yb.F90:3-133): counts[cube] and, if idx != NULL, the obs indices in
 * canonical order and their localization weights, packed by cube
 * (offsets[cube] = start; ncubes+1 entries).  Host pointers.                */
int letkf_gpu_local_obs(letkf_ctx *ctx, int64_t *offsets, int32_t *idx, double *rloc);

/* The same lists for the n cubes listed in `cubes` only, packed in that
 * order (offsets has n+1 entries; idx and rloc may be NULL): for checking a
 * sample of a large grid's lists without copying every list to the host.
 * Host pointers.  No counterpart in the reference.                          */
int letkf_gpu_local_obs_cubes(letkf_ctx *ctx, const int64_t *cubes, int64_t n, int64_t *offsets,
                              int32_t *idx, double *rloc);

/* Transform matrices of the last run for the listed cubes: trans (ens x ens,
 * column-major, trans(i,j) + w(i) as letkf_core returns it) and w.          */
int letkf_gpu_last_trans(letkf_ctx *ctx, const int64_t *cubes, int64_t ncubes,
                         double *trans, double *w);

/* Batched letkf_core (letkf_core.F90:14-233; Sunway letkf_core_batch,
 * code/sw/TradDA/DA/LETKF/src/letkf_core.F90:16-379): for nb independent
 * problems, problem b uses rows offsets[b]..offsets[b+1]-1 of hxens[obs][ens],
 * rdiaginv (float, as the reference), dep and rloc.  Writes trans
 * (nb x ens x ens, column-major each) and w (nb x ens).  Host pointers.      */
int letkf_gpu_core_batch(letkf_ctx *ctx, int64_t nb, const int64_t *offsets,
                         const double *hxens, const float *rdiaginv, const double *dep,
                         const double *rloc, double *trans, double *w);

/* The batched letkf_core above for callers that cannot allocate device
 * memory (a model that owns all of the GPU's memory through its own pool, or
 * a caller that must not add the device-wide synchronization of cudaMalloc and
 * cudaFree).  No counterpart in the reference: it is an addition of this
 * library.  Every pointer is device memory of the current device, owned by the
 * caller; offsets has nb+1 entries.  No context is needed and nothing is
 * allocated: the scratch (per-problem counts, a status word, counters) is a
 * fixed array inside the library that every GPU which loads the library holds
 * until the process exits, sized for at most LETKF_NOALLOC_MAX_PROBLEMS
 * problems; larger nb returns LETKF_ERR_INVALID.  The first call on a device
 * looks up that array's device address (make it before any stream capture);
 * with CUDA's lazy module loading (the default) that first call also loads
 * the library's kernels and the array onto the device, which takes device
 * memory, so make it before a memory pool reserves the rest of the GPU.  The
 * address is kept for the life of the process: do not use the call across a
 * cudaDeviceReset of that device.
 * All calls share the one array, so calls that overlap on the GPU (different
 * streams or host threads at once) race; issue them one after another.  The
 * call waits for `stream` (a cudaStream_t, NULL = the default stream) before it
 * returns, to report LETKF_ERR_INVALID for bad offsets and
 * LETKF_ERR_NOT_CONVERGED from the eigensolves.                              */
#define LETKF_NOALLOC_MAX_PROBLEMS 65536
int letkf_gpu_core_batch_noalloc(int ens, double inflation, int64_t nb, const int64_t *offsets,
                                 const double *hxens, const float *rdiaginv, const double *dep,
                                 const double *rloc, double *trans, double *w, void *stream);

/* Autotuner of the mixed form's schedule: runs the analysis (as
 * letkf_gpu_run) once per candidate chunk size of the core's work queue
 * (consecutive cubes per chunk, chunks taken heaviest first: 8, 16, 32, 64
 * for k = 64; 16, 32, 64, 128 otherwise) and keeps the one with the fastest
 * core for the context's later runs (letkf_stats.sched_chunk).  The chunk
 * size changes the speed only: every candidate gives the same analysis bit
 * for bit.  xa/axa hold the last run's analysis.  For the FP64 form it is one
 * letkf_gpu_run.  No counterpart in the reference.                           */
int letkf_gpu_autotune(letkf_ctx *ctx, const double *xb, const double *axb, const letkf_obs *obs,
                       double *xa, double *axa, int flags);

/* Set the mixed form's work-queue chunk (cubes per chunk, a power of two
 * from 8 to 1024; 0: the default, 16) instead of autotuning it.  Chunks of
 * the one-launch cores (k != 64) are at least 16 cubes; a run whose range
 * would need more than 8191 chunks doubles the size.  LETKF_ERR_INVALID for
 * other values.  No counterpart in the reference.                            */
int letkf_gpu_set_schedule(letkf_ctx *ctx, int chunk);

/* One CUDA graph over the analyses of several contexts (the batching form:
 * instances of different grids and ensemble sizes, each on its own stream
 * forked from and joined to one origin).  No counterpart in the reference.
 * All pointers are device memory; obs holds n observation sets.  The call
 * first runs each analysis once outside the graph to size every buffer for
 * these inputs, then captures them; letkf_batch_launch replays the graph on
 * the same pointers (refresh the inputs in place between launches) and
 * returns at once, letkf_batch_sync waits for it and reports the worst
 * status of the contexts (their stats are updated; a list pool too small for
 * new inputs shows as LETKF_ERR_ALLOC: create the batch again).  Contexts with
 * decomposed observation sets are not captured (LETKF_ERR_UNSUPPORTED).
 * Do not run a captured context by itself while its batch may be running.   */
typedef struct letkf_batch letkf_batch;
int letkf_batch_create(letkf_batch **batch, int n, letkf_ctx *const *ctxs, const double *const *xb,
                       const double *const *axb, const letkf_obs *obs, double *const *xa,
                       double *const *axa);
/* stream: a cudaStream_t for the replay (NULL: the batch's own stream);
 * letkf_batch_sync waits for the same stream.                               */
int letkf_batch_launch(letkf_batch *batch, void *stream);
int letkf_batch_sync(letkf_batch *batch, void *stream);
int64_t letkf_batch_launches(letkf_batch *batch);   /* kernels per replay */
int letkf_batch_destroy(letkf_batch *batch);

int letkf_gpu_get_stats(letkf_ctx *ctx, letkf_stats *stats);
const char *letkf_gpu_last_error(letkf_ctx *ctx);
int letkf_gpu_destroy(letkf_ctx *ctx);

/* Number of kernel launches this library made on the calling thread so far. */
int64_t letkf_gpu_launch_count(void);

/* Fortran-callable shims, by reference with a trailing underscore as the
 * reference's own C interop (letkf_core_half_c_).  They keep one context per
 * process.  letkf_init_gpu_ takes the grid of the whole globe; ierr receives
 * the status code.                                                           */
void letkf_init_gpu_(const int *nlat, const int *nlon, const int *nz, const int *nvar2d,
                     const int *nvar3d, const int *ens, const float *lat, const float *lon,
                     const double *hyai, const double *hybi, const double *p0,
                     const double *ptop, const int *ps_row, const double *loc_dist_km,
                     const double *vert_dist, const double *inflation,
                     const double *obs_polar_deg, const int *gc_filter,
                     const int *gc_filter_vertical, const int *cube_n, const int *cube_nz,
                     const int *overlap, const int *h_mode, const int *precision, int *ierr);
/* Stage the observations of the next letkf_run_gpu_ call (replaces the
 * Redis read of gen_obs_struct).  var is 1-based as Fortran indices are.    */
void letkf_set_obs_gpu_(const int64_t *nobs, const double *lat, const double *lon,
                        const double *ph, const int *lev, const int *var, const double *yo,
                        const double *rinv, int *ierr);
/* letkf_run with the reference's halo layout: xb(ens, n, 1-halo:nlat+halo,
 * 1-halo:nlon+halo); only the interior is read and written, straight from
 * and to the caller's arrays (letkf_gpu_run_halo).                          */
void letkf_run_gpu_(const int *ntimes, const int *halo, const double *xb, const double *axb,
                    double *xa, double *axa, int *ierr);
void letkf_final_gpu_(int *ierr);

#ifdef __cplusplus
}
#endif

#endif /* LETKF_GPU_H */
