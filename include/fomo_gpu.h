/*
 * fomo_gpu.h -- C ABI of libfomo_gpu, the GB300 implementation of FoMo-C's
 * nearest-neighbour render path (and its Thomson white-light variant).
 *
 * The reference has no ABI for this path: FoMoObject::render (fomo-c/src/
 * fomo-object.cpp:374-455) calls emissionfromdatacube (fomo-CHIANTI.cpp:
 * 228-322) and RenderWithNearestNeighbour / RenderWithThomson (fomo-c/src/
 * FoMo-internal.h:23-27) by value on std::vectors.  This header is the
 * boundary a binding (the C++ FoMo.h drop-in in include/FoMo.h, or a ctypes
 * stub) calls; each entry point names the reference code it replaces.
 *
 * Conventions
 *  - Plain pointers and sizes; no torch or CUDA types.  `stream` arguments are
 *    a cudaStream_t passed as void* (NULL = the context's own stream).
 *  - Every call returns 0 (FOMO_OK) or a negative FOMO_E* code; the message is
 *    in fomo_last_error(ctx).  Nothing calls exit() (the reference exits on a
 *    missing table, a bad table size, a failed imaging check or an unknown
 *    render method: fomo-CHIANTI.cpp:126-197,278, fomo-object.cpp:430-434).
 *  - A context is used from one thread at a time; the render server
 *    (fomo_server_*) owns its own context and fomo_server_submit is safe from
 *    any thread.
 *  - Device memory is owned by the context.  Host buffers passed in are read
 *    (uploads) or written (results) before the call returns, unless the call
 *    is documented as asynchronous.
 *  - Cube layout: (i * nx + j) * nlambda + il, lambda fastest, then x, then y
 *    (fomo-nearestneighbour.cpp:208), FP32.
 */
#ifndef FOMO_GPU_H
#define FOMO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FOMO_OK 0
#define FOMO_EINVAL (-1)      /* bad argument */
#define FOMO_ENOMEM (-2)      /* device or host allocation failed */
#define FOMO_EADMISSION (-3)  /* request larger than the context's HBM budget */
#define FOMO_EDEVICE (-4)     /* CUDA error (message has the CUDA error string) */
#define FOMO_ETIMEOUT (-5)    /* wait timed out */
#define FOMO_ENOTFOUND (-6)   /* unknown snapshot / table / ticket id */
#define FOMO_EIO (-7)         /* table file missing or unreadable */
#define FOMO_ETABLE (-8)      /* table malformed, or imaging check failed */
#define FOMO_ECANCELLED (-9)  /* request cancelled */
#define FOMO_EMETHOD (-10)    /* unknown render method */
#define FOMO_ENODEVICE (-11)  /* no CUDA device / extension not usable */

#define FOMO_METHOD_NN 0       /* "NearestNeighbourGPU" */
#define FOMO_METHOD_THOMSON 1  /* "ThomsonGPU" */
#define FOMO_METHOD_PROJECTION 2 /* "Projection": each point added to the pixel nearest its projection
                                    (fomo-projection.cpp:17-193); no LOS march, nz only sets the path length */

#define FOMO_OBS_SPECTROSCOPIC 1 /* FoMo::Spectroscopic (FoMo.h:120-125) */
#define FOMO_OBS_IMAGING 2       /* FoMo::Imaging */

typedef struct fomo_ctx fomo_ctx;

const char* fomo_version(void);

/* Create a context on CUDA device `device`.  hbm_budget_bytes bounds what
 * the context may allocate (0 = 90% of the device's free memory). */
int fomo_ctx_create(int device, size_t hbm_budget_bytes, fomo_ctx** out);
int fomo_ctx_destroy(fomo_ctx* ctx);
const char* fomo_last_error(const fomo_ctx* ctx);
/* Bytes currently allocated by the context, and its budget. */
int fomo_ctx_memory(const fomo_ctx* ctx, size_t* used, size_t* budget);
/* Wait for all work the context issued on its own stream. */
int fomo_ctx_synchronize(fomo_ctx* ctx);

/* Page-lock a caller buffer so uploads/downloads run at full link speed
 * (cudaHostRegister); optional. */
int fomo_host_register(fomo_ctx* ctx, void* ptr, size_t bytes);
int fomo_host_unregister(fomo_ctx* ctx, void* ptr);

/* ---- snapshots: replaces DataCube ingestion (FoMoObject::setdata /
 * push_back_datapoint, fomo-object.cpp:137-162; DataCube::setdata,
 * fomo-datacube.cpp:256-279).  n points with coordinates in Mm, n_e in
 * cm^-3, T in K, v in m/s (variable order n, T, vx, vy, vz as in
 * example/example.cpp:51-57).  Uploads, builds the spatial index that
 * replaces the per-view Boost rtree (fomo-nearestneighbour.cpp:100) and keeps
 * both resident until fomo_snapshot_destroy.  z may be NULL for 2-D data
 * (the reference sets z = 0, nn:82). */
int fomo_snapshot_create(fomo_ctx* ctx, int64_t n, const float* x, const float* y, const float* z,
                         const float* n_e, const float* T, const float* vx, const float* vy, const float* vz,
                         int* id);
int fomo_snapshot_destroy(fomo_ctx* ctx, int id);
/* The same from arrays already in this device's memory (e.g. a simulation
 * running on the GPU): no host round trip.  The arrays are copied into the
 * snapshot's own storage on the context's stream, so work that writes them must
 * be complete before the call; they may be freed after it returns. */
int fomo_snapshot_create_device(fomo_ctx* ctx, int64_t n, const float* x, const float* y, const float* z,
                                const float* n_e, const float* T, const float* vx, const float* vy, const float* vz,
                                int* id);

/* ---- AMRVAC snapshots: replaces read_amrvac_dat_file (fomo-c/example/
 * example_mpi_amrvac/read_amrvac_files.cpp:685-715) and the FoMoObject it
 * fills point by point (fomo_from_amrvac, :228-299).  The data file's header,
 * tree and leaf blocks are parsed on the host; every cell's position and
 * primitive variables (n = rho n_unit, T = p / rho Teunit, v = m / rho V_unit
 * with V_unit = sqrt(2 k_B Teunit / m_p)) are computed on the device in the
 * reference's FP64 order and rounded to FP32 as its DataCube stores them; then
 * the snapshot is built as fomo_snapshot_create does.  Version 3 and 4 files
 * carry their own domain (amrvacpar may be NULL); older files need the
 * amrvac.par file, amrvac_version "old" (level-1 blocks x fastest) or
 * "gitlab" (Morton order), and gamma_eqparposition (the index of gamma among
 * the equation parameters).  L_unit: Mm per code length.  2-D data get z = 0. */
int fomo_snapshot_from_amrvac(fomo_ctx* ctx, const char* datfile, const char* amrvacpar, const char* amrvac_version,
                              int gamma_eqparposition, double n_unit, double Teunit, double L_unit, int* id);
/* The same conversion into caller host arrays of cap floats each (x, y, z,
 * n_e, T, vx, vy, vz in the reference's point order); x == NULL only returns
 * *npoints and *ndim.  It serves the C++ read_amrvac_dat_file of
 * include/FoMo-amrvac.h. */
int fomo_amrvac_points(fomo_ctx* ctx, const char* datfile, const char* amrvacpar, const char* amrvac_version,
                       int gamma_eqparposition, double n_unit, double Teunit, double L_unit, int64_t cap,
                       int64_t* npoints, int* ndim, float* x, float* y, float* z, float* n_e, float* T, float* vx,
                       float* vy, float* vz);

typedef struct {
  int64_t npoints;
  int grid_dims[3];
  float cell_edge;       /* Mm */
  float aabb[6];         /* minx, miny, minz, maxx, maxy, maxz */
  size_t device_bytes;
} fomo_snapshot_info;
int fomo_snapshot_get_info(fomo_ctx* ctx, int id, fomo_snapshot_info* info);

/* ---- G(T, n) tables: replaces readgoftfromchianti (fomo-CHIANTI.cpp:
 * 143-218).  logT (nt), logn (nrho), G (nrho*nt, T fastest).  ion and unit
 * are the header strings (the imaging check compares atoi(ion) with
 * lambda0, fomo-CHIANTI.cpp:278; a unit containing "DN" selects arcsec
 * grids and per-pixel scaling, fomo-nearestneighbour.cpp:254-265). */
int fomo_table_create(fomo_ctx* ctx, const char* ion, double lambda0, double atweight, const char* unit, int nt,
                      int nrho, const float* logT, const float* logn, const float* G, int* id);
/* Parse a CHIANTI G(T) text file exactly as readgoftfromchianti does. */
int fomo_table_load(fomo_ctx* ctx, const char* path, int* id);
int fomo_table_destroy(fomo_ctx* ctx, int id);
/* Header of a table: lambda0, atweight, nt, nrho, is_dn; ion/unit copied into
 * caller buffers of the given capacities (may be NULL). */
int fomo_table_get_info(fomo_ctx* ctx, int id, double* lambda0, double* atweight, int* nt, int* nrho, int* is_dn,
                        char* ion, int ion_cap, char* unit, int unit_cap);

/* Per-point emissivity of a snapshot under a table, in the snapshot's
 * original point order: eps and fwhm (Angstrom; 1 for imaging), as the
 * GoftCube that emissionfromdatacube returns (fomo-CHIANTI.cpp:228-322) and
 * FoMoObject::readgoftcube() exposes (fomo-object.cpp:71-74).  imaging selects
 * FoMo::Imaging.  Computed on the device (and cached for later renders). */
int fomo_emission(fomo_ctx* ctx, int snapshot, int table, int imaging, double abundratio, float* eps, float* fwhm);

/* Abundance renormalisation of a spectral line (fomo-CHIANTI.cpp:23-62,
 * 264-273): the element abundance relative to hydrogen in `abund_file` over the
 * same in `standard_file` (the abundances the G(T) tables were computed with,
 * e.g. CHIANTI's sun_coronal_2012_schmelz.abund).  Pass the result as a
 * request's abundratio.  The reference compares against a built-in copy of the
 * standard file that is empty at the point of use (fomo-CHIANTI.cpp:21), so
 * any file but "/empty" fails there; here the standard file is an argument.
 * ion: the table's ion string ("fe_12": element "fe").  ctx may be NULL. */
int fomo_abundance_ratio(fomo_ctx* ctx, const char* abund_file, const char* standard_file, const char* ion,
                         double* ratio);

/* Per-point Thomson scattering terms of a snapshot, in its original point
 * order: tot = n * total term, pol = n * polarised term, the GoftCube vars
 * that thomsonfromdatacube returns (fomo-thomson.cpp:60-92).  Computed on the
 * device (and cached for later Thomson renders). */
int fomo_thomson_emission(fomo_ctx* ctx, int snapshot, float* tot, float* pol);

/* ---- one render request: the arguments of RenderWithNearestNeighbour /
 * RenderWithThomson (FoMo-internal.h:23-27) for one (l, b) view. */
typedef struct {
  int snapshot;          /* fomo_snapshot_create id */
  int table;             /* fomo_table_* id (ignored for Thomson) */
  int method;            /* FOMO_METHOD_NN, FOMO_METHOD_THOMSON or FOMO_METHOD_PROJECTION */
  int nx, ny, nz;        /* x_pixel, y_pixel, z_pixel (nx, ny >= 2) */
  int nlambda;           /* lambda_pixel: 1 = imaging, > 1 = spectroscopic (fomo-object.cpp:381-384) */
  double l, b;           /* view angles in radians */
  double lambda_width;   /* spectral window in m/s (RenderCube units, fomo-rendercube.cpp:67-85) */
  double abundratio;     /* abundance renormalisation (1.0 = built-in abundances) */
} fomo_request;

/* Per-view quantities of a finished render (what the reference computes in
 * nearestneighbourinterpolation: extents nn:103-108, maxdistance nn:138,
 * path length and pixel area nn:235-262). */
typedef struct {
  double minx, maxx, miny, maxy, minz, maxz;
  double maxdistance, deltaz, pathlength, apix, scale;
  double lambda_width_A; /* lambda_width * lambda0 / c */
  double lambda0;
  int is_dn;
  int observation_type;  /* FOMO_OBS_* */
} fomo_view_info;

/* Render one view into a host cube of ny*nx*nlambda floats.  out_nn_idx
 * (nullable) receives ny*nx*nz original point indices of the nearest
 * neighbour of every LOS sample (-1 where no point lies in the box).
 * Replaces nearestneighbourinterpolation (fomo-nearestneighbour.cpp:31-281)
 * / thomsoninterpolation (fomo-thomson.cpp:94-367) plus the emissivity
 * stage the reference reruns on every render (fomo-object.cpp:389-400);
 * here the emissivity is computed once per (snapshot, table) and cached. */
int fomo_render(fomo_ctx* ctx, const fomo_request* req, float* out_cube, int32_t* out_nn_idx,
                fomo_view_info* info);

/* Same, writing device buffers (caller-owned device memory) asynchronously on
 * `stream`; info (nullable) is filled after a synchronize on that stream. */
int fomo_render_device(fomo_ctx* ctx, const fomo_request* req, float* d_out_cube, int32_t* d_out_nn_idx,
                       fomo_view_info* info, void* stream);

/* Render one NearestNeighbour request into a caller device buffer WITHOUT
 * allocating anything.  No counterpart in the reference: it exists for callers
 * that must not allocate device memory while they render (an application
 * that owns a fixed device-memory pool and forbids allocation in its frame
 * loop, or a real-time path where cudaMalloc/cudaFree would synchronise the
 * device).  The per-render working memory lives in one static device array of
 * about 1.2 MB that every GPU loading this library holds until exit; hence the
 * limits nz <= 4096, nx + ny <= 8192, nlambda <= 256 (larger requests return
 * FOMO_EINVAL).  The snapshot, the table and the emissivity of the pair must
 * already be resident (call fomo_emission or any regular render once first).
 * The first call on a device looks up the array's address, so make it before
 * any stream capture.  All calls share the array: calls that overlap on the
 * GPU (different streams) race and must be serialised.  The cube matches
 * fomo_render's to FP32 summation order (the deferred samples' emission is
 * added with atomics here).  Asynchronous on `stream` (NULL = the context's
 * stream). */
int fomo_render_noalloc(fomo_ctx* ctx, const fomo_request* req, float* d_out_cube, void* stream);

/* Batched render: many views / lines / requests in one persistent launch.
 * Requests that share snapshot, method, angles and resolution share their
 * neighbour lookups (one lookup per LOS sample feeds every line).  outs[r]
 * is a host cube for request r; infos (nullable) has nreq entries.
 * Replaces the per-view loop of RenderWithNearestNeighbour (nn:285-306). */
int fomo_render_batch(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* outs,
                      fomo_view_info* infos);
/* Device-buffer form; asynchronous on `stream`. */
int fomo_render_batch_device(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_outs,
                             void* stream);

/* Batched render captured as a CUDA graph and replayed: the first call for a
 * given batch shape captures, later calls with the same shape (count, sizes,
 * methods) replay with the new angles/tables.  Device outputs. */
int fomo_render_batch_graph(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_outs, void* stream);

/* Ray-tile autotuner for the march (tile shape and CTAs per SM), measured on
 * the given batch; the choice is cached per workload class and, when
 * cache_path is non-NULL, persisted there as text. */
int fomo_autotune(fomo_ctx* ctx, const fomo_request* reqs, int nreq, const char* cache_path);
/* Force a ray tile (0,0 = automatic) and CTAs-per-SM cap (0 = occupancy max). */
int fomo_set_march_config(fomo_ctx* ctx, int tile_w, int tile_h, int blocks_per_sm);

/* Timing of the last render's march kernel (CUDA events on its stream), ms. */
int fomo_last_march_ms(fomo_ctx* ctx, float* ms);

/* Profiling of later direct renders (not graph replays): CUDA-event times of
 * each of the march's kernels, and search counters.  kernel_timing / counters:
 * 1 on, 0 off.  Counting adds atomics to the kernels; timing adds events
 * between them.  No counterpart in the reference, whose only instrumentation
 * is a progress bar (fomo-nearestneighbour.cpp:141,228). */
#define FOMO_KERNEL_SEARCH 0    /* neighbour search (positions to the buffer) */
#define FOMO_KERNEL_SPLIT 1     /* segments whose candidate list overflowed, searched in parts */
#define FOMO_KERNEL_DEFERRED 2  /* samples the search left, one lane each */
#define FOMO_KERNEL_HARD 3      /* deferred samples over a lane's budget, one warp each */
#define FOMO_KERNEL_EMISSION 4  /* emission pass: binning from the stored neighbours */
#define FOMO_KERNEL_FUSED 5     /* fused search + emission (the no-allocation path) */
#define FOMO_KERNEL_FAR 6       /* deferred samples of a record searched together, one warp per 32 */
#define FOMO_KERNEL_COUNT 7
#define FOMO_COUNTER_SEGMENTS 0      /* 64-sample segments searched */
#define FOMO_COUNTER_CANDIDATES 1    /* candidates gathered */
#define FOMO_COUNTER_ROWS 2          /* cell rows visited by the gather */
#define FOMO_COUNTER_POINTS_LOADED 3 /* points loaded by the gather */
#define FOMO_COUNTER_NOT_GATHERED 4  /* segments or parts whose capsule overflowed */
#define FOMO_COUNTER_FALLBACKS 5     /* samples left to the deferred pass */
#define FOMO_COUNTER_SAMPLES 6       /* LOS samples searched */
#define FOMO_COUNTER_SCANNED 7       /* candidates scanned by samples */
#define FOMO_COUNTER_TIES 8          /* samples re-ranked in FP64 */
#define FOMO_COUNTER_FB_NOCAND 9     /* left: no in-box candidate within the coverage radius */
#define FOMO_COUNTER_FB_FAR 10       /* left: best candidate beyond the coverage radius */
#define FOMO_COUNTER_FB_AMBIGUOUS 11 /* left: a candidate within a few ulp of a box face */
#define FOMO_COUNTER_DEFERRED 12     /* samples searched by the deferred pass */
#define FOMO_COUNTER_DEFERRED_RECS 13 /* deferred-sample records */
#define FOMO_COUNTER_HARD 14         /* deferred samples searched by a whole warp */
#define FOMO_COUNTER_RUNS 15         /* runs of equal neighbours binned by the spectral emission pass */
#define FOMO_COUNTER_EX2 16          /* ex2 evaluations of the spectral emission pass */
#define FOMO_COUNTER_FAR_GROUPS 17   /* record halves searched together by the far pass */
#define FOMO_COUNTER_FAR 18          /* deferred samples the far pass resolved */
#define FOMO_COUNTER_COUNT 19
int fomo_set_profiling(fomo_ctx* ctx, int kernel_timing, int counters);
/* The last direct render's kernel times (ms) summed per kind (kernel_ms[k] for
 * FOMO_KERNEL_k, k < nk), and the counters accumulated since they were turned
 * on (counters[k] for FOMO_COUNTER_k, k < nc; the read zeroes them).  Either
 * array may be NULL. */
int fomo_profile_read(fomo_ctx* ctx, float* kernel_ms, int nk, uint64_t* counters, int nc);

/* Ceilings of the march's roofline, measured on the context's device (the
 * march keeps the snapshot in L2 and is bound by L2 latency, instruction issue
 * and the SFU, not by HBM): the L2 read bandwidth (a 64 MB buffer streamed
 * with L2-only loads), the rate of random 16-byte gathers that hit L2 (useful
 * bytes, the access pattern of the march's candidate and payload loads), and
 * the SFU's ex2.approx.f32 throughput (one per lambda bin, line and run of
 * the emission pass).  No counterpart in the reference: a measurement utility
 * for the benchmark.  Allocates and frees a 64 MB buffer. */
typedef struct {
  double l2_read_gbs;
  double l2_gather_gbs;
  double ex2_per_s;
  int sm_count;
} fomo_ceilings;
int fomo_measure_ceilings(fomo_ctx* ctx, fomo_ceilings* out);

/* ---- render server: continuous batching of requests as they arrive. */
typedef struct fomo_server fomo_server;
typedef struct {
  int device;
  size_t hbm_budget_bytes;  /* admission limit for in-flight request buffers (0 = 50% of free) */
  int max_inflight;         /* requests resident on the device at once (0 = 64) */
} fomo_server_config;

typedef struct {
  double t_submit, t_admit, t_start, t_done; /* seconds, server clock */
  int status;                                /* FOMO_OK or error */
} fomo_request_stats;

/* The server creates its own context on config->device.  Snapshots and
 * tables are created through fomo_server_context() before submitting. */
int fomo_server_create(const fomo_server_config* config, fomo_server** out);
fomo_ctx* fomo_server_context(fomo_server* srv);
/* Submit (thread-safe).  The result cube is written to out_host when the
 * request completes.  Requests larger than the HBM budget fail with
 * FOMO_EADMISSION at submit. */
int fomo_server_submit(fomo_server* srv, const fomo_request* req, float* out_host, uint64_t* ticket);
int fomo_server_wait(fomo_server* srv, uint64_t ticket, double timeout_s, fomo_request_stats* stats);
/* Cancel (thread-safe): a queued request is dropped; a running one completes
 * with FOMO_ECANCELLED and its cube is not delivered.  When every request of
 * a running batch is cancelled, the batch is halted on the device: its march
 * kernels take no further rays (a stop word read before each ray). */
int fomo_server_cancel(fomo_server* srv, uint64_t ticket);
/* Drain, stop the scheduler thread and free the context. */
int fomo_server_destroy(fomo_server* srv);
const char* fomo_server_last_error(fomo_server* srv);

#ifdef __cplusplus
}
#endif
#endif
