/*
 * fomo_oracle -- CPU restatement of FoMo-C's nearest-neighbour render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against; the product never links, loads or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Every function restates the reference's algorithm step by step, with the
 * reference's FP32 storage points and FP64 arithmetic order, citing the
 * reference file:line it follows (paths relative to the FoMo repository).
 * It is itself checked against the reference's own sources, compiled here
 * with header shims for the absent GSL and Boost (oracle/Makefile `ref`),
 * through golden vectors committed under tests/golden/.
 *
 * Build: gcc -O2 -ffp-contract=off (no FMA contraction: the reference's FP64
 * expression roundings must be reproduced exactly on aarch64 as on x86-64).
 */
#ifndef FOMO_ORACLE_H
#define FOMO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Physical constants.  c, k_B, m_p as shipped by GSL's gsl_const_mksa.h
 * (fomo-CHIANTI.cpp:17-19); alpha (fomo-CHIANTI.cpp:16); Mm per arcsec
 * (FoMo-internal.h:4); Thomson constants (fomo-thomson.cpp:31-34). */
#define FO_SPEED_OF_LIGHT 2.99792458e8
#define FO_BOLTZMANN 1.3806504e-23
#define FO_MASS_PROTON 1.67262158e-27
#define FO_ALPHA 1.0645
#define FO_MM_PER_ARCSEC 0.715
#define FO_RSUN 695.7
#define FO_LIMB_U 0.58
#define FO_ELECTRON_RADIUS 2.8179e-13
#define FO_IRRADIANCE 2.8e10

/* Status codes (the reference exits instead; see fomo-CHIANTI.cpp:126-197,278). */
#define FO_OK 0
#define FO_ENOFILE (-1)   /* "no CHIANTI G(T) file exists" */
#define FO_ETABLE (-2)    /* "CHIANTI table not read in properly!" */
#define FO_ECAP (-3)      /* caller's buffers too small; sizes returned */
#define FO_EIMAGING (-4)  /* "GOFT table is not correct!" (imaging check) */
#define FO_EARG (-5)

/* Per-view quantities, as doubles, in this order. */
enum {
  FO_V_MINX, FO_V_MAXX, FO_V_MINY, FO_V_MAXY, FO_V_MINZ, FO_V_MAXZ,
  FO_V_MAXDIST, FO_V_DELTAZ, FO_V_PATHLENGTH, FO_V_APIX, FO_V_SCALE, FO_V_LAMBDA_WIDTH_A,
  FO_V_COUNT
};

/* readgoftfromchianti (fomo-CHIANTI.cpp:143-218).  hdr = {lambda0, atweight,
 * minlevel, maxlevel}.  logT has nt entries, logn nrho, G nrho*nt (T fastest). */
int fo_table_read(const char* path, char* ion, int ion_cap, char* unit, int unit_cap, double* hdr, int* nt,
                  int* nrho, float* logT, float* logn, float* G, long cap);

/* emissionfromdatacube (fomo-CHIANTI.cpp:228-322) with goft (:64-121) and
 * linefwhm (:220-226).  imaging selects FoMo::Imaging.  ion is the table's ion
 * string (imaging check :278).  Outputs eps and fwhm (Angstrom, or 1 for imaging). */
int fo_emission(long n, const float* ne, const float* T, int nt, int nrho, const float* logT, const float* logn,
                const float* G, double lambda0, double atweight, const char* ion, int imaging, double abundratio,
                float* eps, float* fwhm);

/* thomsonfromdatacube (fomo-thomson.cpp:39-92): tot = n*totterm, pol = n*polterm. */
void fo_thomson_emission(long n, const float* x, const float* y, const float* z, const float* ne, float* tot,
                         float* pol);

/* nearestneighbourinterpolation (fomo-nearestneighbour.cpp:31-281) for one
 * view, rows [row0, row1) of the image.  mode bit 0 clear: FP64
 * accumulation (the oracle); set: FP32 accumulation exactly as the
 * reference's float `intens`.  mode bit 1 set: brute-force O(N) neighbour
 * search instead of the grid (to check the grid search).  cube: (row1-row0)*nx*L doubles, already scaled (:267).
 * nnidx (nullable): (row1-row0)*nx*nz original point indices, -1 = none.
 * view: FO_V_COUNT doubles. */
int fo_nn_render(long n, const float* x, const float* y, const float* z, const float* peak, const float* fwhm,
                 const float* vx, const float* vy, const float* vz, double lambda0, double l, double b, int nx,
                 int ny, int nz, int L, double lambda_width, int is_dn, int mode, int nthreads, int row0, int row1,
                 double* cube, int32_t* nnidx, double* view);

/* thomsoninterpolation (fomo-thomson.cpp:94-367) for one view (pB only),
 * rows [row0, row1).  The reference takes the first of up to 5 returned
 * neighbours; its order is Boost-version dependent, and here it is the
 * nearest (lowest index on exact ties). */
int fo_thomson_render(long n, const float* x, const float* y, const float* z, const float* tot, const float* pol,
                      double l, double b, int nx, int ny, int nz, int mode, int nthreads, int row0, int row1,
                      double* cube, int32_t* nnidx, double* view);

/* Projection render (fomo-projection.cpp:17-193): every point adds its
 * emission to the pixel nearest its projection, j = round((x' - minx)(nx-1) /
 * (maxx - minx)), i likewise; spectroscopic points add their Gaussian to all L
 * bins (no zero-peak guard, :145).  cube: ny*nx*L doubles.  pix (nullable): the
 * pixel index i*nx + j of every point.  mode bit 0: accumulate in FP32 in point
 * order as the reference does single-threaded.  view: FO_V_COUNT doubles
 * (maxdistance unused, 0). */
int fo_projection_render(long n, const float* x, const float* y, const float* z, const float* peak,
                         const float* fwhm, const float* vx, const float* vy, const float* vz, double lambda0,
                         double l, double b, int nx, int ny, int nz, int L, double lambda_width, int is_dn, int mode,
                         double* cube, int32_t* pix, double* view);

/* The per-element x, y (and lambda for L > 1) grids of the render cube
 * (fomo-nearestneighbour.cpp:152-153,209-211,254-260), from a view record. */
void fo_render_grid(int nx, int ny, int L, const double* view, double lambda0, int is_dn, float* gx, float* gy,
                    float* glambda);

/* Brute-force reference query for testing the grid search: nearest point
 * strictly inside the float box, FP64 Boost distance, lowest index on ties. */
int32_t fo_bruteforce_query(long n, const float* x, const float* y, const float* z, const float* target,
                            const float* lo, const float* hi);

#ifdef __cplusplus
}
#endif
#endif
