/*
 * fomo_oracle.c -- CPU restatement of FoMo-C's nearest-neighbour render path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): see fomo_oracle.h.  Paths cited as
 * file:line are relative to the FoMo repository (fomo-c/src/...).
 *
 * Precision contract: every value the reference stores as float (coordinates,
 * table, eps, fwhm, targets, box corners) is stored as float here, rounded at
 * the same points; every expression the reference evaluates in double is
 * evaluated in double with the same operand order.  Accumulation is FP64
 * (mode 0) or, in mirror mode (mode 1), float exactly as the reference's
 * `intens` vector.  Compile with -ffp-contract=off.
 *
 * Boost.Geometry's rtree query `nearest(target,k) && within(box)` is restated
 * as: the point(s) strictly inside the float box with the smallest squared
 * distance computed in double in Boost's order d_z^2 + (d_y^2 + d_x^2), ties
 * to the lowest index.  A uniform grid with ring search finds it exactly
 * (the ring bound is conservative); fo_bruteforce_query is the O(N) check.
 */
#include "fomo_oracle.h"

#include <ctype.h>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* a3: table parser (fomo-CHIANTI.cpp:143-218)                               */
/* ------------------------------------------------------------------------ */

typedef struct {
  const char* p;
  const char* end;
} cursor;

static void skip_ws(cursor* c) {
  while (c->p < c->end && isspace((unsigned char)*c->p)) c->p++;
}

static int next_token(cursor* c, char* buf, int cap) {
  skip_ws(c);
  int n = 0;
  while (c->p < c->end && !isspace((unsigned char)*c->p)) {
    if (n + 1 < cap) buf[n++] = *c->p;
    c->p++;
  }
  buf[n] = 0;
  return n > 0;
}

static int next_double(cursor* c, double* v) {
  char tok[128];
  if (!next_token(c, tok, sizeof tok)) return 0;
  char* e = NULL;
  *v = strtod(tok, &e);
  return e != tok;
}

static void read_line(cursor* c, char* buf, int cap) {
  int n = 0;
  while (c->p < c->end && *c->p != '\n') {
    if (n + 1 < cap) buf[n++] = *c->p;
    c->p++;
  }
  if (c->p < c->end) c->p++;
  buf[n] = 0;
}

int fo_table_read(const char* path, char* ion, int ion_cap, char* unit, int unit_cap, double* hdr, int* nt_out,
                  int* nrho_out, float* logT, float* logn, float* G, long cap) {
  FILE* f = fopen(path, "rb");
  if (!f) return FO_ENOFILE;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  char* text = (char*)malloc((size_t)sz + 1);
  if (!text) {
    fclose(f);
    return FO_EARG;
  }
  size_t got = fread(text, 1, (size_t)sz, f);
  fclose(f);
  text[got] = 0;
  cursor c = {text, text + got};
  char tok[256];
  double lambda0 = 0, atweight = 0, minlevel = 0, maxlevel = 0;
  next_token(&c, tok, sizeof tok); /* in >> ion */
  if (ion && ion_cap > 0) snprintf(ion, (size_t)ion_cap, "%s", tok);
  next_double(&c, &lambda0);
  next_double(&c, &atweight);
  next_double(&c, &minlevel);
  next_double(&c, &maxlevel);
  char line[1024];
  read_line(&c, line, sizeof line); /* in.ignore(..., '\n') */
  read_line(&c, line, sizeof line); /* getline(in, unitstr) */
  if (unit && unit_cap > 0) snprintf(unit, (size_t)unit_cap, "%s", line);
  read_line(&c, line, sizeof line); /* getline(in, chiantiversion) */
  double dnrho = 0, dnt = 0;
  next_double(&c, &dnrho);
  next_double(&c, &dnt);
  int nrho = (int)dnrho, nt = (int)dnt;
  if (hdr) {
    hdr[0] = lambda0;
    hdr[1] = atweight;
    hdr[2] = minlevel;
    hdr[3] = maxlevel;
  }
  *nt_out = nt;
  *nrho_out = nrho;
  if (nt <= 0 || nrho <= 0) {
    free(text);
    return FO_ETABLE;
  }
  if ((long)nt * (long)nrho > cap || nt > cap || nrho > cap) {
    free(text);
    return FO_ECAP;
  }
  for (int i = 0; i < nt; ++i) {
    double v = 0;
    next_double(&c, &v);
    logT[i] = (float)v;
  }
  /* while (in >> templogrho) { for i<nt: in >> field } ; then size check */
  long rows = 0;
  double v;
  while (next_double(&c, &v)) {
    if (rows < nrho) logn[rows] = (float)v;
    for (int i = 0; i < nt; ++i) {
      double fv = 0;
      if (!next_double(&c, &fv)) fv = 0;
      if (rows < nrho) G[rows * nt + i] = (float)fv;
    }
    rows++;
  }
  free(text);
  if (rows != nrho) return FO_ETABLE;
  return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* a4-a6: G(T,n) interpolation and emissivity                               */
/* ------------------------------------------------------------------------ */

/* goft (fomo-CHIANTI.cpp:64-121): index arithmetic in float (both operands are
 * float), linear interpolation in logT in double on the nearest logn row. */
static float goft_one(float lT, float lr, int nt, int nrho, const float* logT, const float* logn, const float* G) {
  float T0 = logT[0], T1 = logT[1];
  float r0 = logn[0], r1 = logn[1]; /* rhogrid.at(0), rhogrid.at(nt) */
  int floortemp = (int)floorf((lT - T0) / (T1 - T0));
  int ceiltemp = floortemp + 1;
  int rhoindex = (int)roundf((lr - r0) / (r1 - r0));
  if (floortemp < 0 || rhoindex < 0 || ceiltemp > nt - 1 || rhoindex > nrho - 1) return 0.0f;
  int goftindex = rhoindex * nt + ceiltemp;
  double x1 = logT[ceiltemp];
  double y1 = G[goftindex];
  double x2 = logT[floortemp];
  double y2 = G[goftindex - 1];
  double res = ((double)lT - x1) * (y2 - y1) / (x2 - x1) + y1;
  return (float)res;
}

int fo_emission(long n, const float* ne, const float* T, int nt, int nrho, const float* logT, const float* logn,
                const float* G, double lambda0, double atweight, const char* ion, int imaging, double abundratio,
                float* eps, float* fwhm) {
  if (imaging) {
    /* fomo-CHIANTI.cpp:278: atoi(ion) != int(lambda0+0.5) -> exit */
    if (atoi(ion ? ion : "") != (int)(lambda0 + 0.5)) return FO_EIMAGING;
  }
  /* linefwhm constant (fomo-CHIANTI.cpp:224) */
  const double cw =
      2 * sqrt(2 * log(2)) * sqrt(FO_BOLTZMANN / FO_MASS_PROTON / atweight) * lambda0 / FO_SPEED_OF_LIGHT;
  const double normaliseconst = imaging ? 1.0 : 1. / FO_ALPHA;
  const double k = normaliseconst * (imaging ? 1.0 : abundratio);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    /* FoMo::log10 (fomo-operations.cpp:63-84): std::log10(float), <=0 -> 0 */
    float logrho = ne[i] <= 0 ? 0.0f : log10f(ne[i]);
    float Tv = T[i];
    float lT = Tv <= 0 ? 0.0f : log10f(Tv);
    float g = goft_one(lT, logrho, nt, nrho, logT, logn, G);
    float w = imaging ? 1.0f : (float)(cw * (double)sqrtf(Tv));
    float a = (float)(2. * (double)logrho);         /* operator*(2., logrho) */
    float b = (float)pow(10., (double)a);           /* FoMo::pow(10., .)     */
    float c = b * g;                                /* operator*(vec, vec)   */
    float d = (float)(k * (double)c);               /* operator*(double,vec) */
    eps[i] = d / w;                                 /* operator/(vec, vec)   */
    fwhm[i] = w;
  }
  return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* a18: Thomson coefficients (fomo-thomson.cpp:39-92)                       */
/* ------------------------------------------------------------------------ */

static void thomson_geom(float r, float* totterm, float* polterm) {
  const double pi = M_PI;
  const double U = FO_LIMB_U;
  float sinomega = (float)(FO_RSUN / (double)r);
  float coeff = (float)(0.5 * pi * (FO_ELECTRON_RADIUS * FO_ELECTRON_RADIUS) * FO_IRRADIANCE);
  float ss = sinomega * sinomega;
  float cs = 1 - ss;
  float co = (float)sqrt((double)cs);
  float lt = (float)log((1. + (double)sinomega) / (double)co);
  float a = co * ss;
  float b = (float)((-1.0 / 8.0) *
                    (1.0 - 3.0 * (double)ss - (double)cs * ((1.0 + 3.0 * (double)ss) / (double)sinomega) * (double)lt));
  float c = (float)((4.0 / 3.0) - (double)co - (double)(co * cs) / 3.0);
  float d = (float)((1.0 / 8.0) *
                    (5.0 + (double)ss - (double)cs * ((5.0 - (double)ss) / (double)sinomega) * (double)lt));
  *polterm = (float)((double)coeff * (1. / (1. - U / 3.)) * ((double)a + U * (double)(b - a)));
  *totterm = (float)((double)coeff * (1. / (1. - U / 3.)) * (2. * ((double)c + U * (double)(d - c))));
}

void fo_thomson_emission(long n, const float* x, const float* y, const float* z, const float* ne, float* tot,
                         float* pol) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    double px = x[i], py = y[i], pz = z[i];
    float r = (float)sqrt(px * px + py * py + pz * pz);
    float tt, pt;
    thomson_geom(r, &tt, &pt);
    tot[i] = ne[i] * tt;
    pol[i] = ne[i] * pt;
  }
}

/* ------------------------------------------------------------------------ */
/* Exact box-limited nearest-neighbour search (replaces the Boost rtree)    */
/* ------------------------------------------------------------------------ */

typedef struct {
  double ox, oy, oz, h, inv_h;
  int dx, dy, dz;
  long* start;  /* cell -> first slot, dx*dy*dz+1 entries */
  int32_t* ids; /* point ids in cell order */
  const float *x, *y, *z;
} fo_grid;

static int cell_of(double v, double o, double inv_h, int dim) {
  double c = floor((v - o) * inv_h);
  if (!(c >= 0)) return 0; /* also catches NaN */
  if (c > dim - 1) return dim - 1;
  return (int)c;
}

static int grid_build(fo_grid* g, long n, const float* x, const float* y, const float* z) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (long i = 0; i < n; ++i) {
    double v[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; ++d) {
      if (v[d] < lo[d]) lo[d] = v[d];
      if (v[d] > hi[d]) hi[d] = v[d];
    }
  }
  if (n == 0) {
    lo[0] = lo[1] = lo[2] = 0;
    hi[0] = hi[1] = hi[2] = 1;
  }
  double ext[3];
  double vol = 1.0;
  int ndim = 0;
  double maxext = 0;
  for (int d = 0; d < 3; ++d) {
    ext[d] = hi[d] - lo[d];
    if (ext[d] > maxext) maxext = ext[d];
  }
  for (int d = 0; d < 3; ++d) {
    if (ext[d] > 1e-9 * (maxext > 0 ? maxext : 1)) {
      vol *= ext[d];
      ndim++;
    }
  }
  double h = ndim ? pow(vol * 2.0 / (double)(n > 0 ? n : 1), 1.0 / ndim) : 1.0;
  if (!(h > 0)) h = 1.0;
  int dims[3];
  for (;;) {
    long cells = 1;
    for (int d = 0; d < 3; ++d) {
      double k = ceil(ext[d] / h);
      if (k < 1) k = 1;
      if (k > 4096) k = 4096;
      dims[d] = (int)k;
      cells *= dims[d];
    }
    if (cells <= 4 * n + 64) break;
    h *= 1.25;
  }
  g->ox = lo[0];
  g->oy = lo[1];
  g->oz = lo[2];
  g->h = h;
  g->inv_h = 1.0 / h;
  g->dx = dims[0];
  g->dy = dims[1];
  g->dz = dims[2];
  long ncell = (long)dims[0] * dims[1] * dims[2];
  g->start = (long*)calloc((size_t)ncell + 1, sizeof(long));
  g->ids = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  long* cellof = (long*)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
  if (!g->start || !g->ids || !cellof) {
    free(g->start);
    free(g->ids);
    free(cellof);
    return FO_EARG;
  }
  for (long i = 0; i < n; ++i) {
    int cx = cell_of(x[i], g->ox, g->inv_h, g->dx);
    int cy = cell_of(y[i], g->oy, g->inv_h, g->dy);
    int cz = cell_of(z[i], g->oz, g->inv_h, g->dz);
    long c = ((long)cz * g->dy + cy) * g->dx + cx;
    cellof[i] = c;
    g->start[c + 1]++;
  }
  for (long c = 0; c < ncell; ++c) g->start[c + 1] += g->start[c];
  long* fill = (long*)malloc(sizeof(long) * (size_t)ncell);
  memcpy(fill, g->start, sizeof(long) * (size_t)ncell);
  for (long i = 0; i < n; ++i) g->ids[fill[cellof[i]]++] = (int32_t)i;
  free(fill);
  free(cellof);
  g->x = x;
  g->y = y;
  g->z = z;
  return FO_OK;
}

static void grid_free(fo_grid* g) {
  free(g->start);
  free(g->ids);
}

/* Boost comparable distance: d_z^2 + (d_y^2 + d_x^2) in double. */
static inline double boost_dist2(float px, float py, float pz, float tx, float ty, float tz) {
  double dx = (double)px - (double)tx;
  double dy = (double)py - (double)ty;
  double dz = (double)pz - (double)tz;
  double sx = dx * dx;
  double sy = dy * dy;
  double sz = dz * dz;
  return sz + (sy + sx);
}

static inline void scan_cell(const fo_grid* g, long c, const float* t, const float* lo, const float* hi,
                             double* best, int32_t* bi) {
  for (long s = g->start[c]; s < g->start[c + 1]; ++s) {
    int32_t id = g->ids[s];
    float px = g->x[id], py = g->y[id], pz = g->z[id];
    if (!(lo[0] < px && px < hi[0] && lo[1] < py && py < hi[1] && lo[2] < pz && pz < hi[2])) continue;
    double d = boost_dist2(px, py, pz, t[0], t[1], t[2]);
    if (d < *best || (d == *best && id < *bi)) {
      *best = d;
      *bi = id;
    }
  }
}

/* Nearest point strictly inside (lo, hi), FP64 Boost distance, lowest id on ties. */
static int32_t grid_query(const fo_grid* g, const float* t, const float* lo, const float* hi) {
  if (!(lo[0] < hi[0] && lo[1] < hi[1] && lo[2] < hi[2])) return -1;
  int b0[3], b1[3], c[3];
  const double o[3] = {g->ox, g->oy, g->oz};
  const int dim[3] = {g->dx, g->dy, g->dz};
  for (int d = 0; d < 3; ++d) {
    b0[d] = cell_of(lo[d], o[d], g->inv_h, dim[d]);
    b1[d] = cell_of(hi[d], o[d], g->inv_h, dim[d]);
    c[d] = cell_of(t[d], o[d], g->inv_h, dim[d]);
    if (c[d] < b0[d]) c[d] = b0[d];
    if (c[d] > b1[d]) c[d] = b1[d];
  }
  double best = DBL_MAX;
  int32_t bi = -1;
  for (int s = 0;; ++s) {
    if (s > 0 && bi >= 0) {
      double lb = (double)(s - 1) * g->h * (1.0 - 1e-9);
      if (lb > 0 && lb * lb > best) break;
    }
    if (c[0] - s < b0[0] && c[0] + s > b1[0] && c[1] - s < b0[1] && c[1] + s > b1[1] && c[2] - s < b0[2] &&
        c[2] + s > b1[2])
      break;
    int z0 = c[2] - s < b0[2] ? b0[2] : c[2] - s, z1 = c[2] + s > b1[2] ? b1[2] : c[2] + s;
    int y0 = c[1] - s < b0[1] ? b0[1] : c[1] - s, y1 = c[1] + s > b1[1] ? b1[1] : c[1] + s;
    for (int kz = z0; kz <= z1; ++kz) {
      int onz = (kz == c[2] - s || kz == c[2] + s);
      for (int jy = y0; jy <= y1; ++jy) {
        int ony = (jy == c[1] - s || jy == c[1] + s);
        long rowbase = ((long)kz * g->dy + jy) * g->dx;
        if (onz || ony) {
          int x0 = c[0] - s < b0[0] ? b0[0] : c[0] - s, x1 = c[0] + s > b1[0] ? b1[0] : c[0] + s;
          for (int ix = x0; ix <= x1; ++ix) scan_cell(g, rowbase + ix, t, lo, hi, &best, &bi);
        } else {
          if (c[0] - s >= b0[0]) scan_cell(g, rowbase + c[0] - s, t, lo, hi, &best, &bi);
          if (s > 0 && c[0] + s <= b1[0]) scan_cell(g, rowbase + c[0] + s, t, lo, hi, &best, &bi);
        }
      }
    }
  }
  return bi;
}

int32_t fo_bruteforce_query(long n, const float* x, const float* y, const float* z, const float* t, const float* lo,
                            const float* hi) {
  double best = DBL_MAX;
  int32_t bi = -1;
  for (long i = 0; i < n; ++i) {
    float px = x[i], py = y[i], pz = z[i];
    if (!(lo[0] < px && px < hi[0] && lo[1] < py && py < hi[1] && lo[2] < pz && pz < hi[2])) continue;
    double d = boost_dist2(px, py, pz, t[0], t[1], t[2]);
    if (d < best || (d == best && (int32_t)i < bi)) {
      best = d;
      bi = (int32_t)i;
    }
  }
  return bi;
}

/* ------------------------------------------------------------------------ */
/* a8-a16: one view of the NN render                                        */
/* ------------------------------------------------------------------------ */

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* Stage A extents (fomo-nearestneighbour.cpp:76-108) and LOS velocity (:87-90). */
static void nn_extents(long n, const float* x, const float* y, const float* z, const float* vx, const float* vy,
                       const float* vz, double cb, double sb, double cl, double sl, double* ext, double* losvel) {
  double mnx = DBL_MAX, mxx = -DBL_MAX, mny = DBL_MAX, mxy = -DBL_MAX, mnz = DBL_MAX, mxz = -DBL_MAX;
#pragma omp parallel for schedule(static) reduction(min : mnx, mny, mnz) reduction(max : mxx, mxy, mxz)
  for (long i = 0; i < n; ++i) {
    double gx = x[i], gy = y[i], gz = z[i];
    double xa = gx * cb * cl - gy * cb * sl - gz * sb;
    double ya = gx * sl + gy * cl;
    double za = gx * sb * cl - gy * sb * sl + gz * cb;
    if (xa < mnx) mnx = xa;
    if (xa > mxx) mxx = xa;
    if (ya < mny) mny = ya;
    if (ya > mxy) mxy = ya;
    if (za < mnz) mnz = za;
    if (za > mxz) mxz = za;
    if (losvel) {
      double u0 = sb * cl, u1 = -sb * sl, u2 = cb;
      double acc = 0.0;
      acc = acc + u0 * (double)vx[i];
      acc = acc + u1 * (double)vy[i];
      acc = acc + u2 * (double)vz[i];
      losvel[i] = acc;
    }
  }
  ext[0] = mnx;
  ext[1] = mxx;
  ext[2] = mny;
  ext[3] = mxy;
  ext[4] = mnz;
  ext[5] = mxz;
}

static double std_max(double a, double b) { return (a < b) ? b : a; }

int fo_nn_render(long n, const float* x, const float* y, const float* z, const float* peak, const float* fwhm,
                 const float* vx, const float* vy, const float* vz, double lambda0, double l, double b, int nx,
                 int ny, int nz, int L, double lambda_width, int is_dn, int mode, int nthreads, int row0, int row1,
                 double* cube, int32_t* nnidx, double* view) {
  if (n <= 0 || nx < 2 || ny < 2 || nz < 1 || L < 1 || row0 < 0 || row1 > ny || row0 > row1) return FO_EARG;
  set_threads(nthreads);
  const double cb = cos(b), sb = sin(b), cl = cos(l), sl = sin(l);
  double* losvel = (double*)malloc(sizeof(double) * (size_t)n);
  if (!losvel) return FO_EARG;
  double ext[6];
  nn_extents(n, x, y, z, vx, vy, vz, cb, sb, cl, sl, ext, losvel);
  const double minx = ext[0], maxx = ext[1], miny = ext[2], maxy = ext[3], minz = ext[4], maxz = ext[5];
  fo_grid g;
  if (grid_build(&g, n, x, y, z) != FO_OK) {
    free(losvel);
    return FO_EARG;
  }
  const double lambda_width_in_A = lambda_width * lambda0 / FO_SPEED_OF_LIGHT; /* :116 */
  /* maxdistance, final assignment (:138) */
  const double maxdistance = std_max((maxx - minx) / (nx - 1), (maxy - miny) / (ny - 1)) / .3;
  double deltaz = (maxz - minz); /* :142-143 */
  if (nz != 1) deltaz /= (nz - 1);
  const double c = FO_SPEED_OF_LIGHT;
  const long nray = (long)(row1 - row0) * nx;

#pragma omp parallel for schedule(dynamic, 16)
  for (long r = 0; r < nray; ++r) {
    int i = row0 + (int)(r / nx);
    int j = (int)(r % nx);
    double xr = (double)j / (nx - 1) * (maxx - minx) + minx; /* :152 */
    double yr = (double)i / (ny - 1) * (maxy - miny) + miny; /* :153 */
    double* acc = cube + r * L;
    float* accf = (float*)malloc(sizeof(float) * (size_t)L);
    for (int il = 0; il < L; ++il) {
      acc[il] = 0.0;
      accf[il] = 0.0f;
    }
    for (int k = 0; k < nz; ++k) {
      double zr = (double)k * deltaz + minz; /* :162 */
      /* derotation (:165) */
      double p0 = xr * cb * cl + yr * sl + zr * sb * cl;
      double p1 = -xr * cb * sl + yr * cl - zr * sb * sl;
      double p2 = -xr * sb + zr * cb;
      float t[3] = {(float)p0, (float)p1, (float)p2};                                   /* :171 */
      float lo[3] = {(float)(p0 - maxdistance), (float)(p1 - maxdistance), (float)(p2 - maxdistance)}; /* :179 */
      float hi[3] = {(float)(p0 + maxdistance), (float)(p1 + maxdistance), (float)(p2 + maxdistance)};
      int32_t idx = (mode & 2) ? fo_bruteforce_query(n, x, y, z, t, lo, hi) : grid_query(&g, t, lo, hi);
      if (nnidx) nnidx[r * nz + k] = idx;
      double intpolpeak = 0, intpolfwhm = 0, intpollosvel = 0;
      if (idx >= 0) {
        intpolpeak = peak[idx];
        intpolfwhm = fwhm[idx];
        intpollosvel = losvel[idx];
      }
      if (L > 1) {
        for (int il = 0; il < L; ++il) {
          double lambdaval = (double)il / (L - 1) * lambda_width_in_A - lambda_width_in_A / 2.; /* :200 */
          double tempintens = 0;
          if (intpolpeak != 0) {
            /* :204; GCC expands pow(x, 2) to x*x */
            double dl = lambdaval - intpollosvel / c * lambda0;
            tempintens = intpolpeak * exp(-(dl * dl) / (intpolfwhm * intpolfwhm) * 4. * log(2.));
          }
          if ((mode & 1))
            accf[il] = (float)((double)accf[il] + tempintens);
          else
            acc[il] += tempintens;
        }
      } else {
        if ((mode & 1))
          accf[0] = (float)((double)accf[0] + intpolpeak);
        else
          acc[0] += intpolpeak;
      }
    }
    if ((mode & 1))
      for (int il = 0; il < L; ++il) acc[il] = accf[il];
    free(accf);
  }

  /* Stage E scaling (:235-267) */
  double pathlength = (maxz - minz) / (nz - 1);
  if ((maxz == minz) || (nz == 1)) pathlength = 1.;
  double apix = 1.;
  if (is_dn) {
    float dx = (float)((maxx - minx) / (nx - 1)), dy = (float)((maxy - miny) / (ny - 1));
    const double as = M_PI / 180. / 3600.;
    apix = ((double)dx / FO_MM_PER_ARCSEC) * ((double)dy / FO_MM_PER_ARCSEC) * (as * as);
  }
  const double scale = pathlength * 1e8 * apix;
  const long total = nray * L;
  for (long e = 0; e < total; ++e) {
    if ((mode & 1))
      cube[e] = (double)(float)(scale * (double)(float)cube[e]);
    else
      cube[e] = scale * cube[e];
  }
  if (view) {
    for (int d = 0; d < 6; ++d) view[d] = ext[d];
    view[FO_V_MAXDIST] = maxdistance;
    view[FO_V_DELTAZ] = deltaz;
    view[FO_V_PATHLENGTH] = pathlength;
    view[FO_V_APIX] = apix;
    view[FO_V_SCALE] = scale;
    view[FO_V_LAMBDA_WIDTH_A] = lambda_width_in_A;
  }
  grid_free(&g);
  free(losvel);
  return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* a19: Thomson (pB) render (fomo-thomson.cpp:94-367)                       */
/* ------------------------------------------------------------------------ */

int fo_thomson_render(long n, const float* x, const float* y, const float* z, const float* tot, const float* pol,
                      double l, double b, int nx, int ny, int nz, int mode, int nthreads, int row0, int row1,
                      double* cube, int32_t* nnidx, double* view) {
  (void)tot; /* total brightness is computed but not accumulated by the reference (:325-338) */
  if (n <= 0 || nx < 2 || ny < 2 || nz < 1 || row0 < 0 || row1 > ny || row0 > row1) return FO_EARG;
  set_threads(nthreads);
  const double epsilon = 1e-6;
  double cos_b = cos(b), sin_b = sin(b);
  const double cos_l = cos(l), sin_l = sin(l);
  if (fabs(cos_b) < epsilon) cos_b = epsilon; /* :146-152 */
  if (fabs(sin_b) < epsilon) sin_b = epsilon;
  const double threshold = 1.309, steepness = 20.0;
  const double blend = 1.0 / (1.0 + exp(-steepness * (fabs(b) - threshold))); /* :176 */
  double* losvel = (double*)malloc(sizeof(double) * (size_t)n);
  if (!losvel) return FO_EARG;
  double mnx = DBL_MAX, mxx = -DBL_MAX, mny = DBL_MAX, mxy = -DBL_MAX, mnz = DBL_MAX, mxz = -DBL_MAX;
#pragma omp parallel for schedule(static) reduction(min : mnx, mny, mnz) reduction(max : mxx, mxy, mxz)
  for (long i = 0; i < n; ++i) {
    double gx = x[i], gy = y[i], gz = z[i];
    double full_x = gx * cos_b * cos_l - gy * cos_b * sin_l - gz * sin_b; /* :179-181 */
    double full_y = gx * sin_l + gy * cos_l;
    double full_z = gx * sin_b * cos_l - gy * sin_b * sin_l + gz * cos_b;
    double pole_x = gx * cos_l - gy * sin_l; /* :184-186 */
    double pole_y = gx * sin_l + gy * cos_l;
    double pole_z = gz;
    double xa = full_x * (1.0 - blend) + pole_x * blend; /* :189-191 */
    double ya = full_y * (1.0 - blend) + pole_y * blend;
    double za = full_z * (1.0 - blend) + pole_z * blend;
    /* sin^2 chi (:194-199); unit uses the clamped sin_b/cos_b and cos(l), sin(l) */
    double u0 = sin_b * cos(l), u1 = -sin_b * sin(l), u2 = cos_b;
    double ip = 0.0;
    ip = ip + u0 * xa;
    ip = ip + u1 * ya;
    ip = ip + u2 * za;
    double pp = 0.0;
    pp = pp + xa * xa;
    pp = pp + ya * ya;
    pp = pp + za * za;
    losvel[i] = 1. - (ip * ip) / pp; /* GCC expands pow(x, 2) to x*x */
    if (xa < mnx) mnx = xa;
    if (xa > mxx) mxx = xa;
    if (ya < mny) mny = ya;
    if (ya > mxy) mxy = ya;
    if (za < mnz) mnz = za;
    if (za > mxz) mxz = za;
  }
  const double minx = mnx, maxx = mxx, miny = mny, maxy = mxy, minz = mnz, maxz = mxz;
  fo_grid g;
  if (grid_build(&g, n, x, y, z) != FO_OK) {
    free(losvel);
    return FO_EARG;
  }
  /* maxdistance blend (:249-260) */
  const double blending_factor = 1.0 / (1.0 + exp(-10 * (fabs(b) - 0.1745)));
  const double ddx = (maxx - minx) / (nx - 1), ddy = (maxy - miny) / (ny - 1);
  const double equator_formula = std_max(0.5 * sqrt(ddx * ddx + ddy * ddy), 0.1 * (maxx - minx) / (nx - 1));
  const double away_from_equator_formula = std_max((maxx - minx) / (nx - 1), (maxy - miny) / (ny - 1)) / 0.005;
  const double maxdistance = equator_formula * (1.0 - blending_factor) + away_from_equator_formula * blending_factor;
  double deltaz = (maxz - minz);
  if (nz != 1) deltaz /= (nz - 1);
  const double cb = cos(b), sb = sin(b); /* unclamped in the march (:275-276) */
  const long nray = (long)(row1 - row0) * nx;

#pragma omp parallel for schedule(dynamic, 16)
  for (long r = 0; r < nray; ++r) {
    int i = row0 + (int)(r / nx);
    int j = (int)(r % nx);
    double xr = (double)j / (nx - 1) * (maxx - minx) + minx;
    double yr = (double)i / (ny - 1) * (maxy - miny) + miny;
    double acc = 0.0;
    float accf = 0.0f;
    for (int k = 0; k < nz; ++k) {
      double zr = (double)k * deltaz + minz;
      double p0 = xr * cb * cos_l + yr * sin_l + zr * sb * cos_l; /* :295 */
      double p1 = -xr * cb * sin_l + yr * cos_l - zr * sb * sin_l;
      double p2 = -xr * sb + zr * cb;
      float t[3] = {(float)p0, (float)p1, (float)p2};
      float lo[3] = {(float)(p0 - maxdistance), (float)(p1 - maxdistance), (float)(p2 - maxdistance)};
      float hi[3] = {(float)(p0 + maxdistance), (float)(p1 + maxdistance), (float)(p2 + maxdistance)};
      int32_t idx = (mode & 2) ? fo_bruteforce_query(n, x, y, z, t, lo, hi) : grid_query(&g, t, lo, hi);
      if (nnidx) nnidx[r * nz + k] = idx;
      double intpolpol = 0, intpollos = 0;
      if (idx >= 0) {
        intpolpol = pol[idx];
        intpollos = losvel[idx];
      }
      double tempintens2 = intpolpol * intpollos; /* :326 */
      if (tempintens2 < 0.) tempintens2 = 0;
      if ((mode & 1))
        accf = (float)((double)accf + tempintens2);
      else
        acc += tempintens2;
    }
    cube[r] = ((mode & 1)) ? (double)accf : acc;
  }
  double pathlength = (maxz - minz) / (nz - 1);
  if ((maxz == minz) || (nz == 1)) pathlength = 1.;
  const double scale = pathlength * 1e8;
  for (long e = 0; e < nray; ++e) {
    if ((mode & 1))
      cube[e] = (double)(float)(scale * (double)(float)cube[e]);
    else
      cube[e] = scale * cube[e];
  }
  if (view) {
    view[FO_V_MINX] = minx;
    view[FO_V_MAXX] = maxx;
    view[FO_V_MINY] = miny;
    view[FO_V_MAXY] = maxy;
    view[FO_V_MINZ] = minz;
    view[FO_V_MAXZ] = maxz;
    view[FO_V_MAXDIST] = maxdistance;
    view[FO_V_DELTAZ] = deltaz;
    view[FO_V_PATHLENGTH] = pathlength;
    view[FO_V_APIX] = 1.0;
    view[FO_V_SCALE] = scale;
    view[FO_V_LAMBDA_WIDTH_A] = 0.0;
  }
  grid_free(&g);
  free(losvel);
  return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* Render-cube grids (fomo-nearestneighbour.cpp:152-153,209-211,254-260)    */
/* ------------------------------------------------------------------------ */

void fo_render_grid(int nx, int ny, int L, const double* view, double lambda0, int is_dn, float* gx, float* gy,
                    float* glambda) {
  const double minx = view[FO_V_MINX], maxx = view[FO_V_MAXX], miny = view[FO_V_MINY], maxy = view[FO_V_MAXY];
  const double lwa = view[FO_V_LAMBDA_WIDTH_A];
  for (int i = 0; i < ny; ++i) {
    double yr = (double)i / (ny - 1) * (maxy - miny) + miny;
    for (int j = 0; j < nx; ++j) {
      double xr = (double)j / (nx - 1) * (maxx - minx) + minx;
      float xf = (float)xr, yf = (float)yr;
      if (is_dn) {
        xf = (float)(1. / FO_MM_PER_ARCSEC * (double)xf);
        yf = (float)(1. / FO_MM_PER_ARCSEC * (double)yf);
      }
      for (int il = 0; il < L; ++il) {
        long ind = ((long)i * nx + j) * L + il;
        gx[ind] = xf;
        gy[ind] = yf;
        if (L > 1 && glambda) {
          double lambdaval = (double)il / (L - 1) * lwa - lwa / 2.;
          glambda[ind] = (float)(lambdaval + lambda0);
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* f2: projection render (fomo-projection.cpp:17-193)                       */
/* ------------------------------------------------------------------------ */

int fo_projection_render(long n, const float* x, const float* y, const float* z, const float* peak,
                         const float* fwhm, const float* vx, const float* vy, const float* vz, double lambda0,
                         double l, double b, int nx, int ny, int nz, int L, double lambda_width, int is_dn, int mode,
                         double* cube, int32_t* pix, double* view) {
  if (n <= 0 || nx < 2 || ny < 2 || nz < 1 || L < 1) return FO_EARG;
  const double cb = cos(b), sb = sin(b), cl = cos(l), sl = sin(l);
  double* losvel = (double*)malloc(sizeof(double) * (size_t)n);
  float* accf = (float*)calloc((size_t)nx * ny * L, sizeof(float));
  if (!losvel || !accf) {
    free(losvel);
    free(accf);
    return FO_EARG;
  }
  double ext[6];
  nn_extents(n, x, y, z, vx, vy, vz, cb, sb, cl, sl, ext, losvel); /* :37-61 */
  const double minx = ext[0], maxx = ext[1], miny = ext[2], maxy = ext[3], minz = ext[4], maxz = ext[5];
  const double lambda_width_in_A = lambda_width * lambda0 / FO_SPEED_OF_LIGHT; /* :65 */
  const double c = FO_SPEED_OF_LIGHT;
  const long total = (long)nx * ny * L;
  for (long e = 0; e < total; ++e) cube[e] = 0.0;
  /* the points in order, as the reference's loop runs on one thread (:121-159) */
  for (long k = 0; k < n; ++k) {
    const double gx = x[k], gy = y[k], gz = z[k];
    const double xa = gx * cb * cl - gy * cb * sl - gz * sb; /* :47 */
    const double ya = gx * sl + gy * cl;                     /* :48 */
    const int j = (int)round((xa - minx) * (nx - 1) / (maxx - minx)); /* :124 */
    const int i = (int)round((ya - miny) * (ny - 1) / (maxy - miny)); /* :126 */
    if (pix) pix[k] = i * nx + j;
    if (L > 1) {
      for (int il = 0; il < L; ++il) {
        const double lambdaval = (double)il / (L - 1) * lambda_width_in_A - lambda_width_in_A / 2.; /* :133 */
        /* :134; GCC expands pow(x, 2) to x*x */
        const double dl = lambdaval - losvel[k] / c * lambda0;
        const double w = fwhm[k];
        const double tempintens = (double)peak[k] * exp(-(dl * dl) / (w * w) * 4. * log(2.));
        const long ind = ((long)i * nx + j) * L + il;
        if (mode & 1)
          accf[ind] = (float)((double)accf[ind] + tempintens);
        else
          cube[ind] += tempintens;
      }
    } else {
      const long ind = (long)i * nx + j;
      if (mode & 1)
        accf[ind] = accf[ind] + peak[k]; /* float += float (:152) */
      else
        cube[ind] += peak[k];
    }
  }
  /* scaling as the NN render (:161-191) */
  double pathlength = (maxz - minz) / (nz - 1);
  if ((maxz == minz) || (nz == 1)) pathlength = 1.;
  double apix = 1.;
  if (is_dn) {
    float dx = (float)((maxx - minx) / (nx - 1)), dy = (float)((maxy - miny) / (ny - 1));
    const double as = M_PI / 180. / 3600.;
    apix = ((double)dx / FO_MM_PER_ARCSEC) * ((double)dy / FO_MM_PER_ARCSEC) * (as * as);
  }
  const double scale = pathlength * 1e8 * apix;
  for (long e = 0; e < total; ++e)
    cube[e] = (mode & 1) ? (double)(float)(scale * (double)accf[e]) : scale * cube[e];
  if (view) {
    for (int d = 0; d < 6; ++d) view[d] = ext[d];
    view[FO_V_MAXDIST] = 0.0;
    view[FO_V_DELTAZ] = 0.0;
    view[FO_V_PATHLENGTH] = pathlength;
    view[FO_V_APIX] = apix;
    view[FO_V_SCALE] = scale;
    view[FO_V_LAMBDA_WIDTH_A] = lambda_width_in_A;
  }
  free(accf);
  free(losvel);
  return FO_OK;
}

/* ------------------------------------------------------------------------- */
/* AMRVAC snapshot reader (fomo-c/example/example_mpi_amrvac/                */
/* read_amrvac_files.cpp), restated: the data file's header, tree ("forest") */
/* and leaf blocks, the leaves' order, and each cell's position and          */
/* primitive variables, with the reference's FP64 expressions and their      */
/* rounding to FP32 when pushed into the DataCube.                           */
/* ------------------------------------------------------------------------- */

typedef struct {
  int level, idx[3];
} fo_leaf;

/* mortonEncode_for (FoMo-amrvac.h:13-19): bit i of x, y, z to bits 3i, 3i+1, 3i+2. */
static uint64_t fo_morton3(unsigned x, unsigned y, unsigned z) {
  uint64_t r = 0;
  for (int i = 0; i < 21; ++i)
    r |= ((uint64_t)((x >> i) & 1u) << (3 * i)) | ((uint64_t)((y >> i) & 1u) << (3 * i + 1)) |
         ((uint64_t)((z >> i) & 1u) << (3 * i + 2));
  return r;
}

/* loopthroughleafs (read_amrvac_files.cpp:20-44): depth first through the
 * tree; a leaf is recorded with its level and 1-based index at that level. */
static int fo_leaves(const int* forest, long nforest, long* pos, int level, int ndim, const int idx[3],
                     fo_leaf* out, long* nout, long cap) {
  ++*pos;
  if (*pos >= nforest) return FO_ETABLE;
  if (forest[*pos]) {
    if (*nout >= cap) return FO_ECAP;
    out[*nout].level = level;
    out[*nout].idx[0] = idx[0];
    out[*nout].idx[1] = idx[1];
    out[*nout].idx[2] = idx[2];
    ++*nout;
    return FO_OK;
  }
  for (int i = 0; i < (1 << ndim); ++i) {
    int ni[3];
    ni[0] = 2 * (idx[0] - 1) + 1 + i % 2;
    if (ndim == 2) {
      ni[1] = 2 * (idx[1] - 1) + 1 + i / 2;
      ni[2] = 1;
    } else {
      ni[1] = 2 * (idx[1] - 1) + 1 + (i / 2) % 2;
      ni[2] = 2 * (idx[2] - 1) + 1 + i / 4;
    }
    const int rc = fo_leaves(forest, nforest, pos, level + 1, ndim, ni, out, nout, cap);
    if (rc) return rc;
  }
  return FO_OK;
}

typedef struct {
  uint64_t code;
  int i, j, k;
} fo_mblock;

static int fo_mblock_cmp(const void* a, const void* b) {
  const uint64_t x = ((const fo_mblock*)a)->code, y = ((const fo_mblock*)b)->code;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* read_amrvac_par_file (read_amrvac_files.cpp:50-112): the first occurrence of
 * "nxlone<d>", "xprobmin<d>", "xprobmax<d>"; the value starts after the next
 * tab, newline, '=' or blank. */
static int fo_par_value(const char* text, const char* key, double* v) {
  const char* p = strstr(text, key);
  if (!p) return FO_ETABLE;
  p = strpbrk(p + 1, "\t\n= ");
  if (!p) return FO_ETABLE;
  *v = strtod(p + 1, NULL);
  return FO_OK;
}

static int fo_read_file(const char* path, unsigned char** buf, long* size) {
  FILE* f = fopen(path, "rb");
  if (!f) return FO_ENOFILE;
  fseek(f, 0, SEEK_END);
  *size = ftell(f);
  fseek(f, 0, SEEK_SET);
  *buf = (unsigned char*)malloc(*size > 0 ? (size_t)*size : 1);
  const size_t got = fread(*buf, 1, (size_t)*size, f);
  fclose(f);
  if ((long)got != *size) {
    free(*buf);
    return FO_ENOFILE;
  }
  return FO_OK;
}



int fo_amrvac_read(const char* datfile, const char* parfile, int gitlab_order, int gamma_eqparposition,
                   double n_unit, double Teunit, double L_unit, long cap, int* ndim_out, long* npts_out, float* x,
                   float* y, float* z, float* n, float* T, float* vx, float* vy, float* vz) {
  unsigned char* buf = NULL;
  long size = 0;
  int rc = fo_read_file(datfile, &buf, &size);
  if (rc) return rc;
  int version, nw, ndim, nleafs, nparents = 0, neqpar;
  int nx[3] = {1, 1, 1}, nxlone[3] = {1, 1, 1};
  double xprobmin[3] = {0, 0, 0}, xprobmax[3] = {0, 0, 0}, gamma = 0.0;
  long treeoff = 0, blockoff = 0, nforest = 0;
  int ghosts = 0;
  memcpy(&version, buf, 4);
  if (version == 3 || version == 4) {
    /* read_amrvac_new_dat_file (:430-528) / read_amrvac_dat_file_v4 (:535-683) */
    int hdr[11];
    memcpy(hdr, buf, sizeof(hdr));
    treeoff = hdr[1];
    blockoff = hdr[2];
    nw = hdr[3];
    ndim = hdr[5];
    nleafs = hdr[7];
    nparents = hdr[8];
    long off = 10 * 4 + 8; /* version .. it, then t */
    if (ndim < 2 || ndim > 3) {
      free(buf);
      return FO_EARG;
    }
    memcpy(xprobmin, buf + off, 8 * ndim);
    off += 8 * ndim;
    memcpy(xprobmax, buf + off, 8 * ndim);
    off += 8 * ndim;
    memcpy(nxlone, buf + off, 4 * ndim);
    off += 4 * ndim;
    memcpy(nx, buf + off, 4 * ndim);
    off += 4 * ndim;
    off += 16 * nw + 16; /* variable names, physics module */
    memcpy(&neqpar, buf + off, 4);
    off += 4;
    const double* eq = (const double*)(buf + off);
    double eqv;
    for (int i = 0; i < neqpar; ++i) {
      memcpy(&eqv, buf + off + 8 * i, 8);
      const char* name = (const char*)(buf + off + 8 * neqpar + 16 * i);
      /* version 3: the whole 16-byte name is "gamma" (blank or NUL padded);
       * version 4: its first 5 characters (:503-511, :637-646) */
      int len = 16;
      while (len > 0 && (name[len - 1] == ' ' || name[len - 1] == '\0')) --len;
      if ((version == 3 && len == 5 && memcmp(name, "gamma", 5) == 0) ||
          (version == 4 && memcmp(name, "gamma", 5) == 0))
        gamma = eqv;
    }
    (void)eq;
    if (gamma == 0.0) {
      free(buf);
      return FO_ETABLE; /* "No value for gamma found" */
    }
    nforest = nparents + nleafs;
    ghosts = 1; /* two ghost-cell counts per dimension before each block (:159-177) */
  } else {
    /* read_amrvac_old_dat_file (:301-418): the header at the end of the file */
    int tail[7];
    memcpy(tail, buf + size - 8 - 7 * 4, sizeof(tail));
    nleafs = tail[0];
    ndim = tail[2];
    nw = tail[4];
    neqpar = tail[5];
    if (ndim < 2 || ndim > 3) {
      free(buf);
      return FO_EARG;
    }
    const long eqoff = size - 8 - 7 * 4 - 8L * neqpar;
    const long nxoff = eqoff - 4L * ndim;
    memcpy(nx, buf + nxoff, 4 * ndim);
    double eqv;
    memcpy(&eqv, buf + eqoff + 8L * gamma_eqparposition, 8);
    gamma = eqv;
    long nglev = (long)nx[0] * nx[1] * (ndim == 3 ? nx[2] : 1);
    blockoff = 0;
    treeoff = (long)nleafs * nw * nglev * 8;
    nforest = (nxoff - treeoff) / 4;
    /* nxlone, xprobmin, xprobmax from the amrvac.par file */
    unsigned char* par = NULL;
    long psize = 0;
    rc = fo_read_file(parfile, &par, &psize);
    if (rc) {
      free(buf);
      return rc;
    }
    char* text = (char*)malloc((size_t)psize + 1);
    memcpy(text, par, (size_t)psize);
    text[psize] = 0;
    free(par);
    const char* keys[3] = {"nxlone", "xprobmin", "xprobmax"};
    for (int j = 0; j < 3 && !rc; ++j)
      for (int i = 0; i < ndim && !rc; ++i) {
        char key[32];
        snprintf(key, sizeof(key), "%s%d", keys[j], i + 1);
        double v = 0;
        rc = fo_par_value(text, key, &v);
        if (j == 0) nxlone[i] = (int)v;
        if (j == 1) xprobmin[i] = v;
        if (j == 2) xprobmax[i] = v;
      }
    free(text);
    if (rc) {
      free(buf);
      return rc;
    }
  }
  const long nglev1 = (long)nx[0] * nx[1] * (ndim == 3 ? nx[2] : 1);
  /* blocksandsize (:114-129) */
  int nblocks[3] = {1, 1, 1};
  double cellsize[3] = {0, 0, 0};
  for (int i = 0; i < ndim; ++i) {
    if (nxlone[i] % nx[i] != 0) {
      free(buf);
      return FO_ETABLE; /* "Non-integer number of blocks" */
    }
    nblocks[i] = nxlone[i] / nx[i];
    cellsize[i] = (xprobmax[i] - xprobmin[i]) / nxlone[i];
  }
  int* forest = (int*)malloc(sizeof(int) * (size_t)(nforest > 0 ? nforest : 1));
  memcpy(forest, buf + treeoff, 4 * (size_t)nforest);
  fo_leaf* leaves = (fo_leaf*)malloc(sizeof(fo_leaf) * (size_t)(nleafs > 0 ? nleafs : 1));
  long nl = 0, pos = -1;
  if (version != 3 && version != 4 && !gitlab_order) {
    /* the pre-2017 order: level-1 blocks with x fastest (:380-390) */
    for (int k = 0; k < nblocks[2] && !rc; ++k)
      for (int j = 0; j < nblocks[1] && !rc; ++j)
        for (int i = 0; i < nblocks[0] && !rc; ++i) {
          const int idx[3] = {i + 1, j + 1, k + 1};
          rc = fo_leaves(forest, nforest, &pos, 1, ndim, idx, leaves, &nl, nleafs);
        }
  } else {
    /* build_block_info_morton (:183-226): the level-1 blocks in Morton order */
    const long nb = (long)nblocks[0] * nblocks[1] * nblocks[2];
    fo_mblock* mb = (fo_mblock*)malloc(sizeof(fo_mblock) * (size_t)nb);
    long c = 0;
    for (int k = 0; k < nblocks[2]; ++k)
      for (int j = 0; j < nblocks[1]; ++j)
        for (int i = 0; i < nblocks[0]; ++i) {
          mb[c].code = fo_morton3((unsigned)i, (unsigned)j, (unsigned)k);
          mb[c].i = i;
          mb[c].j = j;
          mb[c].k = k;
          ++c;
        }
    qsort(mb, (size_t)nb, sizeof(fo_mblock), fo_mblock_cmp);
    for (long b = 0; b < nb && !rc; ++b) {
      const int idx[3] = {mb[b].i + 1, mb[b].j + 1, mb[b].k + 1};
      rc = fo_leaves(forest, nforest, &pos, 1, ndim, idx, leaves, &nl, nleafs);
    }
    free(mb);
  }
  free(forest);
  if (!rc && nl != nleafs) rc = FO_ETABLE; /* "block_info.size() ... does not match nleafs" */
  const long npts = (long)nleafs * nglev1;
  *ndim_out = ndim;
  *npts_out = npts;
  if (!rc && npts > cap) rc = FO_ECAP;
  if (rc) {
    free(leaves);
    free(buf);
    return rc;
  }
  /* fomo_from_amrvac (:228-299) */
  const double R_spec = FO_BOLTZMANN / (0.5e0 * FO_MASS_PROTON);
  const double V_unit = sqrt(R_spec * Teunit);
  long boff = blockoff, p = 0;
  for (long b = 0; b < nleafs; ++b) {
    if (ghosts) boff += 8L * ndim;
    const double* blk = (const double*)(buf + boff); /* nw variables, each nglev1 cells */
    const int lev = leaves[b].level;
    double bottomleft[3], lcs[3];
    for (int j = 0; j < ndim; ++j) {
      const double p2 = pow(2, lev - 1);
      bottomleft[j] = xprobmin[j] + (leaves[b].idx[j] - 1) * cellsize[j] * nx[j] / p2;
      lcs[j] = cellsize[j] / p2;
    }
    for (long k = 0; k < nglev1; ++k, ++p) {
      const long lc[3] = {1 + k % nx[0], 1 + k / nx[0] % nx[0], 1 + k / nx[0] / nx[1]};
      double cc[3] = {0, 0, 0};
      for (int j = 0; j < ndim; ++j) {
        cc[j] = bottomleft[j] + (lc[j] - .5) * lcs[j];
        cc[j] *= L_unit;
      }
      double v[8];
      for (int w = 0; w < 8 && w < nw; ++w) memcpy(&v[w], (const char*)blk + 8 * ((long)w * nglev1 + k), 8);
      const double rho = v[0];
      /* the kinetic and magnetic terms sum the first two components only (std::inner_product over [1, 3) and [5, 7)) */
      const double kin = ((0. + v[1] * v[1]) + v[2] * v[2]) / rho / 2.;
      const double mag = ((0. + v[5] * v[5]) + v[6] * v[6]) / 2.;
      const double pr = (gamma - 1) * (v[4] - kin - mag);
      x[p] = (float)cc[0];
      y[p] = (float)cc[1];
      z[p] = (float)cc[2];
      n[p] = (float)(rho * n_unit);
      T[p] = (float)(pr / rho * Teunit);
      vx[p] = (float)(v[1] / rho * V_unit);
      vy[p] = (float)(v[2] / rho * V_unit);
      vz[p] = (float)(v[3] / rho * V_unit);
    }
    boff += 8L * nw * nglev1;
  }
  free(leaves);
  free(buf);
  return FO_OK;
}
