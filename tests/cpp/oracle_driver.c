/*
 * Drives every entry point of the CPU oracle (oracle/fomo_oracle.c) on a small
 * seeded case, for the sanitizer build of tests/test_sanitizers.py: a jittered
 * 10x11x12 point cloud with a loop in density and temperature, a synthetic
 * G(T, n) table written to a file and read back, spectroscopic and imaging
 * emissivities, NN renders at b != 0 (grid search and brute force, whose
 * neighbour indices must agree), the Thomson terms and render of the cloud
 * moved past 1 solar radius, the projection render and the render grids.
 *
 *   oracle_driver TABLE_PATH      -> prints "ok" and exits 0
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fomo_oracle.h"

static unsigned long long rng_state = 88172645463325252ull;
static double urand(void) {
  rng_state ^= rng_state << 13;
  rng_state ^= rng_state >> 7;
  rng_state ^= rng_state << 17;
  return (double)(rng_state >> 11) * (1.0 / 9007199254740992.0);
}

static int write_table(const char* path) {
  FILE* f = fopen(path, "w");
  if (!f) return 1;
  const int nt = 41, nrho = 11;
  fprintf(f, "fe_12 193.509 55.845 1 2 extra\n");
  fprintf(f, "erg cm^3 s^-1 sr^-1\n");
  fprintf(f, "version 8\n");
  fprintf(f, "%d %d\n", nrho, nt);
  for (int t = 0; t < nt; ++t) fprintf(f, "%.6f ", 4.0 + 0.1 * t);
  fprintf(f, "\n");
  for (int r = 0; r < nrho; ++r) {
    fprintf(f, "%.6f", 8.0 + 0.4 * r);
    for (int t = 0; t < nt; ++t) {
      const double lt = 4.0 + 0.1 * t;
      fprintf(f, " %.6e", 1e-24 * exp(-(lt - 6.1) * (lt - 6.1) / (2 * 0.15 * 0.15)) * (1.0 + 0.05 * r));
    }
    fprintf(f, "\n");
  }
  fclose(f);
  return 0;
}

#define CHECK(c, msg)                                    \
  do {                                                   \
    if (!(c)) {                                          \
      fprintf(stderr, "check failed: %s\n", msg);        \
      return 1;                                          \
    }                                                    \
  } while (0)

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  CHECK(write_table(argv[1]) == 0, "table written");
  const int gx = 10, gy = 11, gz = 12;
  const long n = (long)gx * gy * gz;
  float *x = malloc(sizeof(float) * n), *y = malloc(sizeof(float) * n), *z = malloc(sizeof(float) * n);
  float *ne = malloc(sizeof(float) * n), *T = malloc(sizeof(float) * n);
  float *vx = malloc(sizeof(float) * n), *vy = malloc(sizeof(float) * n), *vz = malloc(sizeof(float) * n);
  long k = 0;
  for (int a = 0; a < gx; ++a)
    for (int b = 0; b < gy; ++b)
      for (int c = 0; c < gz; ++c, ++k) {
        x[k] = (float)(-5.0 + 10.0 * (a + 0.5 + 0.2 * (urand() - 0.5)) / gx);
        y[k] = (float)(-5.0 + 10.0 * (b + 0.5 + 0.2 * (urand() - 0.5)) / gy);
        z[k] = (float)(-5.0 + 10.0 * (c + 0.5 + 0.2 * (urand() - 0.5)) / gz);
        const double r = sqrt((double)x[k] * x[k] + (double)y[k] * y[k]);
        const double f = 0.5 * (1.0 - tanh((r - 1.0) / 0.2));
        ne[k] = (float)(1e8 + f * 9e8);
        T[k] = (float)(2e6 - f * 1e6);
        vx[k] = (float)(1e4 * sin(2 * 3.14159265358979323846 * z[k] / 10.0));
        vy[k] = 0.0f;
        vz[k] = (float)(3e3 * urand());
      }

  char ion[32], unit[64];
  double hdr[4];
  int nt = 0, nrho = 0;
  float logT[64], logn[64], G[64 * 64];
  CHECK(fo_table_read(argv[1], ion, sizeof(ion), unit, sizeof(unit), hdr, &nt, &nrho, logT, logn, G, 64 * 64) == FO_OK,
        "table read");
  CHECK(nt == 41 && nrho == 11, "table size");

  float *eps = malloc(sizeof(float) * n), *fwhm = malloc(sizeof(float) * n);
  CHECK(fo_emission(n, ne, T, nt, nrho, logT, logn, G, hdr[0], hdr[1], ion, 0, 1.0, eps, fwhm) == FO_OK, "emission");
  /* the imaging check rejects a line table (fomo-CHIANTI.cpp:278) */
  CHECK(fo_emission(n, ne, T, nt, nrho, logT, logn, G, hdr[0], hdr[1], ion, 1, 1.0, eps, fwhm) == FO_EIMAGING,
        "imaging check");
  CHECK(fo_emission(n, ne, T, nt, nrho, logT, logn, G, hdr[0], hdr[1], ion, 0, 1.0, eps, fwhm) == FO_OK, "emission");

  const int nx = 9, ny = 7, nz = 13, L = 8;
  const double width = 0.6 * FO_SPEED_OF_LIGHT / hdr[0];
  double *cube = malloc(sizeof(double) * nx * ny * L), *cube2 = malloc(sizeof(double) * nx * ny * L);
  int32_t *idx = malloc(sizeof(int32_t) * nx * ny * nz), *idx2 = malloc(sizeof(int32_t) * nx * ny * nz);
  double view[FO_V_COUNT], view2[FO_V_COUNT];
  const double angles[3][2] = {{0.0, 0.0}, {0.4, 0.3}, {1.1, -0.35}};
  for (int v = 0; v < 3; ++v) {
    CHECK(fo_nn_render(n, x, y, z, eps, fwhm, vx, vy, vz, hdr[0], angles[v][0], angles[v][1], nx, ny, nz, L, width, 0,
                       0, 2, 0, ny, cube, idx, view) == FO_OK,
          "nn render");
    CHECK(fo_nn_render(n, x, y, z, eps, fwhm, vx, vy, vz, hdr[0], angles[v][0], angles[v][1], nx, ny, nz, L, width, 0,
                       2, 1, 0, ny, cube2, idx2, view2) == FO_OK,
          "nn render (brute force)");
    CHECK(memcmp(idx, idx2, sizeof(int32_t) * nx * ny * nz) == 0, "grid search == brute force");
    long found = 0;
    for (long i = 0; i < (long)nx * ny * nz; ++i) found += idx[i] >= 0;
    CHECK(2 * found > (long)nx * ny * nz, "most samples have a neighbour");
    /* FP32 accumulation mode, one band of rows */
    CHECK(fo_nn_render(n, x, y, z, eps, fwhm, vx, vy, vz, hdr[0], angles[v][0], angles[v][1], nx, ny, nz, L, width, 0,
                       1, 1, 2, 5, cube2, NULL, view2) == FO_OK,
          "nn render (FP32, rows 2-4)");
  }
  float *gxv = malloc(sizeof(float) * nx * ny * L), *gyv = malloc(sizeof(float) * nx * ny * L),
        *glv = malloc(sizeof(float) * nx * ny * L);
  fo_render_grid(nx, ny, L, view, hdr[0], 0, gxv, gyv, glv);

  /* Thomson: the cloud at 1.5 solar radii */
  for (long i = 0; i < n; ++i) x[i] += 1043.55f;
  float *tot = malloc(sizeof(float) * n), *pol = malloc(sizeof(float) * n);
  fo_thomson_emission(n, x, y, z, ne, tot, pol);
  double* tcube = malloc(sizeof(double) * nx * ny);
  CHECK(fo_thomson_render(n, x, y, z, tot, pol, 0.2, 0.3, nx, ny, nz, 0, 2, 0, ny, tcube, idx, view) == FO_OK,
        "thomson render");
  CHECK(fo_thomson_render(n, x, y, z, tot, pol, 0.2, 0.3, nx, ny, nz, 2, 1, 0, ny, tcube, idx2, view2) == FO_OK,
        "thomson render (brute force)");
  CHECK(memcmp(idx, idx2, sizeof(int32_t) * nx * ny * nz) == 0, "thomson grid search == brute force");
  for (long i = 0; i < n; ++i) x[i] -= 1043.55f;

  int32_t* pix = malloc(sizeof(int32_t) * n);
  CHECK(fo_projection_render(n, x, y, z, eps, fwhm, vx, vy, vz, hdr[0], 0.4, 0.3, nx, ny, nz, L, width, 0, 1, cube,
                             pix, view) == FO_OK,
        "projection render");

  /* one brute-force query straight */
  const float tq[3] = {0.1f, -0.2f, 0.3f}, lo[3] = {-0.5f, -0.8f, -0.3f}, hi[3] = {0.7f, 0.4f, 0.9f};
  const int32_t q = fo_bruteforce_query(n, x, y, z, tq, lo, hi);
  CHECK(q >= -1 && q < n, "query");

  free(x), free(y), free(z), free(ne), free(T), free(vx), free(vy), free(vz), free(eps), free(fwhm);
  free(cube), free(cube2), free(idx), free(idx2), free(gxv), free(gyv), free(glv), free(tot), free(pol), free(tcube);
  free(pix);
  printf("ok\n");
  return 0;
}
