/*
 * lockx_case.c -- TEST INFRASTRUCTURE ONLY.
 *
 * The case functions of the channel lock-exchange run used to generate the
 * solver fixtures of the 64 x 16 quad channel (tests/golden/make_lockexchange_golden.py):
 * the reference model is built with these in place of its main/initialization.c
 * and main/state.c, the way its example cases replace them
 * (examples/lockexchange/Makefile:40 copies a case's objects over main's).
 * The interfaces are the reference's main/initialization.h and main/state.h.
 *
 *   depth          flat 20 m
 *   vertical grid  Nkmax uniform levels (rstretch 1)
 *   density        rho' = beta*s (the example's linear equation of state,
 *                  examples/lockexchange/state.c:27) with s = -0.5e-3 for
 *                  x < 320 m and +0.5e-3 beyond: the lock at mid-channel
 *   velocity       face-normal u = N(0, 0.01 m/s) noise, a deterministic
 *                  function of the face centre and depth (a hash of the
 *                  coordinates' bits drawn through Box-Muller), so the
 *                  field does not depend on the order cells are visited
 *   free surface   0; temperature and sediment 0
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "suntans.h"
#include "initialization.h"
#include "state.h"

int GetDZ(REAL *dz, REAL depth, REAL localdepth, int Nkmax, int myproc) {
  int k;
  const REAL dz0 = depth / Nkmax;
  REAL z = 0;
  if (dz != NULL) {
    for (k = 0; k < Nkmax; k++) dz[k] = dz0;
    return Nkmax;
  }
  /* levels needed to reach localdepth */
  for (k = 0; k < Nkmax; k++) {
    z += dz0;
    if (z >= localdepth) return k + 1;
  }
  return Nkmax;
}

REAL ReturnDepth(REAL x, REAL y) { return 20.0; }

REAL ReturnFreeSurface(REAL x, REAL y, REAL d) { return 0.0; }

REAL ReturnSalinity(REAL x, REAL y, REAL z) { return x < 320.0 ? -0.5e-3 : 0.5e-3; }

REAL ReturnTemperature(REAL x, REAL y, REAL z, REAL depth) { return 0.0; }

/* splitmix64 finaliser: a well-mixed 64-bit hash */
static uint64_t mix64(uint64_t v) {
  v += 0x9E3779B97F4A7C15ull;
  v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ull;
  v = (v ^ (v >> 27)) * 0x94D049BB133111EBull;
  return v ^ (v >> 31);
}

static uint64_t bits_of(REAL x) {
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
}

REAL ReturnHorizontalVelocity(REAL x, REAL y, REAL n1, REAL n2, REAL z) {
  const uint64_t h = mix64(bits_of(x) ^ mix64(bits_of(y) ^ mix64(bits_of(z) ^ 0x5EEDull)));
  const uint64_t h2 = mix64(h);
  /* two uniforms in (0, 1], Box-Muller */
  const double u1 = ((double)(h >> 11) + 1.0) / 9007199254740992.0;
  const double u2 = ((double)(h2 >> 11) + 1.0) / 9007199254740992.0;
  return 0.01 * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

REAL ReturnSediment(REAL x, REAL y, REAL z, int sizeno) { return 0.0; }

REAL ReturnBedSedimentRatio(REAL x, REAL y, int layer, int sizeno, int nsize) { return 0.0; }

REAL StateEquation(const propT *prop, const REAL s, const REAL T, const REAL p) { return prop->beta * s; }
