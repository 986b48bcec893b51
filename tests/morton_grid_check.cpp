// Host check of morton_floor_fast (obvhs_gb300/csrc/morton_grid.h) against
// the double-precision coordinate it stands for, sat_u32(RN(RN(c * S) + O)),
// with S and O formed from f32 scene bounds as the Morton kernels form them
// (1 / (max - min) in f64 from the f32 extent, times 2^21; the offset
// -min * that).  Built with -ffp-contract=off so that every float and double
// operation is rounded on its own, as on the device.
//
// usage: morton_grid_check SEED SCENES PER_SCENE
// prints one JSON line; exit status 1 if any decided coordinate differs.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "morton_grid.h"

static uint64_t rng_state;
static uint64_t next_u64() {  // splitmix64
  uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double uniform() { return (double)(next_u64() >> 11) * 0x1p-53; }

static uint32_t sat_u32_ref(double px) {
  if (!(px >= 1.0)) return 0u;  // NaN, negative, below 1
  if (px >= 4294967296.0) return 0xffffffffu;
  return (uint32_t)px;
}

static long long cases, decided, mismatches;

static void check(float c, double S, double O, const MortonAxis* ax) {
  cases++;
  long long k;
  if (!morton_floor_fast(c, ax, &k)) return;
  decided++;
  const uint32_t got = k < 0 ? 0u : k > 0xffffffffll ? 0xffffffffu : (uint32_t)k;
  const double px = (double)c * S + O;
  const uint32_t want = sat_u32_ref(px);
  if (got != want) {
    if (mismatches < 10)
      fprintf(stderr, "mismatch: c=%a S=%a O=%a px=%a got=%u want=%u\n", (double)c, S, O, px, got, want);
    mismatches++;
  }
}

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  rng_state = strtoull(argv[1], 0, 10);
  const long scenes = strtol(argv[2], 0, 10), per = strtol(argv[3], 0, 10);
  const double grid = 2097152.0;
  long long in_range_cases = 0, in_range_decided = 0;
  for (long s = 0; s < scenes; s++) {
    // bounds: a scene around the origin, or offset by up to 10^5 of its size
    const double ext = pow(10.0, -4.0 + 9.0 * uniform());
    const int kind = (int)(next_u64() % 4);
    double lo = kind == 0 ? -ext * uniform() : kind == 1 ? ext * 100.0 * (uniform() - 0.5)
                : kind == 2 ? ext * pow(10.0, 5.0 * uniform()) * (uniform() < 0.5 ? -1.0 : 1.0) : 0.0;
    const float mn = (float)lo, mx = (float)(lo + ext);
    if (!(mx > mn)) continue;
    const double sx = 1.0 / (double)(mx - mn);
    const double S = sx * grid, O = (-(double)mn * sx) * grid;
    const MortonAxis ax = morton_axis(S, O);
    const long long before_cases = cases, before_decided = decided;
    for (long i = 0; i < per; i++) {
      const float c = (float)((double)mn + uniform() * ((double)mx - (double)mn));
      check(c, S, O, &ax);
    }
    if (kind <= 1) {
      in_range_cases += cases - before_cases;
      in_range_decided += decided - before_decided;
    }
    // the bounds, the middle, and centres a few ulps from each grid line K
    const float ends[3] = {mn, mx, mn + (mx - mn) * 0.5f};
    for (int e = 0; e < 3; e++) check(ends[e], S, O, &ax);
    for (int j = 0; j < 64; j++) {
      const double K = (double)(next_u64() % 2097153u);
      float c = (float)((K - O) / S);
      for (int u = 0; u < 4; u++) c = nextafterf(c, -INFINITY);
      for (int u = 0; u < 9; u++, c = nextafterf(c, INFINITY)) check(c, S, O, &ax);
    }
    // values the fast path must leave to double precision or get right
    const float special[8] = {0.0f, -0.0f, 0x1p-140f, -0x1p-130f, INFINITY, -INFINITY, NAN, 0x1p50f};
    for (int e = 0; e < 8; e++) check(special[e], S, O, &ax);
  }
  printf("{\"cases\": %lld, \"decided\": %lld, \"mismatches\": %lld, \"in_range_cases\": %lld, "
         "\"in_range_decided\": %lld}\n",
         cases, decided, mismatches, in_range_cases, in_range_decided);
  return mismatches ? 1 : 0;
}
