// seeding.cu -- the initial sites of the reference's centroidalVoronoi
// (gcvt.h:56-139), host code: fixed sites from the mask (putConstrains,
// gcvt.h:106-122), then `num` distinct pixels drawn by rejection against the
// density (randomPoints, gcvt.h:76-104) from the reference's generator
// (gcvt.h:57-73), so a caller gets the reference's initial sites exactly.
//
// The generator is the reference's combination of a multiply-with-carry, a
// congruential and a shift-register stream over 64-bit words (`unsigned long`
// on LP64 systems).  The reference never seeds it (no call of randinit), so
// its state starts at zero and carries over from call to call; the library
// keeps one such global state, and callers may pass their own instead.
#include "../../include/gcvt_gb300.h"

#include <cmath>
#include <mutex>

namespace {

struct Rng {
  uint64_t z, w, jsr, jcong;
};

uint64_t rng_int(Rng &g) {
  g.z = 36969ull * (g.z & 0xffffull) + (g.z >> 16);
  g.w = 18000ull * (g.w & 0xffffull) + (g.w >> 16);
  const uint64_t mwc = (g.z << 16) + g.w;
  g.jcong = 69069ull * g.jcong + 1234567ull;
  g.jsr ^= g.jsr << 17;
  g.jsr ^= g.jsr >> 13;
  g.jsr ^= g.jsr << 5;
  return (mwc ^ g.jcong) + g.jsr;
}

// [0, 1): the word over 2^64 (double(ULONG_MAX) + 1 rounds to 2^64).
double rng_unit(Rng &g) { return (double)rng_int(g) / 18446744073709551616.0; }

Rng g_rng = {0, 0, 0, 0};
std::mutex g_rng_mutex;

int seed(int16_t *v, const float *density, const uint8_t *mask, int num, int size, Rng &g) {
  const size_t nn = (size_t)size * size;
  // putConstrains
  for (int i = 0; i < size; ++i)
    for (int j = 0; j < size; ++j) {
      const size_t p = (size_t)j * size + i;
      if (mask && mask[p]) {
        v[2 * p] = (int16_t)i;
        v[2 * p + 1] = (int16_t)j;
      } else {
        v[2 * p] = v[2 * p + 1] = GCVT_MARKER;
      }
    }
  // randomPoints
  double mx = 0, avg = 0, cnt = 0;
  size_t free_px = 0;
  for (size_t i = 0; i < nn; ++i) {
    if (density[i] > mx) mx = density[i];
    if (density[i] != 0) {
      cnt += 1;
      avg += density[i];
      if (density[i] > 0 && v[2 * i] == GCVT_MARKER) ++free_px;
    }
  }
  if (num == 0) return GCVT_OK;
  if ((size_t)num > free_px) return GCVT_ERR_ARGUMENT;  // the draw could never end
  mx = std::fmin(mx, avg / cnt * 100.);
  // the reference loops until it succeeds; a draw budget turns a density
  // too small for any acceptance into an error instead of a hang
  long long budget = 1000LL * (long long)nn + 1000000LL;
  for (int k = 0; k < num; ++k) {
    int x, y;
    double z;
    do {
      if (--budget < 0) return GCVT_ERR_INPUT;
      x = (int)(rng_unit(g) * size);
      y = (int)(rng_unit(g) * size);
      z = rng_unit(g) * mx;
    } while (v[2 * ((size_t)y * size + x)] != GCVT_MARKER || density[(size_t)y * size + x] <= z);
    v[2 * ((size_t)y * size + x)] = (int16_t)x;
    v[2 * ((size_t)y * size + x) + 1] = (int16_t)y;
  }
  return GCVT_OK;
}

}  // namespace

extern "C" int gcvt_seed_sites(int16_t *voronoi, const float *density, const uint8_t *mask,
                               int num, int size, uint64_t *state) {
  if (!voronoi || !density || size < 1 || size > 32767 || num < 0) return GCVT_ERR_ARGUMENT;
  if (state) {
    Rng g = {state[0], state[1], state[2], state[3]};
    const int rc = seed(voronoi, density, mask, num, size, g);
    state[0] = g.z;
    state[1] = g.w;
    state[2] = g.jsr;
    state[3] = g.jcong;
    return rc;
  }
  std::lock_guard<std::mutex> lock(g_rng_mutex);
  return seed(voronoi, density, mask, num, size, g_rng);
}

extern "C" int gcvt_centroidal_voronoi(int16_t *voronoi, float *density, const uint8_t *mask,
                                       int vertices, int size, int depth, int max_iter) {
  if (!voronoi || !density || !mask) return GCVT_ERR_ARGUMENT;
  int rc = gcvt_seed_sites(voronoi, density, mask, vertices, size, nullptr);
  if (rc) return rc;
  return gcvt_compute(voronoi, density, mask, size, depth, max_iter);
}
