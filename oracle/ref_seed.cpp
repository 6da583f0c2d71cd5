// ref_seed.cpp -- TEST INFRASTRUCTURE ONLY: the reference's own site seeding
// (source/gcvt.h:56-122: the random generator, randomPoints, putConstrains),
// compiled from the reference checkout by oracle/build_oracle.py into
// oracle/_ref/libseed_ref.so, to pin the oracle's and the library's restated
// seeding bit for bit.
//
// gcvt.h does not compile under glibc as it stands: it defines
// `double random()`, which clashes with stdlib's `long random(void)`
// (gcvt.h:73).  The standard headers are included first and `random` is then
// renamed for the reference header only.  gcvt.h also declares gCVT
// (gcvt.h:29), which centroidalVoronoi calls; a stand-in that does nothing is
// defined here so the library has no undefined symbol (it is never called).
#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#define random gcvt_ref_random
#include "gcvt.h"
#undef random

void gCVT(short *, float *, bool *, int, int, int) {}

extern "C" {

// Generator state (z, w, jsr, jcong): copied out to get[4] when get is not
// null, then replaced by set[4] when set is not null.
void refseed_state(unsigned long long *get, const unsigned long long *set) {
  if (get) {
    get[0] = z;
    get[1] = w;
    get[2] = jsr;
    get[3] = jcong;
  }
  if (set) {
    z = (unsigned long)set[0];
    w = (unsigned long)set[1];
    jsr = (unsigned long)set[2];
    jcong = (unsigned long)set[3];
  }
}

// putConstrains + randomPoints, the first half of centroidalVoronoi
// (gcvt.h:124-135): voronoi is 2 size^2 int16, mask size^2 bytes.
void refseed_sites(short *voronoi, float *density, const unsigned char *mask, int num,
                   int size) {
  std::vector<char> m((size_t)size * size);
  for (size_t i = 0; i < m.size(); ++i) m[i] = mask[i] != 0;
  putConstrains(voronoi, reinterpret_cast<bool *>(m.data()), size);
  randomPoints(voronoi, density, num, size);
}

}  // extern "C"
