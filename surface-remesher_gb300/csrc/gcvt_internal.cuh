// gcvt_internal.cuh -- device-side data layout and kernel declarations of the
// GB300 CVT engine.  Everything here is private to libgcvt_gb300.so.
//
// Grid conventions follow the reference (gcvt.h:26-27): pixel (x, y) is index
// y*n + x; a label is the reference's short2 (x in the low 16 bits, y in the
// high 16 bits of a 32-bit word); MARKER = -32768 marks "no site".
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace cvtgb {

constexpr int kMarker = -32768;
constexpr uint32_t kMarkerWord = 0x80008000u;
constexpr int kNoneAbove = -32768;  // "no site above" in the column summaries
constexpr int kNoneBelow = 32767;   // "no site below"
constexpr int kBand = 64;           // PBA+ phase-1 band height: n / m1 == 64 for
                                    // every entry of gcvt.cu:842-847
constexpr int kRowsPerBlock = 4;    // rows (one warp each) per row-pass block
constexpr int kUpdateThreads = 256;
constexpr int kMinN = 256;   // n must be a multiple of 256 (S = n/32 >= 8)
constexpr int kMaxN = 8192;  // row-pass shared memory: 4 rows x 32 KB at 8192

__host__ __device__ inline uint32_t pack_xy(int x, int y) {
  return (uint32_t)(uint16_t)x | ((uint32_t)(uint16_t)y << 16);
}

// Slot of the site at (x, y): sites are numbered group by group (32 columns),
// inside a group band by band and column by column, inside a word by row.
__device__ __forceinline__ int site_slot(const uint64_t *bits, const int *word_rank,
                                         const int *group_offset, int n, int x, int y) {
  const size_t w = (size_t)(y >> 6) * n + x;
  const uint64_t below = bits[w] & ((1ull << (y & 63)) - 1ull);
  return group_offset[x >> 5] + word_rank[w] + __popcll(below);
}

// Per-context device state.  Kernels of one Lloyd iteration read it; the last
// block of the update kernel advances it, so a whole iteration runs without a
// host round trip and can be captured in a CUDA graph.
struct DevState {
  int parity;          // which site bitmap is current
  int iter;            // Lloyd iterations completed (gcvtIterations)
  int level_iters;     // iterations completed at the current level
  int stopped;         // set when the level's loop condition ends it
  int level;           // pyramid level (0 = finest)
  int max_iter;        // total iteration cap (maxIter)
  int use_stop_rule;   // 1: energy stop rule of gcvt.cu:1125-1140; 0: fixed count
  int fixed_iters;     // iterations per level when use_stop_rule == 0
  int error;           // input validation flags
  unsigned done_blocks;
  float omega;         // over-relaxation (pbaOmega)
  float pad0;
  double last_energy;  // lastEnergy
  double sampled;      // Energy, sampled when iter % 10 == 0
  double energy;       // energy of the most recent iteration
  double energy_scale; // 4^level / n^2
};

// Buffers of one resolution level, passed by value to every kernel.
struct LevelBufs {
  int n;
  uint64_t *bits[2];       // site bitmaps [band][column], bit i = row 64*band+i
  int16_t *prev;           // [band][column]: nearest site row above the band
  int16_t *next;           // [band][column]: nearest site row below the band
  const float *density;    // n*n
  const uint8_t *fixed;    // full-resolution mask, indexed with this level's n
                           // (only used to build fixed_bits)
  float4 *mhi, *mlo;       // per-site compensated moments (W, SX, SY, E), SX and
                           // SY relative to the site, indexed by the site's slot
  uint64_t *fixed_bits;    // fixed sites of this level, same layout as bits
  int *word_rank;          // [band][column]: sites in earlier words of the
                           // column's 32-column group (band-major order)
  int *group_count;        // per 32-column group: its number of sites
  int *group_offset;       // exclusive prefix of group_count
  uint32_t *labels;        // n*n label words (label passes only)
  const int2 *support;     // per row [first, last+1) of nonzero density
  DevState *st;
  float *blk_energy;       // one two-float partial per update block
};

// Kernels (launch helpers in labeller.cu / lloyd.cu).
cudaError_t launch_grid_to_bits(const uint32_t *grid, int n, uint64_t *bits, int *err,
                                cudaStream_t s);
cudaError_t launch_bits_to_grid(const uint64_t *bits, int n, uint32_t *grid, cudaStream_t s);
cudaError_t launch_summary(const LevelBufs &b, int respect_stop, cudaStream_t s);
cudaError_t launch_fixed_bits(const uint8_t *mask, int n, uint64_t *fixed_bits, cudaStream_t s);
cudaError_t launch_rows(const LevelBufs &b, int label_mode, int respect_stop, cudaStream_t s);
cudaError_t launch_update(const LevelBufs &b, cudaStream_t s);
cudaError_t launch_zoom(const uint64_t *src, int n, uint64_t *dst, cudaStream_t s);
cudaError_t launch_density_halve(const float *in, float *out, int n_out, cudaStream_t s);
cudaError_t launch_read_moments(const LevelBufs &b, double *out4, cudaStream_t s);
cudaError_t launch_row_support(const float *density, int n, int2 *sup, cudaStream_t s);
size_t rows_smem_bytes(int n);
cudaError_t rows_configure();
int update_blocks(int n);

}  // namespace cvtgb
