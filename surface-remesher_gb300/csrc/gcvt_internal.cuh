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
// "no label" inside jump flooding: the point (16383, 16383), farther from
// every pixel of a grid of side <= 8192 than any site
constexpr uint32_t kJfaNone = 0x3fff3fffu;
constexpr int kNoneAbove = -32768;  // "no site above" in the column summaries
constexpr int kNoneBelow = 32767;   // "no site below"
constexpr int kBand = 64;           // PBA+ phase-1 band height: n / m1 == 64 for
                                    // every entry of gcvt.cu:842-847
constexpr int kWarpSites = 8192;    // one site per warp up to this many sites
constexpr int kListWords = 512;    // bitmap words per site-list block
constexpr int kMinN = 256;   // n must be a multiple of 256 (S = n/32 >= 8)
constexpr int kMaxN = 8192;  // largest grid (the row pass's whole-row buffer: 32 KB)

__host__ __device__ inline uint32_t pack_xy(int x, int y) {
  return (uint32_t)(uint16_t)x | ((uint32_t)(uint16_t)y << 16);
}


// Per-context device state.  Kernels of one Lloyd iteration read it; the last
// block of the update kernel advances it, so a whole iteration runs without a
// host round trip and can be captured in a CUDA graph.
struct DevState {
  int cur;             // which of the three site bitmaps holds the current sites
  int iter;            // Lloyd iterations completed (gcvtIterations)
  int level_iters;     // iterations completed at the current level
  int stopped;         // set when the level's loop condition ends it
  int level;           // pyramid level (0 = finest)
  int max_iter;        // total iteration cap (maxIter)
  int use_stop_rule;   // 1: energy stop rule of gcvt.cu:1125-1140; 0: fixed count
  int fixed_iters;     // iterations per level when use_stop_rule == 0
  int window;          // initial half-size of the candidate window (pixels)
  unsigned done_blocks;
  float omega;         // over-relaxation (pbaOmega)
  float pad0;
  double last_energy;  // lastEnergy
  double sampled;      // Energy, sampled when iter % 10 == 0
  double energy;       // energy of the most recent iteration
  double energy_scale; // 4^level / n^2
  int cover;           // bound on |p - owner(p)| over the density pixels p
  unsigned cover_acc;  // max |p - owner(p)|^2 from the labels (k_cover)
  int list_count;      // sites in the site list (k_list)
  unsigned ticket;     // next 32-site group of the Lloyd kernel
  // The iteration's own view, copied by k_list before the iteration's k_cell
  // runs: the schedule (last warp of k_cell) changes the fields above for
  // the next iteration while other warps of the same launch may still start.
  int snap_cur, snap_stopped, snap_window, snap_cover, snap_count;
  float snap_omega;
  int hint_slack;      // window hint left for a site: 2 R + hint_slack (tuned)
  double target_energy; // > 0: the level also stops once an iteration's energy
                        // is at most this (time-to-energy runs); 0: off
  // Learned steps (learned.cu): the energy gate of a proposed jump.
  int gate_active;     // a jump is being judged (k_gate_switch .. k_gate_resolve)
  int gate_accept;     // the jumped sites' energy is below the sites' (k_cell MODE 5)
  unsigned gate_jump2; // largest squared jump of the proposal
  float feat_scale;    // mean cell radius: the unit of the learned features
  int gate_tried, gate_kept;  // jumps proposed / kept
  double gate_e0;      // energy of the sites the jump starts from
  double gate_e1;      // energy of the jumped sites
  // Labelling (labeller.cu): rows whose candidate hull did not fit the
  // bounded buffer of k_rows, for k_rows_full (zero between labellings).
  unsigned row_ovf[kMaxN / 32];
};

// Buffers of one resolution level, passed by value to every kernel.
struct LevelBufs {
  int n;
  uint64_t *bits[3];       // site bitmaps [band][column], bit i = row 64*band+i;
                           // the Lloyd kernel reads bits[cur], writes
                           // bits[cur+1] and clears bits[cur+2] (mod 3)
  int16_t *prev;           // [band][column]: nearest site row above the band
  int16_t *next;           // [band][column]: nearest site row below the band
  const float *density;    // n*n
  const int2 *support;     // per row [first, last+1) of nonzero density
  const int2 *sup_range;   // rows [x, y) containing every nonzero density
  const uint64_t *fixed_bits;  // fixed sites of this level, same layout as bits
  uint32_t *labels;        // n*n label words (label passes only)
  DevState *st;
  uint32_t *list;          // current sites in bitmap order: x | fixed << 15 | y << 16
  unsigned *counts[3];     // sites per kListWords words of bits[k]
  uint8_t *hint;           // per pixel: window half-size for the site there
  float4 *gslot;           // per 32-site group: energy (two-float), max cell
                           // radius^2 and max move^2 (as bits)
  float4 *sslot;           // per 64 groups: the same, reduced
  unsigned *scnt;          // per 64 groups: groups finished
  // learned steps (null when off): per pixel the last four moves of the site
  // there (int8 dx, dy each, newest in the low bytes) and (training runs
  // only) the site's id, one buffer per site bitmap (hist[k] describes the
  // sites of bits[k]); per list slot the site's features, the MLP's
  // prediction and the window of the site's cell (jaux); the state saved
  // before a jump, restored when the jump is rejected
  uint64_t *hist[3];
  int *ids[3];
  float *feat;
  float *pred;
  uint32_t *jaux;
  DevState *gsave;
  // one site per warp (small problems): per listed site its energy two-float,
  // cell radius^2 and move^2 until its group is reduced; per group the sites
  // done (null: lane-per-site only)
  float4 *sitev;
  unsigned *gcnt;
};

__device__ __forceinline__ const uint64_t *cur_bits(const LevelBufs &a) {
  const int c = a.st->cur;
  return c == 0 ? a.bits[0] : (c == 1 ? a.bits[1] : a.bits[2]);
}

// Kernels (launch helpers in labeller.cu / lloyd.cu / cells.cu).
cudaError_t launch_grid_to_bits(const uint32_t *grid, int n, uint64_t *bits, int *err,
                                int *count, cudaStream_t s);
// the site grid of a bitmap: pack_xy(x, y) per site (pack_xy(y, x) with
// swap), `empty` elsewhere
cudaError_t launch_bits_to_grid(const uint64_t *bits, int n, uint32_t *grid, cudaStream_t s,
                                uint32_t empty = kMarkerWord, bool swap = false);
// jump flooding's seeding: (x << 16) | y per site, kJfaNone elsewhere
inline cudaError_t launch_jfa_seed(const uint64_t *bits, int n, uint32_t *grid, cudaStream_t s) {
  return launch_bits_to_grid(bits, n, grid, s, kJfaNone, true);
}
cudaError_t launch_summary(const LevelBufs &b, int respect_stop, cudaStream_t s);
cudaError_t launch_fixed_bits(const uint8_t *mask, int n, uint64_t *fixed_bits, cudaStream_t s);
cudaError_t launch_rows(const LevelBufs &b, int respect_stop, cudaStream_t s);
cudaError_t launch_list(const LevelBufs &b, int respect_stop, cudaStream_t s);
cudaError_t launch_count(const LevelBufs &b, cudaStream_t s);
// MODE 0, 4 and 5 run one site per warp when b.sitev and b.gcnt are set,
// else one site per lane; MODE 1 and 2 run one site per lane.
cudaError_t launch_cells(const LevelBufs &b, int moments_only, double *out4, cudaStream_t s,
                         int grid = 0);
int cells_default_grid();
cudaError_t launch_zoom(const uint64_t *src, int n, uint64_t *dst, cudaStream_t s);
cudaError_t launch_density_halve(const float *in, float *out, int n_out, cudaStream_t s);
cudaError_t launch_row_support(const float *density, int n, int2 *sup, int2 *range,
                               unsigned long long *pixels, cudaStream_t s);
cudaError_t launch_cover(const LevelBufs &b, cudaStream_t s);
size_t rows_smem_bytes(int n);
cudaError_t rows_configure();
cudaError_t launch_extract(const uint64_t *bits, const uint64_t *fixed, int n, unsigned *colcnt,
                           double scale, double left, double lower, double *xy,
                           unsigned capacity, unsigned *total, cudaStream_t s);
int delaunay_sites(const uint64_t *bits, const uint64_t *fixed, int n, int *tris, unsigned cap,
                   unsigned *ntris, cudaStream_t s);
cudaError_t launch_list_batch(const LevelBufs *charts, int nchart, const unsigned *lofs,
                              unsigned nblocks, unsigned *gofs, unsigned *done, unsigned *ticket,
                              cudaStream_t s);
// MODE 0: plain iteration; 4: plain iteration + features of the learned step;
// 5: the jumped sites' iteration, which also judges the jump.
cudaError_t launch_cells_batch(const LevelBufs *charts, int nchart, const unsigned *gofs,
                               unsigned *ticket, cudaStream_t s, int mode = 0);
cudaError_t launch_jfa(uint32_t *a, uint32_t *b, int n, int *err, uint32_t **result,
                       cudaStream_t s, int tail_halo = 16);
cudaError_t launch_jfa_compare(const uint32_t *jfa, const uint32_t *exact, int n,
                               unsigned long long *counts, cudaStream_t s);
cudaError_t jfa_configure();
int mlp_param_count();
cudaError_t mlp_configure();
cudaError_t launch_mlp_infer(const float *feat, const int *count, const float *params_bf,
                             float *pred, int grid, cudaStream_t s);
cudaError_t launch_mlp_tc(const float *feat, const int *count, const float *params_bf,
                          float *pred, int *err, cudaStream_t s);
// A learned jump over the charts descs[0 .. nchart): jumped sites, gate
// switch, gate resolution (learned.cu).
cudaError_t launch_apply(const LevelBufs *descs, int nchart, cudaStream_t s);
cudaError_t launch_gate_switch(const LevelBufs *descs, int nchart, cudaStream_t s);
cudaError_t launch_gate_resolve(const LevelBufs *descs, int nchart, cudaStream_t s);
cudaError_t launch_features(const LevelBufs &b, int *ids, int *xy, int grid, cudaStream_t s);
cudaError_t launch_ids_init(const LevelBufs &b, int grid, cudaStream_t s);
cudaError_t launch_mlp_train_step(const float *samples, long long count, float *master,
                                  float *grad, float *m, float *v, float *params_bf, float *loss,
                                  int batch, unsigned long long seed, int step, float lr,
                                  cudaStream_t s);
cudaError_t launch_mlp_grad(const float *samples, long long count, const float *master,
                            float *grad, float *loss, int batch, unsigned long long seed, int step,
                            cudaStream_t s);
cudaError_t launch_round_params(const float *master, float *params_bf, cudaStream_t s);
// Grow-only device scratch for one call of a one-shot entry point; holds the
// device's scratch lock for its lifetime (calls on a device serialise).
// take() returns 256-byte aligned device memory valid until the Scratch is
// destroyed, or nullptr when no memory can be had.  The destructor waits for
// `stream` (the stream the call queues its work on) before it releases the
// lock, so a call that returns early with kernels still queued cannot hand
// memory they use to the next call.
class Scratch {
 public:
  explicit Scratch(cudaStream_t stream = nullptr);
  ~Scratch();
  Scratch(const Scratch &) = delete;
  Scratch &operator=(const Scratch &) = delete;
  void *take(size_t bytes);
  template <class T> T *take(size_t count) { return static_cast<T *>(take(count * sizeof(T))); }

 private:
  void *pool_;
  cudaStream_t stream_;
  size_t block_, used_, total_;
  bool ok_;
};

int delaunay_sites_in(const uint64_t *bits, const uint64_t *fixed, int n, int *tris,
                      unsigned cap, unsigned *ntris, cudaStream_t s, Scratch &sc);
int cdt_compute(const uint64_t *bits, const uint64_t *fixed, int n, unsigned *colcnt,
                const double *cxy, int C, const int *segs, int S, double scale, double left,
                double lower, int *out, unsigned cap, unsigned *ntris, int *detail,
                cudaStream_t s);

// Exclusive scan of n counts into offset[0..n] (offset[n] = total) and a copy
// in cursor[0..n-1]; one block, n <= 2^26.
cudaError_t launch_scan(const int *count, int n, int *offset, int *cursor, cudaStream_t s);
cudaError_t cells_configure();
size_t list_blocks(int n);
size_t cell_groups(int n);

}  // namespace cvtgb
