// api.cu -- host side of libgcvt_gb300.so: the context (device buffers
// allocated once), the Lloyd driver of gCVT (gcvt.cu:1087-1156) and the C ABI
// declared in include/gcvt_gb300.h.
//
// One Lloyd iteration is two launches (cells.cu: site list, cells) that read
// their buffer roles and the omega / stop state from device memory, so ten
// iterations are captured once as a CUDA graph and replayed.  The host reads the state back once per
// ten iterations, where the reference's schedule can end a level
// (gcvt.cu:1125-1140).  Label grids come from the PBA+ passes (labeller.cu).
#include "gcvt_internal.cuh"
#include "../../include/gcvt_gb300.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

using namespace cvtgb;

struct gcvt_ctx {
  int device = 0;
  int n_max = 0;
  int n = 0;            // loaded problem size
  int loaded = 0;
  int input_err = 0;    // the loaded grid is malformed at full resolution
  int cur_n = 0;        // size of the level currently held in the bitmaps
  int sites = 0;        // sites in the grid the bitmaps were built from
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  float *density[8] = {};      // pyramid, [0] = full resolution
  int2 *support[8] = {};       // per level: [first, last+1) of nonzero density per row
  int2 *sup_range[8] = {};     // per level: rows holding nonzero density
  uint64_t *fixed_bits[8] = {};
  unsigned long long *sup_pixels = nullptr;  // per level: pixels of nonzero density
  uint8_t *mask = nullptr;
  uint32_t *input = nullptr;  // the loaded site grid, kept for gcvt_ctx_run
  uint32_t *grid = nullptr;   // staging: labels and site dumps
  uint64_t *bits[3] = {};
  int16_t *prev = nullptr, *next = nullptr;
  DevState *st = nullptr;
  DevState *st_host = nullptr;  // pinned mirror
  uint32_t *list = nullptr;     // site list, n_max^2 entries
  unsigned *counts[3] = {};     // per bitmap: sites per list block
  uint8_t *hint = nullptr;      // per pixel window hints
  float4 *gslot = nullptr, *sslot = nullptr;
  unsigned *scnt = nullptr;
  unsigned *colcnt = nullptr;   // point extraction: n_max column counts + total
  uint32_t *jfa = nullptr;      // jump flooding: two n_max^2 label grids + counters
  // tuning (gcvt_ctx_autotune): persistent Lloyd grid in blocks (0: all that
  // fit), window hint slack, jump-flooding fusion depth (tail halo)
  int cell_grid = 0;
  int hint_slack = 2;
  int jfa_halo = 0;             // jump flooding: 0 = every step its own launch
  int cell_mode = 0;            // 0 auto, 1 one site per lane, 2 one site per warp
  float4 *sitev = nullptr;      // one site per warp: kWarpSites site values
  unsigned *gcnt = nullptr;     //   and kWarpSites / 32 group counters
  // learned steps (gcvt_ctx_learning): histories, ids, features, predictions,
  // bfloat16-rounded MLP parameters
  int learning = 0, track_ids = 0, have_mlp = 0;
  int mlp_tensor_cores = 1;  // MLP forward on tcgen05 (else CUDA cores)
  uint64_t *hist[3] = {};    // one per site bitmap
  int *ids[3] = {};
  float *feat = nullptr, *pred = nullptr, *mlp_bf = nullptr;
  uint32_t *jaux = nullptr;  // per list slot: the window of the site's cell
  DevState *gsave = nullptr; // the state a rejected jump restores
  LevelBufs *desc = nullptr; // device copy of the level's buffers (learned steps)
  size_t feat_cap = 0;
  double target_energy = 0;  // gcvt_ctx_set_target_energy
  int cover_valid = 0;          // the covering bound, list counts and hints
                                // fit the current sites
  double *moments = nullptr;    // 4*n_max^2 doubles, allocated on first use
  int *err = nullptr;           // [0] malformed-grid flag, [1] site count
  int last_levels = 0;
  cudaGraphExec_t chunk_exec = nullptr;  // kChunk iterations of one level
  int chunk_n = 0;
  int chunk_level = -1;
};

namespace {

constexpr int kChunk = 10;  // iterations per graph; the schedule acts every 10

#define CK(call)                                  \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return GCVT_ERR_CUDA;  \
  } while (0)

bool valid_n(int n) { return n >= kMinN && n <= kMaxN && n % 256 == 0; }
bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
size_t bits_words(int n) { return (size_t)(n / kBand) * n; }

LevelBufs level_bufs(gcvt_ctx *c, int n, int level) {
  LevelBufs b = {};
  b.n = n;
  for (int k = 0; k < 3; ++k) b.bits[k] = c->bits[k];
  b.prev = c->prev;
  b.next = c->next;
  b.density = c->density[level];
  b.support = c->support[level];
  b.sup_range = c->sup_range[level];
  b.fixed_bits = c->fixed_bits[level];
  b.labels = c->grid;
  b.st = c->st;
  b.list = c->list;
  for (int k = 0; k < 3; ++k) b.counts[k] = c->counts[k];
  b.hint = c->hint;
  b.gslot = c->gslot;
  b.sslot = c->sslot;
  b.scnt = c->scnt;
  // one site per warp when the sites are too few to fill the GPU one per lane
  if (c->cell_mode == 2 || (c->cell_mode == 0 && c->sites <= kWarpSites)) {
    b.sitev = c->sitev;
    b.gcnt = c->gcnt;
  }
  if (c->learning && level == 0) {
    for (int k = 0; k < 3; ++k) {
      b.hist[k] = c->hist[k];
      if (c->track_ids) b.ids[k] = c->ids[k];
    }
    b.feat = c->feat;
    b.pred = c->pred;
    b.jaux = c->jaux;
    b.gsave = c->gsave;
  }
  return b;
}

int pull_state(gcvt_ctx *c) {
  CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return GCVT_OK;
}

int push_state(gcvt_ctx *c) {
  CK(cudaMemcpyAsync(c->st, c->st_host, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
  return GCVT_OK;
}

// Enqueue kChunk Lloyd iterations through a CUDA graph captured once per
// (size, level); a stream that cannot be captured (the legacy default stream)
// gets plain launches.
int enqueue_chunk(gcvt_ctx *c, int n, int level) {
  if (c->chunk_exec && (c->chunk_n != n || c->chunk_level != level)) {
    cudaGraphExecDestroy(c->chunk_exec);
    c->chunk_exec = nullptr;
  }
  const LevelBufs b = level_bufs(c, n, level);
  if (!c->chunk_exec) {
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      for (int i = 0; i < kChunk; ++i) {
        CK(launch_list(b, 1, c->stream));
        CK(launch_cells(b, 0, nullptr, c->stream, c->cell_grid));
      }
      return GCVT_OK;
    }
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < kChunk && le == cudaSuccess; ++i) {
      le = launch_list(b, 1, c->stream);
      if (le == cudaSuccess) le = launch_cells(b, 0, nullptr, c->stream, c->cell_grid);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return GCVT_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&c->chunk_exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      c->chunk_exec = nullptr;
      return GCVT_ERR_CUDA;
    }
    c->chunk_n = n;
    c->chunk_level = level;
  }
  CK(cudaGraphLaunch(c->chunk_exec, c->stream));
  return GCVT_OK;
}

// Sites of level size n go to size 2n (gcvt.cu:1036-1051): zoom from the
// current bitmap into the next one, clear the other two.
int zoom_level(gcvt_ctx *c, int n) {
  int rc = pull_state(c);
  if (rc) return rc;
  const int p = c->st_host->cur, q = (p + 1) % 3, r = (p + 2) % 3;
  const size_t bytes2 = bits_words(2 * n) * sizeof(uint64_t);
  CK(cudaMemsetAsync(c->bits[q], 0, bytes2, c->stream));
  CK(launch_zoom(c->bits[p], n, c->bits[q], c->stream));
  c->cover_valid = 0;
  CK(cudaMemsetAsync(c->bits[p], 0, bytes2, c->stream));
  CK(cudaMemsetAsync(c->bits[r], 0, bytes2, c->stream));
  c->st_host->cur = q;
  return push_state(c);
}

// What the Lloyd kernel carries from one iteration to the next, set up for
// the current sites of size n: the covering bound (label the sites, take the
// largest pixel-to-owner distance over the density support), the site counts
// of the current bitmap, zero counts for the next one, no window hints.
int ensure_cover(gcvt_ctx *c, int n, int level) {
  if (c->cover_valid) return GCVT_OK;
  int rc = pull_state(c);
  if (rc) return rc;
  const LevelBufs b = level_bufs(c, n, level);
  CK(launch_summary(b, 0, c->stream));
  CK(launch_rows(b, 0, c->stream));
  CK(cudaMemsetAsync(c->hint, 0, (size_t)n * n, c->stream));
  CK(launch_cover(b, c->stream));  // also each site's first window (hint)
  CK(launch_count(b, c->stream));
  const size_t nlb = list_blocks(n);
  CK(cudaMemsetAsync(c->counts[(c->st_host->cur + 1) % 3], 0, nlb * sizeof(unsigned), c->stream));
  if (c->learning && level == 0) {  // no moves yet; ids = list positions
    CK(cudaMemsetAsync(c->hist[c->st_host->cur], 0, (size_t)n * n * sizeof(uint64_t),
                       c->stream));
    if (c->track_ids) {
      CK(launch_list(b, 0, c->stream));
      CK(launch_ids_init(b, 4 * 152, c->stream));
    }
  }
  c->cover_valid = 1;
  return GCVT_OK;
}

// Initial half-size of the candidate window at a level: 2.5 mean cell radii
// (mean cell area = density pixels / sites).  Only a starting guess: a cell
// whose certificate fails grows its own window.
int initial_window(gcvt_ctx *c, int level, int *w, float *radius = nullptr) {
  unsigned long long pix = 0;
  CK(cudaMemcpyAsync(&pix, c->sup_pixels + level, sizeof(pix), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const double per_site = c->sites > 0 ? (double)pix / c->sites : 64.0;
  const int v = (int)std::ceil(2.5 * std::sqrt(per_site / 3.14159265358979));
  *w = v < 2 ? 2 : (v > 1024 ? 1024 : v);
  if (radius) {  // mean cell radius
    const double r = std::sqrt(per_site / 3.14159265358979);
    *radius = (float)(r > 0.5 ? r : 0.5);
  }
  return GCVT_OK;
}

// Run one level until the device schedule stops it.  fixed > 0: exactly that
// many iterations without the stop rule.
// Start a level on the device: schedule state (fixed > 0: that many
// iterations without the stop rule), covering bound, list counts, hints.
int start_level(gcvt_ctx *c, int n, int level, int fixed, int max_iter) {
  int window = 0;
  float radius = 1.f;
  int rc = initial_window(c, level, &window, &radius);
  if (rc) return rc;
  if ((rc = pull_state(c))) return rc;
  DevState &h = *c->st_host;
  h.level = level;
  h.stopped = 0;
  h.level_iters = 0;
  h.use_stop_rule = fixed > 0 ? 0 : 1;
  h.fixed_iters = fixed;
  h.max_iter = max_iter;
  h.window = window;
  h.energy_scale = std::pow(4.0, level) / ((double)n * (double)n);
  h.done_blocks = 0;
  h.hint_slack = c->hint_slack;
  h.feat_scale = radius;
  h.target_energy = level == 0 ? c->target_energy : 0.0;
  if ((rc = push_state(c))) return rc;
  c->cur_n = n;
  return ensure_cover(c, n, level);
}

int run_level(gcvt_ctx *c, int n, int level, int fixed, int max_iter, int poll) {
  int rc = start_level(c, n, level, fixed, max_iter);
  if (rc) return rc;
  if (fixed > 0 && !poll) {
    for (int done = 0; done < fixed; done += kChunk)
      if ((rc = enqueue_chunk(c, n, level))) return rc;
    return GCVT_OK;
  }
  for (;;) {
    if ((rc = enqueue_chunk(c, n, level))) return rc;
    if ((rc = pull_state(c))) return rc;
    if (c->st_host->stopped) return GCVT_OK;
  }
}

int copy_in(void *dst, const void *src, size_t bytes, int mem, cudaStream_t s) {
  CK(cudaMemcpyAsync(dst, src, bytes,
                     mem == GCVT_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
  return GCVT_OK;
}

int copy_out(void *dst, const void *src, size_t bytes, int mem, cudaStream_t s) {
  CK(cudaMemcpyAsync(dst, src, bytes,
                     mem == GCVT_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  if (mem == GCVT_MEM_HOST) CK(cudaStreamSynchronize(s));
  return GCVT_OK;
}

int reset_schedule(gcvt_ctx *c) {
  DevState &h = *c->st_host;
  std::memset(&h, 0, sizeof(DevState));
  h.cur = 0;
  h.omega = 2.0f;           // gcvt.cu:1108
  h.last_energy = 1e18;     // gcvt.cu:1105
  h.max_iter = 0x7fffffff;
  h.window = 8;
  return push_state(c);
}

// Density-side tables of one level: row support, row range and pixel count
// of the nonzero density, fixed-site bitmap.
int level_tables(gcvt_ctx *c, int n, int level) {
  CK(launch_row_support(c->density[level], n, c->support[level], c->sup_range[level],
                        c->sup_pixels + level, c->stream));
  CK(launch_fixed_bits(c->mask, n, c->fixed_bits[level], c->stream));
  return GCVT_OK;
}

// Build bitmap 0 from a device site grid of size n (pba2DInitializeInput's
// site part), clear the other two, reset the schedule; reports whether the
// grid is well formed and counts its sites.
int build_sites(gcvt_ctx *c, const uint32_t *grid, int n, int *bad) {
  const size_t bytes = bits_words(c->n_max) * sizeof(uint64_t);
  for (int k = 0; k < 3; ++k) CK(cudaMemsetAsync(c->bits[k], 0, bytes, c->stream));
  CK(cudaMemsetAsync(c->err, 0, 2 * sizeof(int), c->stream));
  CK(launch_grid_to_bits(grid, n, c->bits[0], c->err, c->err + 1, c->stream));
  int h[2] = {0, 0};
  CK(cudaMemcpyAsync(h, c->err, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  int rc = reset_schedule(c);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  c->cover_valid = 0;
  *bad = h[0] != 0;
  c->sites = h[1];
  return GCVT_OK;
}

// Upload a site grid; a malformed grid is recorded and reported by the calls
// that need the sites (gcvt_ctx_run validates its own coarse grid instead).
int load_sites(gcvt_ctx *c, int n, const int16_t *voronoi, int mem) {
  c->loaded = 0;
  int rc = copy_in(c->input, voronoi, (size_t)n * n * sizeof(uint32_t), mem, c->stream);
  if (rc) return rc;
  int bad = 0;
  if ((rc = build_sites(c, c->input, n, &bad))) return rc;
  c->input_err = bad;
  c->n = n;
  c->cur_n = n;
  c->loaded = 1;
  return GCVT_OK;
}

int level_of(gcvt_ctx *c, int n) {
  int level = 0;
  while (level < 7 && (c->n >> level) != n) ++level;
  return level;
}

}  // namespace

extern "C" {

const char *gcvt_status_string(int status) {
  switch (status) {
    case GCVT_OK: return "ok";
    case GCVT_ERR_ARGUMENT: return "invalid argument";
    case GCVT_ERR_SIZE: return "unsupported grid size";
    case GCVT_ERR_CUDA: return "CUDA runtime error";
    case GCVT_ERR_INPUT: return "site grid pixel does not hold its own coordinates";
    case GCVT_ERR_STATE: return "no problem loaded";
    case GCVT_ERR_ALLOC: return "allocation failed";
  }
  return "unknown status";
}

int gcvt_version(void) { return 10100; }

int gcvt_ctx_create(int n_max, gcvt_ctx **out) {
  if (!out) return GCVT_ERR_ARGUMENT;
  *out = nullptr;
  if (!valid_n(n_max)) return GCVT_ERR_SIZE;
  gcvt_ctx *c = new (std::nothrow) gcvt_ctx();
  if (!c) return GCVT_ERR_ALLOC;
  auto fail = [&](int code) {
    gcvt_ctx_destroy(c);
    return code;
  };
  if (cudaGetDevice(&c->device) != cudaSuccess) return fail(GCVT_ERR_CUDA);
  if (rows_configure() != cudaSuccess) return fail(GCVT_ERR_CUDA);
  if (cells_configure() != cudaSuccess) return fail(GCVT_ERR_CUDA);
  c->n_max = n_max;
  const size_t nn = (size_t)n_max * n_max;
  const size_t words = bits_words(n_max);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(GCVT_ERR_CUDA);
  c->stream = c->own_stream;
  auto dal = [](void *p, size_t bytes) {
    return cudaMalloc(reinterpret_cast<void **>(p), bytes) == cudaSuccess;
  };
  bool ok = true;
  for (int l = 0; l < 8 && ok; ++l) {
    const int nl = n_max >> l;
    if (nl < kMinN) break;
    ok = ok && dal(&c->density[l], (size_t)nl * nl * sizeof(float));
    ok = ok && dal(&c->support[l], (size_t)nl * sizeof(int2));
    ok = ok && dal(&c->sup_range[l], sizeof(int2));
    ok = ok && dal(&c->fixed_bits[l], bits_words(nl) * sizeof(uint64_t));
  }
  ok = ok && dal(&c->sup_pixels, 8 * sizeof(unsigned long long));
  ok = ok && dal(&c->mask, nn);
  ok = ok && dal(&c->input, nn * sizeof(uint32_t));
  ok = ok && dal(&c->grid, nn * sizeof(uint32_t));
  for (int k = 0; k < 3; ++k) ok = ok && dal(&c->bits[k], words * sizeof(uint64_t));
  ok = ok && dal(&c->prev, words * sizeof(int16_t));
  ok = ok && dal(&c->next, words * sizeof(int16_t));
  ok = ok && dal(&c->st, sizeof(DevState));
  ok = ok && dal(&c->list, nn * sizeof(uint32_t));
  for (int k = 0; k < 3; ++k) ok = ok && dal(&c->counts[k], list_blocks(n_max) * sizeof(unsigned));
  ok = ok && dal(&c->hint, nn);
  const size_t groups = cell_groups(n_max), slots = (groups + 63) / 64;
  ok = ok && dal(&c->gslot, groups * sizeof(float4));
  ok = ok && dal(&c->sslot, slots * sizeof(float4));
  ok = ok && dal(&c->scnt, slots * sizeof(unsigned));
  ok = ok && dal(&c->sitev, kWarpSites * sizeof(float4));
  ok = ok && dal(&c->gcnt, (kWarpSites / 32) * sizeof(unsigned));
  ok = ok && dal(&c->colcnt, ((size_t)n_max + 1) * sizeof(unsigned));
  ok = ok && dal(&c->err, 2 * sizeof(int));
  if (!ok) return fail(GCVT_ERR_ALLOC);
  if (cudaMemsetAsync(c->scnt, 0, slots * sizeof(unsigned), c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->gcnt, 0, (kWarpSites / 32) * sizeof(unsigned), c->stream) != cudaSuccess)
    return fail(GCVT_ERR_CUDA);
  if (cudaMallocHost(reinterpret_cast<void **>(&c->st_host), sizeof(DevState)) != cudaSuccess)
    return fail(GCVT_ERR_ALLOC);
  for (int k = 0; k < 3; ++k)
    if (cudaMemsetAsync(c->bits[k], 0, words * sizeof(uint64_t), c->stream) != cudaSuccess)
      return fail(GCVT_ERR_CUDA);
  if (reset_schedule(c) != GCVT_OK) return fail(GCVT_ERR_CUDA);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(GCVT_ERR_CUDA);
  *out = c;
  return GCVT_OK;
}

int gcvt_ctx_destroy(gcvt_ctx *c) {
  if (!c) return GCVT_ERR_ARGUMENT;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->chunk_exec) cudaGraphExecDestroy(c->chunk_exec);
  for (int l = 0; l < 8; ++l) {
    cudaFree(c->density[l]);
    cudaFree(c->support[l]);
    cudaFree(c->sup_range[l]);
    cudaFree(c->fixed_bits[l]);
  }
  cudaFree(c->sup_pixels);
  cudaFree(c->mask);
  cudaFree(c->input);
  cudaFree(c->grid);
  for (int k = 0; k < 3; ++k) cudaFree(c->bits[k]);
  cudaFree(c->prev);
  cudaFree(c->next);
  cudaFree(c->st);
  cudaFree(c->list);
  for (int k = 0; k < 3; ++k) cudaFree(c->counts[k]);
  cudaFree(c->hint);
  cudaFree(c->gslot);
  cudaFree(c->sslot);
  cudaFree(c->scnt);
  cudaFree(c->sitev);
  cudaFree(c->gcnt);
  cudaFree(c->colcnt);
  cudaFree(c->jfa);
  for (int k = 0; k < 3; ++k) {
    cudaFree(c->hist[k]);
    cudaFree(c->ids[k]);
  }
  cudaFree(c->feat);
  cudaFree(c->pred);
  cudaFree(c->jaux);
  cudaFree(c->gsave);
  cudaFree(c->desc);
  cudaFree(c->mlp_bf);
  cudaFree(c->moments);
  cudaFree(c->err);
  if (c->st_host) cudaFreeHost(c->st_host);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return GCVT_OK;
}

int gcvt_ctx_set_stream(gcvt_ctx *c, void *stream) {
  if (!c) return GCVT_ERR_ARGUMENT;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return GCVT_OK;
}

int gcvt_ctx_load(gcvt_ctx *c, int n, const int16_t *voronoi, const float *density,
                  const uint8_t *mask, int mem) {
  if (!c || !voronoi || !density) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!valid_n(n) || n > c->n_max) return GCVT_ERR_SIZE;
  const size_t nn = (size_t)n * n;
  int rc;
  c->loaded = 0;
  if ((rc = copy_in(c->density[0], density, nn * sizeof(float), mem, c->stream))) return rc;
  if (mask) {
    if ((rc = copy_in(c->mask, mask, nn, mem, c->stream))) return rc;
  } else {
    CK(cudaMemsetAsync(c->mask, 0, nn, c->stream));
  }
  if ((rc = level_tables(c, n, 0))) return rc;
  return load_sites(c, n, voronoi, mem);
}

int gcvt_ctx_label(gcvt_ctx *c, int16_t *labels, int mem) {
  if (!c || !labels) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  const int n = c->cur_n;
  const LevelBufs b = level_bufs(c, n, level_of(c, n));
  CK(launch_summary(b, 0, c->stream));
  CK(launch_rows(b, 0, c->stream));
  return copy_out(labels, c->grid, (size_t)n * n * sizeof(uint32_t), mem, c->stream);
}

int gcvt_ctx_iterate(gcvt_ctx *c, int iterations) {
  if (!c || iterations < 0) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  if (iterations == 0) return GCVT_OK;
  if (c->cur_n != c->n) return GCVT_ERR_STATE;
  return run_level(c, c->n, 0, iterations, 0x7fffffff, c->target_energy > 0.0);
}

int gcvt_ctx_run(gcvt_ctx *c, int depth, int max_iter, gcvt_run_info *info) {
  if (!c || depth < 1) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  const int size = c->n;
  if (!pow2(size)) return GCVT_ERR_SIZE;
  for (int i = 0; i < depth; ++i)       // gcvt.cu:1091
    if ((size >> i) < 256) { depth = i; break; }
  int rc;
  // density pyramid (gcvt.cu:985-993) and its tables
  for (int l = 1; l < depth; ++l) {
    CK(launch_density_halve(c->density[l - 1], c->density[l], size >> l, c->stream));
    if ((rc = level_tables(c, size >> l, l))) return rc;
  }
  // the coarsest grid is the first (size >> (depth-1))^2 entries of the loaded
  // array (gcvt.cu:1099-1103)
  const int n0 = size >> (depth - 1);
  int bad = 0;
  if ((rc = build_sites(c, c->input, n0, &bad))) return rc;
  if (bad) return GCVT_ERR_INPUT;
  c->input_err = 0;
  c->cur_n = n0;
  int levels = 0;
  for (int level = depth - 1; level >= 0; --level) {
    const int n = size >> level;
    ++levels;
    if ((rc = run_level(c, n, level, 0, max_iter, 1))) return rc;
    if (level) {
      if ((rc = zoom_level(c, n))) return rc;
      c->cur_n = 2 * n;
    }
  }
  c->last_levels = levels;
  return gcvt_ctx_info(c, info);
}

int gcvt_ctx_sites(gcvt_ctx *c, int16_t *voronoi, int mem) {
  if (!c || !voronoi) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  int rc = pull_state(c);
  if (rc) return rc;
  const int n = c->cur_n;
  CK(launch_bits_to_grid(c->bits[c->st_host->cur], n, c->grid, c->stream));
  return copy_out(voronoi, c->grid, (size_t)n * n * sizeof(uint32_t), mem, c->stream);
}

int gcvt_ctx_moments(gcvt_ctx *c, double *out4, int mem) {
  if (!c || !out4) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  const int n = c->cur_n;
  const int level = level_of(c, n);
  if (!c->moments &&
      cudaMalloc(reinterpret_cast<void **>(&c->moments),
                 (size_t)4 * c->n_max * c->n_max * sizeof(double)) != cudaSuccess)
    return GCVT_ERR_ALLOC;
  int window = 0;
  int rc = initial_window(c, level, &window);
  if (rc) return rc;
  if ((rc = pull_state(c))) return rc;
  c->st_host->window = window;
  if ((rc = push_state(c))) return rc;
  if ((rc = ensure_cover(c, n, level))) return rc;
  CK(cudaMemsetAsync(c->moments, 0, (size_t)4 * n * n * sizeof(double), c->stream));
  const LevelBufs b = level_bufs(c, n, level);
  CK(launch_list(b, 0, c->stream));
  CK(launch_cells(b, 1, c->moments, c->stream, c->cell_grid));
  return copy_out(out4, c->moments, (size_t)4 * n * n * sizeof(double), mem, c->stream);
}

int gcvt_ctx_extract_points(gcvt_ctx *c, double scale, double left, double lower, double *xy,
                            int capacity, int *count, int mem) {
  if (!c || !count || capacity < 0 || (capacity > 0 && !xy)) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  int rc = pull_state(c);
  if (rc) return rc;
  const int n = c->cur_n;
  const int level = level_of(c, n);
  double *dst = xy;
  if (mem == GCVT_MEM_HOST) {  // stage in the moments buffer (32 B per pixel >= 16 B per point)
    if (!c->moments &&
        cudaMalloc(reinterpret_cast<void **>(&c->moments),
                   (size_t)4 * c->n_max * c->n_max * sizeof(double)) != cudaSuccess)
      return GCVT_ERR_ALLOC;
    dst = c->moments;
  }
  const unsigned cap = (unsigned)capacity;
  CK(launch_extract(c->bits[c->st_host->cur], c->fixed_bits[level], n, c->colcnt, scale, left,
                    lower, dst, cap, c->colcnt + c->n_max, c->stream));
  unsigned total = 0;
  CK(cudaMemcpyAsync(&total, c->colcnt + c->n_max, sizeof(unsigned), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *count = (int)total;
  const size_t written = total < cap ? total : cap;
  if (mem == GCVT_MEM_HOST && written)
    return copy_out(xy, dst, written * 2 * sizeof(double), GCVT_MEM_HOST, c->stream);
  return GCVT_OK;
}

int gcvt_ctx_delaunay(gcvt_ctx *c, int32_t *triangles, int capacity, int *count, int mem) {
  if (!c || !count || capacity < 0 || (capacity > 0 && !triangles)) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  int rc = pull_state(c);
  if (rc) return rc;
  const int n = c->cur_n;
  const int level = level_of(c, n);
  const unsigned cap = (unsigned)capacity;
  int32_t *dst = mem == GCVT_MEM_HOST ? nullptr : triangles;
  bool owned = false;
  if (mem == GCVT_MEM_HOST && cap) {
    // device staging: the label grid's buffer when it holds the triangles
    if ((size_t)cap * 3 * sizeof(int32_t) <= (size_t)c->n_max * c->n_max * sizeof(uint32_t)) {
      dst = reinterpret_cast<int32_t *>(c->grid);
    } else {
      if (cudaMalloc(reinterpret_cast<void **>(&dst), (size_t)cap * 3 * sizeof(int32_t)) !=
          cudaSuccess)
        return GCVT_ERR_ALLOC;
      owned = true;
    }
  }
  unsigned total = 0;
  rc = delaunay_sites(c->bits[c->st_host->cur], c->fixed_bits[level], n, dst, cap, &total,
                      c->stream);
  if (!rc) {
    *count = (int)total;
    const size_t written = total < cap ? total : cap;
    if (mem == GCVT_MEM_HOST && written)
      rc = copy_out(triangles, dst, written * 3 * sizeof(int32_t), GCVT_MEM_HOST, c->stream);
  }
  if (owned) cudaFree(dst);
  return rc;
}

int gcvt_ctx_cdt(gcvt_ctx *c, double scale, double left, double lower, const double *cpoints,
                 int num_cpoints, const int32_t *segments, int num_segments, int32_t *triangles,
                 int capacity, int *count, int *detail, int mem) {
  if (!c || !count || capacity < 0 || (capacity > 0 && !triangles) || num_cpoints < 0 ||
      num_segments < 0 || (num_cpoints && !cpoints) || (num_segments && !segments))
    return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  int rc = pull_state(c);
  if (rc) return rc;
  const int n = c->cur_n;
  const int level = level_of(c, n);
  const double *dpts = cpoints;
  const int *dsegs = segments;
  int *dtri = triangles;
  void *stage = nullptr;
  if (mem == GCVT_MEM_HOST) {  // device copies of the inputs and the triangles
    const size_t bp = (size_t)num_cpoints * 2 * sizeof(double),
                 bs = (size_t)num_segments * 2 * sizeof(int32_t),
                 bt = (size_t)capacity * 3 * sizeof(int32_t);
    if (cudaMalloc(&stage, bp + bs + bt + 64) != cudaSuccess) return GCVT_ERR_ALLOC;
    char *q = static_cast<char *>(stage);
    dpts = reinterpret_cast<const double *>(q);
    dsegs = reinterpret_cast<const int *>(q + bp);
    dtri = reinterpret_cast<int *>(q + ((bp + bs + 15) & ~(size_t)15));
    if ((bp && cudaMemcpyAsync(q, cpoints, bp, cudaMemcpyHostToDevice, c->stream) !=
                   cudaSuccess) ||
        (bs && cudaMemcpyAsync(q + bp, segments, bs, cudaMemcpyHostToDevice, c->stream) !=
                   cudaSuccess)) {
      cudaFree(stage);
      return GCVT_ERR_CUDA;
    }
  }
  unsigned total = 0;
  rc = cdt_compute(c->bits[c->st_host->cur], c->fixed_bits[level], n, c->colcnt, dpts,
                   num_cpoints, dsegs, num_segments, scale, left, lower, dtri,
                   (unsigned)capacity, &total, detail, c->stream);
  if (!rc) {
    *count = (int)total;
    const size_t written = total < (unsigned)capacity ? total : (unsigned)capacity;
    if (mem == GCVT_MEM_HOST && written)
      rc = copy_out(triangles, dtri, written * 3 * sizeof(int32_t), GCVT_MEM_HOST, c->stream);
  }
  if (stage) {
    cudaStreamSynchronize(c->stream);
    cudaFree(stage);
  }
  return rc;
}

int gcvt_ctx_jfa_label(gcvt_ctx *c, int16_t *labels, unsigned long long *stats, int mem) {
  if (!c || (!labels && !stats)) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  const size_t nmax2 = (size_t)c->n_max * c->n_max;
  if (!c->jfa && cudaMalloc(reinterpret_cast<void **>(&c->jfa),
                            2 * nmax2 * sizeof(uint32_t) + 64) != cudaSuccess)
    return GCVT_ERR_ALLOC;
  int rc = pull_state(c);
  if (rc) return rc;
  const int n = c->cur_n;
  uint32_t *a = c->jfa, *b = c->jfa + nmax2;
  unsigned long long *counts = reinterpret_cast<unsigned long long *>(c->jfa + 2 * nmax2);
  CK(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
  CK(launch_jfa_seed(c->bits[c->st_host->cur], n, a, c->stream));
  uint32_t *res = nullptr;
  CK(launch_jfa(a, b, n, c->err, &res, c->stream, c->jfa_halo));
  if (stats) {
    const LevelBufs lb = level_bufs(c, n, level_of(c, n));
    CK(launch_summary(lb, 0, c->stream));
    CK(launch_rows(lb, 0, c->stream));  // exact labels into the staging grid
    CK(cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), c->stream));
    CK(launch_jfa_compare(res, c->grid, n, counts, c->stream));
    unsigned long long h[2] = {0, 0};
    CK(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    stats[0] = h[0];
    stats[1] = h[1];
    stats[2] = (unsigned long long)n * n;
  }
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, c->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (herr) return GCVT_ERR_CUDA;  // a tile copy did not arrive
  if (labels) return copy_out(labels, res, (size_t)n * n * sizeof(uint32_t), mem, c->stream);
  return GCVT_OK;
}

int gcvt_ctx_set_tuning(gcvt_ctx *c, const gcvt_tuning *t) {
  if (!c || !t) return GCVT_ERR_ARGUMENT;
  if (t->cell_blocks_per_sm < 0 || t->cell_blocks_per_sm > 32 || t->hint_slack < 0 ||
      t->hint_slack > 64 || (t->jfa_tail_halo != 0 && t->jfa_tail_halo != 8 &&
                             t->jfa_tail_halo != 16 && t->jfa_tail_halo != 32) ||
      t->cell_mode < 0 || t->cell_mode > 2)
    return GCVT_ERR_ARGUMENT;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess)
    return GCVT_ERR_CUDA;
  const int grid = t->cell_blocks_per_sm * sms;
  if ((grid != c->cell_grid || t->cell_mode != c->cell_mode) && c->chunk_exec) {
    cudaGraphExecDestroy(c->chunk_exec);  // the captured launches change
    c->chunk_exec = nullptr;
  }
  c->cell_grid = grid;
  c->cell_mode = t->cell_mode;
  c->hint_slack = t->hint_slack;
  c->jfa_halo = t->jfa_tail_halo;
  return GCVT_OK;
}

int gcvt_ctx_autotune(gcvt_ctx *c, gcvt_tuning *out) {
  if (!c) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  if (c->cur_n != c->n) return GCVT_ERR_STATE;
  const int n = c->n;
  int rc = pull_state(c);
  if (rc) return rc;
  // save what iterations change
  const size_t wbytes = bits_words(n) * sizeof(uint64_t), cbytes = list_blocks(n) * sizeof(unsigned);
  const size_t hbytes = (size_t)n * n;
  const size_t total = 3 * wbytes + 3 * cbytes + hbytes + sizeof(DevState);
  unsigned char *save = nullptr;  // [0, total): the state to return to; [total, 2 total): the base
  if (cudaMalloc(reinterpret_cast<void **>(&save), 2 * total) != cudaSuccess)
    return GCVT_ERR_ALLOC;
  DevState saved_host = *c->st_host;
  const int saved_valid = c->cover_valid;
  size_t slot = 0;  // which copy copy_state uses
  auto copy_state = [&](bool to_save) -> int {
    size_t off = slot;
    auto mv = [&](void *p, size_t bytes) {
      const cudaError_t e = cudaMemcpyAsync(to_save ? save + off : p, to_save ? p : save + off,
                                            bytes, cudaMemcpyDeviceToDevice, c->stream);
      off += bytes;
      return e == cudaSuccess;
    };
    bool ok = true;
    for (int k = 0; k < 3; ++k) ok = ok && mv(c->bits[k], wbytes);
    for (int k = 0; k < 3; ++k) ok = ok && mv(c->counts[k], cbytes);
    ok = ok && mv(c->hint, hbytes);
    ok = ok && mv(c->st, sizeof(DevState));
    return ok ? GCVT_OK : GCVT_ERR_CUDA;
  };
  int sms = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  gcvt_tuning best = {0, c->hint_slack, c->jfa_halo, 1e30f, 1e30f, c->cell_mode};
  const int slack[3] = {1, 2, 3};
  const int keep_grid = c->cell_grid, keep_slack = c->hint_slack, keep_mode = c->cell_mode;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    rc = GCVT_ERR_CUDA;
  // the covering bound and counts of the current sites, then the snapshot
  if (!rc) rc = start_level(c, n, 0, 0x7fffffff, 0x7fffffff);
  if (!rc) rc = pull_state(c);
  if (!rc) rc = copy_state(true);
  // the base of the search: 16 iterations on, where most of a run's
  // iterations look like (the first few after a load are heavier)
  if (!rc) {
    const LevelBufs lb = level_bufs(c, n, 0);
    for (int it = 0; it < 16 && !rc; ++it)
      if (launch_list(lb, 1, c->stream) != cudaSuccess ||
          launch_cells(lb, 0, nullptr, c->stream) != cudaSuccess)
        rc = GCVT_ERR_CUDA;
  }
  if (!rc) rc = pull_state(c);
  slot = total;
  if (!rc) rc = copy_state(true);
  // Lloyd grids: 16, 24 and 32 blocks (warps) per SM, and the block counts
  // that make the 32-site groups an exact number of waves (k groups per
  // warp: no half-empty last wave)
  int per_sm[12] = {16, 24, 32}, ngrid = 3;
  const int groups = (c->st_host->snap_count + 31) / 32;
  for (int k = 1; k <= 8 && sms > 0; ++k) {
    const int b = (groups + k * sms - 1) / (k * sms);
    bool seen = b < 12 || b > 32;
    for (int q = 0; q < ngrid; ++q) seen = seen || per_sm[q] == b;
    if (!seen && ngrid < 12) per_sm[ngrid++] = b;
  }
  // cells one site per lane, and (few sites, no learned-step state) one per warp
  const int modes[2] = {1, 2};
  const int nmode = (c->sites <= kWarpSites && !c->learning) ? 2 : 1;
  // each: mode x grid x hint slack, three iterations from the same base
  for (int mi = 0; mi < nmode && !rc; ++mi)
  for (int gi = 0; gi < ngrid && !rc; ++gi)
    for (int si = 0; si < 3 && !rc; ++si) {
      if ((rc = copy_state(false))) break;
      c->st_host->hint_slack = slack[si];
      if ((rc = push_state(c))) break;
      c->cell_mode = modes[mi];
      const LevelBufs lb = level_bufs(c, n, 0);
      const int grid = per_sm[gi] * sms;
      float ms = 0.f;
      for (int it = 0; it < 4 && !rc; ++it) {
        if (it == 1 && cudaEventRecord(e0, c->stream) != cudaSuccess) rc = GCVT_ERR_CUDA;
        if (launch_list(lb, 1, c->stream) != cudaSuccess ||
            launch_cells(lb, 0, nullptr, c->stream, grid) != cudaSuccess)
          rc = GCVT_ERR_CUDA;
      }
      if (!rc && (cudaEventRecord(e1, c->stream) != cudaSuccess ||
                  cudaEventSynchronize(e1) != cudaSuccess ||
                  cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = GCVT_ERR_CUDA;
      if (!rc && ms / 3 < best.lloyd_ms) {
        best.lloyd_ms = ms / 3;
        best.cell_blocks_per_sm = per_sm[gi];
        best.hint_slack = slack[si];
        best.cell_mode = modes[mi];
      }
    }
  c->cell_mode = keep_mode;
  // jump flooding: fusion depth
  if (!rc && !c->jfa &&
      cudaMalloc(reinterpret_cast<void **>(&c->jfa),
                 2 * (size_t)c->n_max * c->n_max * sizeof(uint32_t) + 64) != cudaSuccess)
    rc = GCVT_ERR_ALLOC;
  slot = 0;
  if (!rc) rc = copy_state(false);
  const int halos[4] = {0, 8, 16, 32};
  for (int hi = 0; hi < 4 && !rc; ++hi) {
    uint32_t *ja = c->jfa, *jb = c->jfa + (size_t)c->n_max * c->n_max, *res = nullptr;
    float ms = 0.f;
    for (int it = 0; it < 3 && !rc; ++it) {
      float one = 0.f;
      if (launch_jfa_seed(c->bits[saved_host.cur], n, ja, c->stream) != cudaSuccess ||
          cudaEventRecord(e0, c->stream) != cudaSuccess ||
          launch_jfa(ja, jb, n, c->err, &res, c->stream, halos[hi]) != cudaSuccess ||
          cudaEventRecord(e1, c->stream) != cudaSuccess ||
          cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&one, e0, e1) != cudaSuccess)
        rc = GCVT_ERR_CUDA;
      if (it) ms += one;  // the first run warms up
    }
    if (!rc && ms / 2 < best.jfa_ms) {
      best.jfa_ms = ms / 2;
      best.jfa_tail_halo = halos[hi];
    }
  }
  // back to the state before the search
  if (!rc) rc = copy_state(false);
  if (!rc) {
    *c->st_host = saved_host;
    rc = push_state(c);
  }
  if (!rc) CK(cudaStreamSynchronize(c->stream));
  c->cover_valid = saved_valid;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(save);
  if (rc) {
    c->cell_grid = keep_grid;
    c->hint_slack = keep_slack;
    c->cell_mode = keep_mode;
    return rc;
  }
  rc = gcvt_ctx_set_tuning(c, &best);
  if (!rc && out) *out = best;
  return rc;
}

int gcvt_mlp_param_count(void) { return mlp_param_count(); }

int gcvt_ctx_learning(gcvt_ctx *c, int enable, int track_ids) {
  if (!c) return GCVT_ERR_ARGUMENT;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return GCVT_ERR_CUDA;
  for (int k = 0; k < 3; ++k) {
    cudaFree(c->hist[k]);
    cudaFree(c->ids[k]);
    c->hist[k] = nullptr;
    c->ids[k] = nullptr;
  }
  c->learning = c->track_ids = 0;
  if (c->chunk_exec) {  // captured launches hold the old buffer pointers
    cudaGraphExecDestroy(c->chunk_exec);
    c->chunk_exec = nullptr;
  }
  c->cover_valid = 0;  // the next level start sets histories (and ids) up
  if (!enable) return GCVT_OK;
  const size_t nn = (size_t)c->n_max * c->n_max;
  bool ok = true;
  for (int k = 0; k < 3 && ok; ++k)
    ok = cudaMalloc(reinterpret_cast<void **>(&c->hist[k]), nn * sizeof(uint64_t)) == cudaSuccess;
  for (int k = 0; k < 3 && ok && track_ids; ++k)
    ok = cudaMalloc(reinterpret_cast<void **>(&c->ids[k]), nn * sizeof(int)) == cudaSuccess;
  if (ok && !c->mlp_bf)
    ok = cudaMalloc(reinterpret_cast<void **>(&c->mlp_bf), mlp_param_count() * sizeof(float)) ==
         cudaSuccess;
  if (ok && !c->gsave)
    ok = cudaMalloc(reinterpret_cast<void **>(&c->gsave), sizeof(DevState)) == cudaSuccess;
  if (ok && !c->desc)
    ok = cudaMalloc(reinterpret_cast<void **>(&c->desc), sizeof(LevelBufs)) == cudaSuccess;
  if (!ok) {
    gcvt_ctx_learning(c, 0, 0);
    return GCVT_ERR_ALLOC;
  }
  c->learning = 1;
  c->track_ids = track_ids ? 1 : 0;
  return GCVT_OK;
}

}  // extern "C"

namespace {
// Feature and prediction buffers for the current site count.
int ensure_feat(gcvt_ctx *c) {
  const size_t need = (size_t)(c->sites > 0 ? c->sites : 1);
  if (c->feat_cap >= need) return GCVT_OK;
  cudaFree(c->feat);
  cudaFree(c->pred);
  cudaFree(c->jaux);
  c->feat = c->pred = nullptr;
  c->jaux = nullptr;
  c->feat_cap = 0;
  if (c->chunk_exec) {
    cudaGraphExecDestroy(c->chunk_exec);
    c->chunk_exec = nullptr;
  }
  if (cudaMalloc(reinterpret_cast<void **>(&c->feat), need * 10 * sizeof(float)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&c->pred), need * 2 * sizeof(float)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&c->jaux), need * sizeof(uint32_t)) != cudaSuccess)
    return GCVT_ERR_ALLOC;
  CK(cudaMemsetAsync(c->feat, 0, need * 10 * sizeof(float), c->stream));
  c->feat_cap = need;
  return GCVT_OK;
}

// One learned step (two Lloyd iterations when the jump stands, one when it
// does not): the plain iteration from the current sites with their features,
// the MLP, the jumped sites, their iteration (which judges the jump), and the
// gate's resolution.  Every launch reads the device state, so a level that
// has stopped makes them all no-ops.
int enqueue_jump(gcvt_ctx *c) {
  const int n = c->n;
  const LevelBufs b = level_bufs(c, n, 0);
  CK(launch_list(b, 1, c->stream));
  CK(launch_cells(b, 4, nullptr, c->stream, c->cell_grid));
  if (c->mlp_tensor_cores)
    CK(launch_mlp_tc(c->feat, &c->st->snap_count, c->mlp_bf, c->pred, c->err, c->stream));
  else
    CK(launch_mlp_infer(c->feat, &c->st->snap_count, c->mlp_bf, c->pred, 4 * 152, c->stream));
  CK(launch_apply(c->desc, 1, c->stream));
  CK(launch_gate_switch(c->desc, 1, c->stream));
  CK(launch_list(b, 1, c->stream));
  CK(launch_cells(b, 5, nullptr, c->stream, c->cell_grid));
  CK(launch_gate_resolve(c->desc, 1, c->stream));
  return GCVT_OK;
}
}  // namespace

extern "C" {

int gcvt_ctx_set_mlp(gcvt_ctx *c, const float *params, int count) {
  if (!c || !params || count != mlp_param_count()) return GCVT_ERR_ARGUMENT;
  if (!c->learning) return GCVT_ERR_STATE;
  float *tmp = nullptr;
  if (cudaMalloc(reinterpret_cast<void **>(&tmp), count * sizeof(float)) != cudaSuccess)
    return GCVT_ERR_ALLOC;
  int rc = GCVT_OK;
  if (cudaMemcpyAsync(tmp, params, count * sizeof(float), cudaMemcpyHostToDevice, c->stream) !=
          cudaSuccess ||
      launch_round_params(tmp, c->mlp_bf, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    rc = GCVT_ERR_CUDA;
  cudaFree(tmp);
  if (!rc) c->have_mlp = 1;
  return rc;
}

int gcvt_ctx_features(gcvt_ctx *c, float *feat, int *ids, int *xy, int capacity, int *count) {
  if (!c || !count || capacity < 0) return GCVT_ERR_ARGUMENT;
  if (!c->loaded || !c->learning) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  if (c->cur_n != c->n) return GCVT_ERR_STATE;
  int rc = ensure_feat(c);
  if (rc) return rc;
  if ((rc = start_level(c, c->n, 0, 1, 0x7fffffff))) return rc;  // level set up, state kept
  const LevelBufs b = level_bufs(c, c->n, 0);
  int *dids = nullptr, *dxy = nullptr;
  const size_t cap = c->feat_cap;
  if (cudaMalloc(reinterpret_cast<void **>(&dids), cap * sizeof(int)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&dxy), cap * 2 * sizeof(int)) != cudaSuccess) {
    cudaFree(dids);
    return GCVT_ERR_ALLOC;
  }
  int total = 0;
  rc = GCVT_OK;
  if (launch_list(b, 0, c->stream) != cudaSuccess ||
      launch_cells(b, 2, nullptr, c->stream, c->cell_grid) != cudaSuccess ||
      launch_features(b, dids, dxy, 4 * 152, c->stream) != cudaSuccess ||
      cudaMemcpyAsync(&total, &c->st->snap_count, sizeof(int), cudaMemcpyDeviceToHost,
                      c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    rc = GCVT_ERR_CUDA;
  const size_t w = (size_t)(total < capacity ? total : capacity);
  if (!rc && w) {
    if ((feat && cudaMemcpy(feat, c->feat, w * 10 * sizeof(float), cudaMemcpyDeviceToHost) !=
                     cudaSuccess) ||
        (ids && cudaMemcpy(ids, dids, w * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (xy && cudaMemcpy(xy, dxy, w * 2 * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
      rc = GCVT_ERR_CUDA;
  }
  cudaFree(dids);
  cudaFree(dxy);
  *count = total;
  return rc;
}

int gcvt_ctx_iterate_learned(gcvt_ctx *c, int iterations, int jump_every, int *tried, int *kept) {
  if (!c || iterations < 0 || jump_every < 1) return GCVT_ERR_ARGUMENT;
  if (!c->loaded || !c->learning || !c->have_mlp) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  if (c->cur_n != c->n) return GCVT_ERR_STATE;
  if (iterations == 0) return GCVT_OK;
  int rc = ensure_feat(c);
  if (rc) return rc;
  if ((rc = start_level(c, c->n, 0, iterations, 0x7fffffff))) return rc;
  const LevelBufs b = level_bufs(c, c->n, 0);
  CK(cudaMemcpyAsync(c->desc, &b, sizeof(LevelBufs), cudaMemcpyHostToDevice, c->stream));
  if ((rc = pull_state(c))) return rc;
  const int tried0 = c->st_host->gate_tried, kept0 = c->st_host->gate_kept;
  // rounds of (jump_every - 1) plain iterations and one learned step until
  // the device schedule has run `iterations` iterations (or met the target
  // energy); the state is read back every ten or more iterations
  const int per_poll = (kChunk + jump_every - 1) / jump_every;
  for (;;) {
    for (int r = 0; r < per_poll; ++r) {
      for (int i = 0; i + 1 < jump_every; ++i) {
        CK(launch_list(b, 1, c->stream));
        CK(launch_cells(b, 0, nullptr, c->stream, c->cell_grid));
      }
      if ((rc = enqueue_jump(c))) return rc;
    }
    if ((rc = pull_state(c))) return rc;
    if (c->st_host->stopped) break;
  }
  if (tried) *tried = c->st_host->gate_tried - tried0;
  if (kept) *kept = c->st_host->gate_kept - kept0;
  return GCVT_OK;
}

int gcvt_ctx_set_target_energy(gcvt_ctx *c, double target) {
  if (!c || !(target >= 0.0)) return GCVT_ERR_ARGUMENT;
  c->target_energy = target;
  return GCVT_OK;
}

int gcvt_mlp_forward(const float *params, const float *feat, int count, float *out,
                     int tensor_cores) {
  if (!params || (count > 0 && (!feat || !out)) || count < 0) return GCVT_ERR_ARGUMENT;
  if (count == 0) return GCVT_OK;
  const int np = mlp_param_count();
  float *d = nullptr;
  const size_t floats = (size_t)2 * np + (size_t)count * 12 + 2;
  if (cudaMalloc(reinterpret_cast<void **>(&d), floats * sizeof(float)) != cudaSuccess)
    return GCVT_ERR_ALLOC;
  float *master = d, *pbf = d + np, *df = d + 2 * np, *dout = df + (size_t)count * 10;
  int *dcount = reinterpret_cast<int *>(dout + (size_t)count * 2), *derr = dcount + 1;
  int rc = GCVT_OK, herr = 0;
  if (cudaMemcpy(master, params, np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(df, feat, (size_t)count * 10 * sizeof(float), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(dcount, &count, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(derr, 0, sizeof(int)) != cudaSuccess ||
      launch_round_params(master, pbf, nullptr) != cudaSuccess ||
      (tensor_cores ? launch_mlp_tc(df, dcount, pbf, dout, derr, nullptr)
                    : launch_mlp_infer(df, dcount, pbf, dout, 4 * 152, nullptr)) != cudaSuccess ||
      cudaMemcpy(out, dout, (size_t)count * 2 * sizeof(float), cudaMemcpyDeviceToHost) !=
          cudaSuccess ||
      cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = GCVT_ERR_CUDA;
  if (herr) rc = GCVT_ERR_CUDA;
  cudaFree(d);
  return rc;
}

int gcvt_mlp_train(const float *samples, long long count, float *params, int steps, int batch,
                   float lr, unsigned long long seed, float *loss) {
  if (!samples || !params || count < 1 || steps < 1 || batch < 1) return GCVT_ERR_ARGUMENT;
  if (mlp_configure() != cudaSuccess) return GCVT_ERR_CUDA;
  const int np = mlp_param_count();
  float *ds = nullptr, *dp = nullptr;
  cudaStream_t s = nullptr;
  if (cudaMalloc(reinterpret_cast<void **>(&ds), (size_t)count * 12 * sizeof(float)) !=
          cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&dp), (size_t)(5 * np + steps) * sizeof(float)) !=
          cudaSuccess) {
    cudaFree(ds);
    return GCVT_ERR_ALLOC;
  }
  // master, grad, m, v, bf copy, then one loss per step
  float *master = dp, *grad = dp + np, *m = dp + 2 * np, *v = dp + 3 * np, *pbf = dp + 4 * np;
  float *dloss = dp + 5 * np;
  int rc = GCVT_OK;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMemcpyAsync(ds, samples, (size_t)count * 12 * sizeof(float), cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(master, params, np * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(grad, 0, (size_t)(4 * np + steps) * sizeof(float), s) != cudaSuccess)
    rc = GCVT_ERR_CUDA;
  for (int st = 0; st < steps && !rc; ++st)
    if (launch_mlp_train_step(ds, count, master, grad, m, v, pbf, dloss + st, batch, seed, st, lr,
                              s) != cudaSuccess)
      rc = GCVT_ERR_CUDA;
  if (!rc && (cudaMemcpyAsync(params, master, np * sizeof(float), cudaMemcpyDeviceToHost, s) !=
                  cudaSuccess ||
              (loss && cudaMemcpyAsync(loss, dloss, steps * sizeof(float), cudaMemcpyDeviceToHost,
                                       s) != cudaSuccess) ||
              cudaStreamSynchronize(s) != cudaSuccess))
    rc = GCVT_ERR_CUDA;
  if (s) cudaStreamDestroy(s);
  cudaFree(ds);
  cudaFree(dp);
  return rc;
}

int gcvt_mlp_gradient(const float *samples, long long count, const float *params, int batch,
                      unsigned long long seed, int step, float *grad, float *loss) {
  if (!samples || !params || !grad || count < 1 || batch < 1 || step < 0)
    return GCVT_ERR_ARGUMENT;
  if (mlp_configure() != cudaSuccess) return GCVT_ERR_CUDA;
  const int np = mlp_param_count();
  float *ds = nullptr, *dp = nullptr;
  cudaStream_t s = nullptr;
  if (cudaMalloc(reinterpret_cast<void **>(&ds), (size_t)count * 12 * sizeof(float)) !=
          cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&dp), (size_t)(2 * np + 1) * sizeof(float)) !=
          cudaSuccess) {
    cudaFree(ds);
    return GCVT_ERR_ALLOC;
  }
  float *master = dp, *dgrad = dp + np, *dloss = dp + 2 * np;
  int rc = GCVT_OK;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMemcpyAsync(ds, samples, (size_t)count * 12 * sizeof(float), cudaMemcpyHostToDevice,
                      s) != cudaSuccess ||
      cudaMemcpyAsync(master, params, np * sizeof(float), cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemsetAsync(dgrad, 0, (size_t)(np + 1) * sizeof(float), s) != cudaSuccess ||
      launch_mlp_grad(ds, count, master, dgrad, dloss, batch, seed, step, s) != cudaSuccess ||
      cudaMemcpyAsync(grad, dgrad, np * sizeof(float), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      (loss && cudaMemcpyAsync(loss, dloss, sizeof(float), cudaMemcpyDeviceToHost, s) !=
                   cudaSuccess) ||
      cudaStreamSynchronize(s) != cudaSuccess)
    rc = GCVT_ERR_CUDA;
  if (s) cudaStreamDestroy(s);
  cudaFree(ds);
  cudaFree(dp);
  return rc;
}

int gcvt_ctx_info(gcvt_ctx *c, gcvt_run_info *info) {
  if (!c) return GCVT_ERR_ARGUMENT;
  if (!info) return GCVT_OK;
  int rc = pull_state(c);
  if (rc) return rc;
  info->iterations = c->st_host->iter;
  info->levels = c->last_levels;
  info->omega = c->st_host->omega;
  info->energy = c->st_host->energy;
  info->sampled_energy = c->st_host->sampled;
  return GCVT_OK;
}

// Mean device time of (one Lloyd iteration: site list + cells, one labelling
// pass, one jump-flooding labelling) over `iterations` iterations at full
// resolution, each bracketed by events on the context's stream.  The sites
// move as in gcvt_ctx_iterate.
int gcvt_ctx_time_kernels(gcvt_ctx *c, int iterations, float *ms3) {
  if (!c || !ms3 || iterations < 1) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  if (c->cur_n != c->n) return GCVT_ERR_STATE;
  int window = 0;
  int rc = initial_window(c, 0, &window);
  if (rc) return rc;
  if ((rc = pull_state(c))) return rc;
  DevState &h = *c->st_host;
  h.level = 0;
  h.stopped = 0;
  h.level_iters = 0;
  h.use_stop_rule = 0;
  h.fixed_iters = 0x7fffffff;
  h.window = window;
  h.hint_slack = c->hint_slack;
  h.energy_scale = 1.0 / ((double)c->n * (double)c->n);
  if ((rc = push_state(c))) return rc;
  if ((rc = ensure_cover(c, c->n, 0))) return rc;
  cudaEvent_t ev[3] = {};
  for (int i = 0; i < 3; ++i)
    if (cudaEventCreate(&ev[i]) != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaEventDestroy(ev[j]);
      return GCVT_ERR_CUDA;
    }
  float acc[2] = {0.f, 0.f};
  const LevelBufs b = level_bufs(c, c->n, 0);
  int status = GCVT_OK;
  for (int it = 0; it < iterations && status == GCVT_OK; ++it) {
    float ms0 = 0.f, ms1 = 0.f;
    if (cudaEventRecord(ev[0], c->stream) != cudaSuccess ||
        launch_list(b, 1, c->stream) != cudaSuccess ||
        launch_cells(b, 0, nullptr, c->stream, c->cell_grid) != cudaSuccess ||
        cudaEventRecord(ev[1], c->stream) != cudaSuccess ||
        launch_summary(b, 0, c->stream) != cudaSuccess ||
        launch_rows(b, 0, c->stream) != cudaSuccess ||
        cudaEventRecord(ev[2], c->stream) != cudaSuccess ||
        cudaEventSynchronize(ev[2]) != cudaSuccess ||
        cudaEventElapsedTime(&ms0, ev[0], ev[1]) != cudaSuccess ||
        cudaEventElapsedTime(&ms1, ev[1], ev[2]) != cudaSuccess)
      status = GCVT_ERR_CUDA;
    acc[0] += ms0;
    acc[1] += ms1;
  }
  // jump flooding of the sites now held, kernels only
  float acc2 = 0.f;
  const size_t nmax2 = (size_t)c->n_max * c->n_max;
  if (status == GCVT_OK && !c->jfa &&
      cudaMalloc(reinterpret_cast<void **>(&c->jfa), 2 * nmax2 * sizeof(uint32_t) + 64) !=
          cudaSuccess)
    status = GCVT_ERR_ALLOC;
  if (status == GCVT_OK && (status = pull_state(c)) == GCVT_OK) {
    uint32_t *ja = c->jfa, *jb = c->jfa + nmax2, *res = nullptr;
    for (int it = 0; it < iterations && status == GCVT_OK; ++it) {
      float ms = 0.f;
      if (launch_jfa_seed(c->bits[c->st_host->cur], c->n, ja, c->stream) != cudaSuccess ||
          cudaEventRecord(ev[0], c->stream) != cudaSuccess ||
          launch_jfa(ja, jb, c->n, c->err, &res, c->stream, c->jfa_halo) != cudaSuccess ||
          cudaEventRecord(ev[1], c->stream) != cudaSuccess ||
          cudaEventSynchronize(ev[1]) != cudaSuccess ||
          cudaEventElapsedTime(&ms, ev[0], ev[1]) != cudaSuccess)
        status = GCVT_ERR_CUDA;
      acc2 += ms;
    }
  }
  for (int i = 0; i < 3; ++i) cudaEventDestroy(ev[i]);
  if (status) return status;
  ms3[0] = acc[0] / iterations;
  ms3[1] = acc[1] / iterations;
  ms3[2] = acc2 / iterations;
  return GCVT_OK;
}

// One context per device serves the one-call forms; like the reference's
// globals (gcvt.cu:50-62) it is shared, so calls are serialised.
static std::mutex g_mutex;
static gcvt_ctx *g_ctx[64] = {};

static int shared_ctx(int n, gcvt_ctx **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GCVT_ERR_CUDA;
  gcvt_ctx *&c = g_ctx[dev];
  if (c && c->n_max < n) {
    gcvt_ctx_destroy(c);
    c = nullptr;
  }
  if (!c) {
    int rc = gcvt_ctx_create(n, &c);
    if (rc) return rc;
  }
  *out = c;
  return GCVT_OK;
}

int gcvt_compute(int16_t *voronoi, const float *density, const uint8_t *mask, int size,
                 int depth, int max_iter) {
  if (!voronoi || !density || !mask || depth < 1) return GCVT_ERR_ARGUMENT;
  if (!valid_n(size) || !pow2(size)) return GCVT_ERR_SIZE;
  std::lock_guard<std::mutex> lock(g_mutex);
  gcvt_ctx *c = nullptr;
  int rc = shared_ctx(size, &c);
  if (rc) return rc;
  if ((rc = gcvt_ctx_load(c, size, voronoi, density, mask, GCVT_MEM_HOST))) return rc;
  if ((rc = gcvt_ctx_run(c, depth, max_iter, nullptr))) return rc;
  return gcvt_ctx_label(c, voronoi, GCVT_MEM_HOST);
}

int gcvt_label_grid(const int16_t *sites, int16_t *labels, int n, int mem) {
  if (!sites || !labels) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!valid_n(n)) return GCVT_ERR_SIZE;
  std::lock_guard<std::mutex> lock(g_mutex);
  gcvt_ctx *c = nullptr;
  int rc = shared_ctx(n, &c);
  if (rc) return rc;
  if ((rc = load_sites(c, n, sites, mem))) return rc;
  return gcvt_ctx_label(c, labels, mem);
}

// ---- batches: many contexts, one launch pair per iteration ----------------

}  // extern "C"

struct gcvt_batch {
  int device = 0;
  std::vector<gcvt_ctx *> charts;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  LevelBufs *descs = nullptr;  // device: one LevelBufs per chart
  unsigned *lofs = nullptr;    // device: first list block of each chart, and the total
  unsigned *gofs = nullptr;    // device: first 32-site group of each chart, and the total
  unsigned *done = nullptr;    // device: list blocks finished
  unsigned *ticket = nullptr;  // device: next group
  unsigned nblocks = 0;
  std::vector<LevelBufs> host_descs;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev = nullptr;    // orders the batch's stream with its members' streams
  // learned steps over the batch: every chart's list slots in one feature /
  // prediction / window array (chart i from slot_ofs[i]), one MLP launch
  float *mlp_bf = nullptr;
  float *feat = nullptr, *pred = nullptr;
  uint32_t *jaux = nullptr;
  int *mlp_count = nullptr;    // device: slots the MLP runs over; [1]: its error flag
  size_t feat_cap = 0;
  std::vector<size_t> slot_ofs;
  bool learned = false;        // the descriptors point into the arrays above
};

namespace {

// Level start of every chart on the batch's stream, then the charts' buffer
// descriptors to the device.
int batch_start(gcvt_batch *b, int fixed, int max_iter) {
  std::vector<unsigned> lofs(b->charts.size() + 1, 0);
  for (size_t i = 0; i < b->charts.size(); ++i) {
    gcvt_ctx *c = b->charts[i];
    if (!c->loaded) return GCVT_ERR_STATE;
    if (c->input_err) return GCVT_ERR_INPUT;
    if (c->cur_n != c->n) return GCVT_ERR_STATE;
    // work already queued on the member's own stream comes first
    CK(cudaEventRecord(b->ev, c->stream));
    CK(cudaStreamWaitEvent(b->stream, b->ev, 0));
    cudaStream_t keep = c->stream;
    c->stream = b->stream;
    const int rc = start_level(c, c->n, 0, fixed, max_iter);
    c->stream = keep;
    if (rc) return rc;
    b->host_descs[i] = level_bufs(c, c->n, 0);
    if (b->learned) {
      b->host_descs[i].feat = b->feat + b->slot_ofs[i] * 10;
      b->host_descs[i].pred = b->pred + b->slot_ofs[i] * 2;
      b->host_descs[i].jaux = b->jaux + b->slot_ofs[i];
    }
    lofs[i + 1] = lofs[i] + (unsigned)list_blocks(c->n);
  }
  if (lofs.back() != b->nblocks && b->exec) {  // the captured grid no longer fits
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  b->nblocks = lofs.back();
  CK(cudaMemcpyAsync(b->descs, b->host_descs.data(), b->host_descs.size() * sizeof(LevelBufs),
                     cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(b->lofs, lofs.data(), lofs.size() * sizeof(unsigned),
                     cudaMemcpyHostToDevice, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return GCVT_OK;
}

// The members' streams wait for the batch's work.
int batch_finish(gcvt_batch *b) {
  CK(cudaEventRecord(b->ev, b->stream));
  for (gcvt_ctx *c : b->charts) CK(cudaStreamWaitEvent(c->stream, b->ev, 0));
  return GCVT_OK;
}

// Feature, prediction and window slots for every member's sites (their
// counts at load; merges only lower them).
int batch_feat(gcvt_batch *b) {
  b->slot_ofs.assign(b->charts.size() + 1, 0);
  for (size_t i = 0; i < b->charts.size(); ++i)
    b->slot_ofs[i + 1] = b->slot_ofs[i] + (size_t)(b->charts[i]->sites > 0 ? b->charts[i]->sites : 1);
  const size_t need = b->slot_ofs.back();
  if (need > b->feat_cap) {
    cudaFree(b->feat);
    cudaFree(b->pred);
    cudaFree(b->jaux);
    b->feat = b->pred = nullptr;
    b->jaux = nullptr;
    b->feat_cap = 0;
    if (cudaMalloc(reinterpret_cast<void **>(&b->feat), need * 10 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void **>(&b->pred), need * 2 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void **>(&b->jaux), need * sizeof(uint32_t)) != cudaSuccess)
      return GCVT_ERR_ALLOC;
    CK(cudaMemsetAsync(b->feat, 0, need * 10 * sizeof(float), b->stream));
    b->feat_cap = need;
  }
  const int cnt[2] = {(int)need, 0};
  CK(cudaMemcpyAsync(b->mlp_count, cnt, sizeof(cnt), cudaMemcpyHostToDevice, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return GCVT_OK;
}

// One learned step of every member (see enqueue_jump): the MLP runs once over
// all charts' slots.
int batch_jump(gcvt_batch *b) {
  const int nc = (int)b->charts.size();
  CK(launch_list_batch(b->descs, nc, b->lofs, b->nblocks, b->gofs, b->done, b->ticket, b->stream));
  CK(launch_cells_batch(b->descs, nc, b->gofs, b->ticket, b->stream, 4));
  CK(launch_mlp_tc(b->feat, b->mlp_count, b->mlp_bf, b->pred, b->mlp_count + 1, b->stream));
  CK(launch_apply(b->descs, nc, b->stream));
  CK(launch_gate_switch(b->descs, nc, b->stream));
  CK(launch_list_batch(b->descs, nc, b->lofs, b->nblocks, b->gofs, b->done, b->ticket, b->stream));
  CK(launch_cells_batch(b->descs, nc, b->gofs, b->ticket, b->stream, 5));
  CK(launch_gate_resolve(b->descs, nc, b->stream));
  return GCVT_OK;
}

int batch_chunk(gcvt_batch *b) {
  const int nc = (int)b->charts.size();
  if (!b->exec) {
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      for (int i = 0; i < kChunk; ++i) {
        CK(launch_list_batch(b->descs, nc, b->lofs, b->nblocks, b->gofs, b->done, b->ticket,
                             b->stream));
        CK(launch_cells_batch(b->descs, nc, b->gofs, b->ticket, b->stream));
      }
      return GCVT_OK;
    }
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < kChunk && le == cudaSuccess; ++i) {
      le = launch_list_batch(b->descs, nc, b->lofs, b->nblocks, b->gofs, b->done, b->ticket,
                             b->stream);
      if (le == cudaSuccess) le = launch_cells_batch(b->descs, nc, b->gofs, b->ticket, b->stream);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return GCVT_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      b->exec = nullptr;
      return GCVT_ERR_CUDA;
    }
  }
  CK(cudaGraphLaunch(b->exec, b->stream));
  return GCVT_OK;
}

}  // namespace

extern "C" {

int gcvt_batch_create(int count, gcvt_ctx *const *charts, gcvt_batch **out) {
  if (!out || count < 1 || !charts) return GCVT_ERR_ARGUMENT;
  *out = nullptr;
  gcvt_batch *b = new (std::nothrow) gcvt_batch();
  if (!b) return GCVT_ERR_ALLOC;
  auto fail = [&](int code) {
    gcvt_batch_destroy(b);
    return code;
  };
  if (cudaGetDevice(&b->device) != cudaSuccess) return fail(GCVT_ERR_CUDA);
  for (int i = 0; i < count; ++i) {
    gcvt_ctx *c = charts[i];
    if (!c) return fail(GCVT_ERR_ARGUMENT);
    if (c->device != b->device) return fail(GCVT_ERR_ARGUMENT);
    for (gcvt_ctx *d : b->charts)
      if (d == c) return fail(GCVT_ERR_ARGUMENT);  // a context appears once
    b->charts.push_back(c);
  }
  b->host_descs.resize(count);
  if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(GCVT_ERR_CUDA);
  b->stream = b->own_stream;
  bool ok = cudaMalloc(reinterpret_cast<void **>(&b->descs), count * sizeof(LevelBufs)) == cudaSuccess;
  ok = ok && cudaMalloc(reinterpret_cast<void **>(&b->lofs), (count + 1) * sizeof(unsigned)) == cudaSuccess;
  ok = ok && cudaMalloc(reinterpret_cast<void **>(&b->gofs), (count + 1) * sizeof(unsigned)) == cudaSuccess;
  ok = ok && cudaMalloc(reinterpret_cast<void **>(&b->done), 2 * sizeof(unsigned)) == cudaSuccess;
  if (!ok) return fail(GCVT_ERR_ALLOC);
  b->ticket = b->done + 1;
  if (cudaMemset(b->done, 0, 2 * sizeof(unsigned)) != cudaSuccess) return fail(GCVT_ERR_CUDA);
  if (cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) != cudaSuccess)
    return fail(GCVT_ERR_CUDA);
  *out = b;
  return GCVT_OK;
}

int gcvt_batch_destroy(gcvt_batch *b) {
  if (!b) return GCVT_ERR_ARGUMENT;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  cudaFree(b->descs);
  cudaFree(b->lofs);
  cudaFree(b->gofs);
  cudaFree(b->done);
  cudaFree(b->mlp_bf);
  cudaFree(b->feat);
  cudaFree(b->pred);
  cudaFree(b->jaux);
  cudaFree(b->mlp_count);
  if (b->ev) cudaEventDestroy(b->ev);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return GCVT_OK;
}

int gcvt_batch_set_stream(gcvt_batch *b, void *stream) {
  if (!b) return GCVT_ERR_ARGUMENT;
  b->stream = stream ? (cudaStream_t)stream : b->own_stream;
  return GCVT_OK;
}

int gcvt_batch_set_mlp(gcvt_batch *b, const float *params, int count) {
  if (!b || !params || count != mlp_param_count()) return GCVT_ERR_ARGUMENT;
  if (!b->mlp_bf &&
      (cudaMalloc(reinterpret_cast<void **>(&b->mlp_bf), count * sizeof(float)) != cudaSuccess ||
       cudaMalloc(reinterpret_cast<void **>(&b->mlp_count), 2 * sizeof(int)) != cudaSuccess))
    return GCVT_ERR_ALLOC;
  float *tmp = nullptr;
  if (cudaMalloc(reinterpret_cast<void **>(&tmp), count * sizeof(float)) != cudaSuccess)
    return GCVT_ERR_ALLOC;
  int rc = GCVT_OK;
  if (cudaMemcpyAsync(tmp, params, count * sizeof(float), cudaMemcpyHostToDevice, b->stream) !=
          cudaSuccess ||
      launch_round_params(tmp, b->mlp_bf, b->stream) != cudaSuccess ||
      cudaMemsetAsync(b->mlp_count, 0, 2 * sizeof(int), b->stream) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    rc = GCVT_ERR_CUDA;
  cudaFree(tmp);
  return rc;
}

int gcvt_batch_iterate_learned(gcvt_batch *b, int iterations, int jump_every, int *tried,
                               int *kept) {
  if (!b || iterations < 0 || jump_every < 1) return GCVT_ERR_ARGUMENT;
  if (!b->mlp_bf) return GCVT_ERR_STATE;
  for (gcvt_ctx *c : b->charts)
    if (!c->learning) return GCVT_ERR_STATE;
  if (iterations == 0) return GCVT_OK;
  int rc = batch_feat(b);
  if (rc) return rc;
  b->learned = true;
  rc = batch_start(b, iterations, 0x7fffffff);
  b->learned = false;
  if (rc) return rc;
  std::vector<int> tried0(b->charts.size()), kept0(b->charts.size());
  auto pull_all = [&](bool *all_stopped) -> int {
    bool all = true;
    for (size_t i = 0; i < b->charts.size(); ++i) {
      gcvt_ctx *c = b->charts[i];
      cudaStream_t keep = c->stream;
      c->stream = b->stream;
      const int r = pull_state(c);
      c->stream = keep;
      if (r) return r;
      all = all && c->st_host->stopped;
    }
    if (all_stopped) *all_stopped = all;
    return GCVT_OK;
  };
  if ((rc = pull_all(nullptr))) return rc;
  for (size_t i = 0; i < b->charts.size(); ++i) {
    tried0[i] = b->charts[i]->st_host->gate_tried;
    kept0[i] = b->charts[i]->st_host->gate_kept;
  }
  const int nc = (int)b->charts.size();
  const int per_poll = (kChunk + jump_every - 1) / jump_every;
  for (;;) {
    for (int r = 0; r < per_poll; ++r) {
      for (int i = 0; i + 1 < jump_every; ++i) {
        CK(launch_list_batch(b->descs, nc, b->lofs, b->nblocks, b->gofs, b->done, b->ticket,
                             b->stream));
        CK(launch_cells_batch(b->descs, nc, b->gofs, b->ticket, b->stream));
      }
      if ((rc = batch_jump(b))) return rc;
    }
    bool all = false;
    if ((rc = pull_all(&all))) return rc;
    if (all) break;
  }
  int err = 0;
  CK(cudaMemcpyAsync(&err, b->mlp_count + 1, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (err) return GCVT_ERR_CUDA;
  int t = 0, k = 0;
  for (size_t i = 0; i < b->charts.size(); ++i) {
    t += b->charts[i]->st_host->gate_tried - tried0[i];
    k += b->charts[i]->st_host->gate_kept - kept0[i];
  }
  if (tried) *tried = t;
  if (kept) *kept = k;
  return batch_finish(b);
}

int gcvt_batch_iterate(gcvt_batch *b, int iterations) {
  if (!b || iterations < 0) return GCVT_ERR_ARGUMENT;
  if (iterations == 0) return GCVT_OK;
  int rc = batch_start(b, iterations, 0x7fffffff);
  if (rc) return rc;
  for (int done = 0; done < iterations; done += kChunk)
    if ((rc = batch_chunk(b))) return rc;
  return batch_finish(b);
}

int gcvt_batch_run(gcvt_batch *b, int max_iter, gcvt_run_info *infos) {
  if (!b) return GCVT_ERR_ARGUMENT;
  int rc = batch_start(b, 0, max_iter);
  if (rc) return rc;
  for (;;) {
    if ((rc = batch_chunk(b))) return rc;
    bool all = true;
    for (gcvt_ctx *c : b->charts) {
      cudaStream_t keep = c->stream;
      c->stream = b->stream;
      rc = pull_state(c);
      c->stream = keep;
      if (rc) return rc;
      all = all && c->st_host->stopped;
    }
    if (all) break;
  }
  if ((rc = batch_finish(b))) return rc;
  for (size_t i = 0; i < b->charts.size(); ++i) {
    b->charts[i]->last_levels = 1;
    if (infos && (rc = gcvt_ctx_info(b->charts[i], infos + i))) return rc;
  }
  return GCVT_OK;
}

}  // extern "C"

// The reference's C++ entry point (gcvt.h:29): same signature and behaviour;
// failures print the reason and exit, as gpuAssert does (gcvt.cu:41-47).
void gCVT(short *Voronoi, float *density_d, bool *mask, int size, int depth, int maxIter) {
  int rc = gcvt_compute(reinterpret_cast<int16_t *>(Voronoi), density_d,
                        reinterpret_cast<const uint8_t *>(mask), size, depth, maxIter);
  if (rc != GCVT_OK) {
    std::fprintf(stderr, "gCVT: %s\n", gcvt_status_string(rc));
    std::exit(rc);
  }
}
