// api.cu -- host side of libgcvt_gb300.so: the context (device buffers
// allocated once), the Lloyd driver of gCVT (gcvt.cu:1087-1156) and the C ABI
// declared in include/gcvt_gb300.h.
//
// One Lloyd iteration is three launches (column summaries, fused row pass,
// update), all reading their buffer roles and the omega / stop state from
// device memory, so ten iterations are captured once as a CUDA graph and
// replayed.  The host reads the state back once per ten iterations, where the
// reference's schedule can end a level (gcvt.cu:1125-1140).
#include "gcvt_internal.cuh"
#include "../../include/gcvt_gb300.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

using namespace cvtgb;

struct gcvt_ctx {
  int device = 0;
  int n_max = 0;
  int n = 0;            // loaded problem size
  int loaded = 0;
  int input_err = 0;    // the loaded grid is malformed at full resolution
  int cur_n = 0;        // size of the level currently held in the bitmaps
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  float *density[8] = {};  // pyramid, [0] = full resolution
  int dens_levels = 0;
  uint8_t *mask = nullptr;
  uint32_t *input = nullptr;  // the loaded site grid, kept for gcvt_ctx_run
  uint32_t *grid = nullptr;   // staging: labels and site dumps
  uint64_t *bits[2] = {};
  int16_t *prev = nullptr, *next = nullptr;
  uint64_t *fixed_bits[8] = {};   // per level
  int *word_rank = nullptr, *group_count = nullptr, *group_offset = nullptr;
  float4 *mhi = nullptr, *mlo = nullptr;
  DevState *st = nullptr;
  DevState *st_host = nullptr;  // pinned mirror
  float *blk_energy = nullptr;    // 2 floats per update block
  int2 *support[8] = {};          // per level: row support of the density
  double *moments = nullptr;    // 4*n_max^2 doubles, allocated on first use
  int *err = nullptr;
  int last_levels = 0;
  // graph of kChunk iterations for one level size
  cudaGraphExec_t chunk_exec = nullptr;
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

LevelBufs level_bufs(gcvt_ctx *c, int n, int level) {
  LevelBufs b;
  b.n = n;
  b.bits[0] = c->bits[0];
  b.bits[1] = c->bits[1];
  b.prev = c->prev;
  b.next = c->next;
  b.density = c->density[level];
  b.fixed = c->mask;
  b.fixed_bits = c->fixed_bits[level];
  b.word_rank = c->word_rank;
  b.group_count = c->group_count;
  b.group_offset = c->group_offset;
  b.mhi = c->mhi;
  b.mlo = c->mlo;
  b.labels = c->grid;
  b.st = c->st;
  b.blk_energy = c->blk_energy;
  b.support = c->support[level];
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

// Enqueue one Lloyd iteration at size n.
int enqueue_iteration(gcvt_ctx *c, int n, int level) {
  LevelBufs b = level_bufs(c, n, level);
  CK(launch_summary(b, 1, c->stream));
  CK(launch_rows(b, 0 /*lloyd*/, 1, c->stream));
  CK(launch_update(b, c->stream));
  return GCVT_OK;
}

// Enqueue kChunk iterations through a CUDA graph captured once per (size,
// level); a stream that cannot be captured (the legacy default stream) gets
// plain launches.
int enqueue_chunk(gcvt_ctx *c, int n, int level) {
  if (c->chunk_exec && (c->chunk_n != n || c->chunk_level != level)) {
    cudaGraphExecDestroy(c->chunk_exec);
    c->chunk_exec = nullptr;
  }
  if (!c->chunk_exec) {
    cudaGraph_t g;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      for (int i = 0; i < kChunk; ++i) {
        int rc = enqueue_iteration(c, n, level);
        if (rc) return rc;
      }
      return GCVT_OK;
    }
    int rc = GCVT_OK;
    for (int i = 0; i < kChunk && rc == GCVT_OK; ++i) rc = enqueue_iteration(c, n, level);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (rc != GCVT_OK) return rc;
    CK(ce);
    ce = cudaGraphInstantiate(&c->chunk_exec, g, 0);
    cudaGraphDestroy(g);
    CK(ce);
    c->chunk_n = n;
    c->chunk_level = level;
  }
  CK(cudaGraphLaunch(c->chunk_exec, c->stream));
  return GCVT_OK;
}

// Bring the bitmaps to size n_new = 2 * cur_n (gcvt.cu:1036-1051).
int zoom_level(gcvt_ctx *c, int n) {
  int rc = pull_state(c);
  if (rc) return rc;
  int p = c->st_host->parity;
  size_t words2 = (size_t)(2 * n / kBand) * (2 * n);
  CK(cudaMemsetAsync(c->bits[p ^ 1], 0, words2 * sizeof(uint64_t), c->stream));
  CK(launch_zoom(c->bits[p], n, c->bits[p ^ 1], c->stream));
  CK(cudaMemsetAsync(c->bits[p], 0, words2 * sizeof(uint64_t), c->stream));
  c->st_host->parity = p ^ 1;
  return push_state(c);
}

// Run one level until the device schedule stops it.  fixed > 0: exactly that
// many iterations without the stop rule.
int run_level(gcvt_ctx *c, int n, int level, int fixed, int max_iter, int poll) {
  int rc = pull_state(c);
  if (rc) return rc;
  DevState &h = *c->st_host;
  h.level = level;
  h.stopped = 0;
  h.level_iters = 0;
  h.use_stop_rule = fixed > 0 ? 0 : 1;
  h.fixed_iters = fixed;
  h.max_iter = max_iter;
  h.energy_scale = std::pow(4.0, level) / ((double)n * (double)n);
  h.done_blocks = 0;
  rc = push_state(c);
  if (rc) return rc;
  c->cur_n = n;
  if (fixed > 0 && !poll) {
    for (int done = 0; done < fixed; done += kChunk) {
      rc = enqueue_chunk(c, n, level);
      if (rc) return rc;
    }
    return GCVT_OK;
  }
  for (;;) {
    rc = enqueue_chunk(c, n, level);
    if (rc) return rc;
    rc = pull_state(c);
    if (rc) return rc;
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

int reset_schedule(gcvt_ctx *c, int parity) {
  DevState &h = *c->st_host;
  std::memset(&h, 0, sizeof(DevState));
  h.parity = parity;
  h.omega = 2.0f;           // gcvt.cu:1108
  h.last_energy = 1e18;     // gcvt.cu:1105
  h.max_iter = 0x7fffffff;
  return push_state(c);
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

int gcvt_version(void) { return 10000; }

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
  c->n_max = n_max;
  const size_t nn = (size_t)n_max * n_max;
  const size_t words = (size_t)(n_max / kBand) * n_max;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(GCVT_ERR_CUDA);
  c->stream = c->own_stream;
  auto dal = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess; };
  bool ok = true;
  c->dens_levels = 0;
  for (int l = 0; l < 8 && ok; ++l) {
    int nl = n_max >> l;
    if (nl < kMinN) break;
    ok &= dal((void **)&c->density[l], (size_t)nl * nl * sizeof(float));
    c->dens_levels = l + 1;
  }
  ok = ok && dal((void **)&c->mask, nn);
  ok = ok && dal((void **)&c->input, nn * sizeof(uint32_t));
  ok = ok && dal((void **)&c->grid, nn * sizeof(uint32_t));
  ok = ok && dal((void **)&c->bits[0], words * sizeof(uint64_t));
  ok = ok && dal((void **)&c->bits[1], words * sizeof(uint64_t));
  ok = ok && dal((void **)&c->prev, words * sizeof(int16_t));
  ok = ok && dal((void **)&c->word_rank, words * sizeof(int));
  ok = ok && dal((void **)&c->group_count, (size_t)(n_max / 32) * sizeof(int));
  ok = ok && dal((void **)&c->group_offset, (size_t)(n_max / 32) * sizeof(int));
  for (int l = 0; l < c->dens_levels && ok; ++l)
    ok &= dal((void **)&c->fixed_bits[l], (size_t)((n_max >> l) / kBand) * (n_max >> l) * sizeof(uint64_t));
  ok = ok && dal((void **)&c->next, words * sizeof(int16_t));
  ok = ok && dal((void **)&c->mhi, nn * sizeof(float4));
  ok = ok && dal((void **)&c->mlo, nn * sizeof(float4));
  ok = ok && dal((void **)&c->st, sizeof(DevState));
  ok = ok && dal((void **)&c->blk_energy, (size_t)update_blocks(n_max) * 2 * sizeof(float));
  for (int l = 0; l < c->dens_levels && ok; ++l)
    ok &= dal((void **)&c->support[l], (size_t)(n_max >> l) * sizeof(int2));
  ok = ok && dal((void **)&c->err, sizeof(int));
  if (!ok) return fail(GCVT_ERR_ALLOC);
  if (cudaMallocHost((void **)&c->st_host, sizeof(DevState)) != cudaSuccess)
    return fail(GCVT_ERR_ALLOC);
  if (cudaMemsetAsync(c->mhi, 0, nn * sizeof(float4), c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->mlo, 0, nn * sizeof(float4), c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->bits[0], 0, words * sizeof(uint64_t), c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->bits[1], 0, words * sizeof(uint64_t), c->stream) != cudaSuccess)
    return fail(GCVT_ERR_CUDA);
  if (reset_schedule(c, 0) != GCVT_OK) return fail(GCVT_ERR_CUDA);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(GCVT_ERR_CUDA);
  *out = c;
  return GCVT_OK;
}

int gcvt_ctx_destroy(gcvt_ctx *c) {
  if (!c) return GCVT_ERR_ARGUMENT;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->chunk_exec) cudaGraphExecDestroy(c->chunk_exec);
  for (int l = 0; l < 8; ++l) cudaFree(c->density[l]);
  cudaFree(c->mask);
  cudaFree(c->input);
  cudaFree(c->grid);
  cudaFree(c->bits[0]);
  cudaFree(c->bits[1]);
  cudaFree(c->prev);
  cudaFree(c->word_rank);
  cudaFree(c->group_count);
  cudaFree(c->group_offset);
  for (int l = 0; l < 8; ++l) cudaFree(c->fixed_bits[l]);
  cudaFree(c->next);
  cudaFree(c->mhi);
  cudaFree(c->mlo);
  cudaFree(c->st);
  cudaFree(c->blk_energy);
  for (int l = 0; l < 8; ++l) cudaFree(c->support[l]);
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

}  // extern "C"

namespace {
// Upload a site grid and build the bitmap (pba2DInitializeInput's site part).
int load_sites(gcvt_ctx *c, int n, const int16_t *voronoi, int mem) {
  const size_t nn = (size_t)n * n;
  const size_t words_max = (size_t)(c->n_max / kBand) * c->n_max;
  int rc;
  c->loaded = 0;
  if ((rc = copy_in(c->input, voronoi, nn * sizeof(uint32_t), mem, c->stream))) return rc;
  CK(cudaMemsetAsync(c->bits[0], 0, words_max * sizeof(uint64_t), c->stream));
  CK(cudaMemsetAsync(c->bits[1], 0, words_max * sizeof(uint64_t), c->stream));
  CK(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
  CK(launch_grid_to_bits(c->input, n, c->bits[0], c->err, c->stream));
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, c->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = reset_schedule(c, 0))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  c->input_err = herr != 0;
  c->n = n;
  c->cur_n = n;
  c->loaded = 1;
  return GCVT_OK;
}
}  // namespace

extern "C" {

int gcvt_ctx_load(gcvt_ctx *c, int n, const int16_t *voronoi, const float *density,
                  const uint8_t *mask, int mem) {
  if (!c || !voronoi || !density) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!valid_n(n) || n > c->n_max) return GCVT_ERR_SIZE;
  const size_t nn = (size_t)n * n;
  int rc;
  c->loaded = 0;
  if ((rc = copy_in(c->density[0], density, nn * sizeof(float), mem, c->stream))) return rc;
  CK(launch_row_support(c->density[0], n, c->support[0], c->stream));
  if (mask) {
    if ((rc = copy_in(c->mask, mask, nn, mem, c->stream))) return rc;
  } else {
    CK(cudaMemsetAsync(c->mask, 0, nn, c->stream));
  }
  CK(launch_fixed_bits(c->mask, n, c->fixed_bits[0], c->stream));
  return load_sites(c, n, voronoi, mem);
}

int gcvt_ctx_label(gcvt_ctx *c, int16_t *labels, int mem) {
  if (!c || !labels) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  const int n = c->cur_n;
  LevelBufs b = level_bufs(c, n, 0);
  CK(launch_summary(b, 0, c->stream));
  CK(launch_rows(b, 1 /*labels*/, 0, c->stream));
  return copy_out(labels, c->grid, (size_t)n * n * sizeof(uint32_t), mem, c->stream);
}

int gcvt_ctx_iterate(gcvt_ctx *c, int iterations) {
  if (!c || iterations < 0) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  if (iterations == 0) return GCVT_OK;
  if (c->cur_n != c->n) return GCVT_ERR_STATE;
  return run_level(c, c->n, 0, iterations, 0x7fffffff, 0);
}

int gcvt_ctx_run(gcvt_ctx *c, int depth, int max_iter, gcvt_run_info *info) {
  if (!c || depth < 1) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  const int size = c->n;
  if (!pow2(size)) return GCVT_ERR_SIZE;
  for (int i = 0; i < depth; ++i)       // gcvt.cu:1091
    if ((size >> i) < 256) { depth = i; break; }
  int rc;
  // density pyramid (gcvt.cu:985-993)
  for (int l = 1; l < depth; ++l) {
    CK(launch_density_halve(c->density[l - 1], c->density[l], size >> l, c->stream));
    CK(launch_row_support(c->density[l], size >> l, c->support[l], c->stream));
    CK(launch_fixed_bits(c->mask, size >> l, c->fixed_bits[l], c->stream));
  }
  // the coarsest grid is the first (size >> (depth-1))^2 entries of the loaded
  // array (gcvt.cu:1099-1103)
  const int n0 = size >> (depth - 1);
  const size_t words_max = (size_t)(c->n_max / kBand) * c->n_max;
  CK(cudaMemsetAsync(c->bits[0], 0, words_max * sizeof(uint64_t), c->stream));
  CK(cudaMemsetAsync(c->bits[1], 0, words_max * sizeof(uint64_t), c->stream));
  CK(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
  CK(launch_grid_to_bits(c->input, n0, c->bits[0], c->err, c->stream));
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, c->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = reset_schedule(c, 0))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  if (herr) return GCVT_ERR_INPUT;
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
  CK(launch_bits_to_grid(c->bits[c->st_host->parity], n, c->grid, c->stream));
  return copy_out(voronoi, c->grid, (size_t)n * n * sizeof(uint32_t), mem, c->stream);
}

int gcvt_ctx_moments(gcvt_ctx *c, double *out4, int mem) {
  if (!c || !out4) return GCVT_ERR_ARGUMENT;
  if (mem != GCVT_MEM_HOST && mem != GCVT_MEM_DEVICE) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  const int n = c->cur_n;
  if (!c->moments) CK(cudaMalloc((void **)&c->moments, (size_t)4 * c->n_max * c->n_max * sizeof(double)));
  int level = 0;
  while ((c->n >> level) != n && level < 7) ++level;
  LevelBufs b = level_bufs(c, n, level);
  CK(launch_summary(b, 0, c->stream));
  CK(launch_rows(b, 0 /*lloyd*/, 0, c->stream));
  CK(launch_read_moments(b, c->moments, c->stream));
  return copy_out(out4, c->moments, (size_t)4 * n * n * sizeof(double), mem, c->stream);
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

int gcvt_ctx_time_kernels(gcvt_ctx *c, int iterations, float *ms3) {
  if (!c || !ms3 || iterations < 1) return GCVT_ERR_ARGUMENT;
  if (!c->loaded) return GCVT_ERR_STATE;
  if (c->input_err) return GCVT_ERR_INPUT;
  if (c->cur_n != c->n) return GCVT_ERR_STATE;
  int rc = pull_state(c);
  if (rc) return rc;
  DevState &h = *c->st_host;
  h.level = 0;
  h.stopped = 0;
  h.level_iters = 0;
  h.use_stop_rule = 0;
  h.fixed_iters = 0x7fffffff;
  h.energy_scale = 1.0 / ((double)c->n * (double)c->n);
  if ((rc = push_state(c))) return rc;
  cudaEvent_t ev[4];
  for (int i = 0; i < 4; ++i) CK(cudaEventCreate(&ev[i]));
  float acc[3] = {0.f, 0.f, 0.f};
  LevelBufs b = level_bufs(c, c->n, 0);
  for (int it = 0; it < iterations; ++it) {
    CK(cudaEventRecord(ev[0], c->stream));
    CK(launch_summary(b, 1, c->stream));
    CK(cudaEventRecord(ev[1], c->stream));
    CK(launch_rows(b, 0, 1, c->stream));
    CK(cudaEventRecord(ev[2], c->stream));
    CK(launch_update(b, c->stream));
    CK(cudaEventRecord(ev[3], c->stream));
    CK(cudaEventSynchronize(ev[3]));
    for (int k = 0; k < 3; ++k) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
      acc[k] += ms;
    }
  }
  for (int i = 0; i < 4; ++i) cudaEventDestroy(ev[i]);
  for (int k = 0; k < 3; ++k) ms3[k] = acc[k] / iterations;
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
