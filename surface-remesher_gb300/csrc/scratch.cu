// scratch.cu -- grow-only device scratch for the one-shot entry points
// (gcvt_rasterize, gcvt_lift, gcvt_vertex_weights, gcvt_ctx_delaunay).  Their
// buffers depend on the input (triangles, grid cells, list lengths, sites),
// so they were allocated and freed per call; on a GB300 host a cudaMalloc /
// cudaFree pair costs tens of microseconds, more than some of these calls'
// kernels.  A Scratch hands out
// 256-byte aligned pieces of blocks it keeps for the device: a call that
// outgrows the current block gets another one, and the next call finds one
// block covering the total.  Calls on a device are serialised by its lock,
// which is released only after the call's stream has drained.
#include "gcvt_internal.cuh"

#include <algorithm>
#include <mutex>
#include <vector>

namespace cvtgb {

namespace {

struct Pool {
  std::mutex m;
  std::vector<std::pair<char *, size_t>> blocks;  // (base, capacity)
};

Pool g_pool[64];

}  // namespace

Scratch::Scratch(cudaStream_t stream)
    : pool_(nullptr), stream_(stream), block_(0), used_(0), total_(0), ok_(false) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  Pool *p = &g_pool[dev];
  p->m.lock();
  pool_ = p;
  ok_ = true;
}

Scratch::~Scratch() {
  if (!pool_) return;
  Pool *p = static_cast<Pool *>(pool_);
  // nothing queued by this call may still use the memory once it is released
  // (on the success paths the call has synchronised already: no wait)
  cudaStreamSynchronize(stream_);
  // several blocks this time: replace them by one block of their total, so a
  // call of the same size needs no allocation next time
  if (p->blocks.size() > 1 && cudaDeviceSynchronize() == cudaSuccess) {
    size_t cap = 0;
    for (auto &b : p->blocks) {
      cudaFree(b.first);
      cap += b.second;
    }
    p->blocks.clear();
    char *q = nullptr;
    if (cudaMalloc((void **)&q, cap) == cudaSuccess) p->blocks.push_back({q, cap});
  }
  p->m.unlock();
}

void *Scratch::take(size_t bytes) {
  if (!ok_) return nullptr;
  Pool *p = static_cast<Pool *>(pool_);
  bytes = (bytes + 255) & ~(size_t)255;
  if (bytes == 0) bytes = 256;
  while (block_ < p->blocks.size()) {
    auto &b = p->blocks[block_];
    if (used_ + bytes <= b.second) {
      void *r = b.first + used_;
      used_ += bytes;
      total_ += bytes;
      return r;
    }
    ++block_;
    used_ = 0;
  }
  // a new block: at least this piece, at least what the call has taken so far
  const size_t cap = std::max(bytes, std::max(total_, (size_t)(4 << 20)));
  char *q = nullptr;
  if (cudaMalloc((void **)&q, cap) != cudaSuccess) return nullptr;
  p->blocks.push_back({q, cap});
  block_ = p->blocks.size() - 1;
  used_ = bytes;
  total_ += bytes;
  return q;
}

}  // namespace cvtgb
