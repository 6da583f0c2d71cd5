// noalloc.cu -- exact labelling for callers that cannot allocate device
// memory: code running where cudaMalloc is unavailable or forbidden (a
// plugin handed pre-allocated buffers by a host that owns all device memory,
// a real-time loop that must not allocate after start-up, an allocator that
// is not the CUDA runtime's).  The caller passes the site grid and the label
// grid; every other buffer the labeller needs lives in one static device
// array of this file.
//
// The array holds the site bitmap, the column summaries, the iteration state
// and an error flag for grids up to kNoAllocMaxN = 2048 (about 0.8 MB; every
// GPU that loads the library keeps it until the process exits).  All calls
// share it: a call rewrites everything it reads before reading it, so the
// previous call's contents never leak, but two calls whose work overlaps on
// the GPU (different streams or threads without ordering between them) race
// on it.
//
// Host code may not use the array's name as a device address (in host code it
// names a host-side stand-in).  The first call on a device takes the array's
// device address with cudaGetSymbolAddress, with that device current, and
// caches it for the device.  A call is synchronous -- it reads back the error
// flag and waits for its stream -- so it cannot be captured into a graph.  A malformed site grid is found by the GPU while the labelling
// runs, so on GCVT_ERR_INPUT the label grid has been written with unspecified
// contents.
#include "gcvt_internal.cuh"
#include "../../include/gcvt_gb300.h"

#include <mutex>

namespace cvtgb {

constexpr int kNoAllocMaxN = 2048;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kWords = (size_t)(kNoAllocMaxN / kBand) * kNoAllocMaxN;
constexpr size_t kOffBits = 0;
constexpr size_t kOffPrev = align_up(kOffBits + kWords * sizeof(uint64_t));
constexpr size_t kOffNext = align_up(kOffPrev + kWords * sizeof(int16_t));
constexpr size_t kOffState = align_up(kOffNext + kWords * sizeof(int16_t));
constexpr size_t kOffErr = align_up(kOffState + sizeof(DevState));
constexpr size_t kNoAllocBytes = align_up(kOffErr + sizeof(int));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Per-call reset of what must start at zero: the state (bitmap 0 current, not
// stopped) and the error flag.  The bitmap and the summaries are fully
// rewritten by the labelling kernels before they are read.
__global__ void k_noalloc_reset(DevState *st, int *err) {
  if (threadIdx.x == 0) {
    DevState s = {};
    s.omega = 2.0f;
    *st = s;
    *err = 0;
  }
}

namespace {
std::mutex g_setup_mutex;
unsigned char *g_scratch_ptr[64] = {};  // device address of the array, per device
bool g_configured[64] = {};

int scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GCVT_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GCVT_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
  }
  if (!g_configured[dev]) {
    if (rows_configure() != cudaSuccess) return GCVT_ERR_CUDA;
    g_configured[dev] = true;
  }
  *out = g_scratch_ptr[dev];
  return GCVT_OK;
}
}  // namespace

}  // namespace cvtgb

using namespace cvtgb;

extern "C" int gcvt_label_grid_static(const int16_t *sites, int16_t *labels, int n,
                                      void *stream) {
  if (!sites || !labels) return GCVT_ERR_ARGUMENT;
  if (n < kMinN || n > kNoAllocMaxN || n % 256 != 0) return GCVT_ERR_SIZE;
  unsigned char *base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint64_t *bits = reinterpret_cast<uint64_t *>(base + kOffBits);
  DevState *st = reinterpret_cast<DevState *>(base + kOffState);
  int *err = reinterpret_cast<int *>(base + kOffErr);
  k_noalloc_reset<<<1, 32, 0, s>>>(st, err);
  if (cudaGetLastError() != cudaSuccess) return GCVT_ERR_CUDA;
  if (launch_grid_to_bits(reinterpret_cast<const uint32_t *>(sites), n, bits, err, nullptr, s) !=
      cudaSuccess)
    return GCVT_ERR_CUDA;
  LevelBufs b = {};
  b.n = n;
  b.bits[0] = bits;
  b.bits[1] = bits;
  b.bits[2] = bits;
  b.prev = reinterpret_cast<int16_t *>(base + kOffPrev);
  b.next = reinterpret_cast<int16_t *>(base + kOffNext);
  b.labels = reinterpret_cast<uint32_t *>(labels);
  b.st = st;
  if (launch_summary(b, 0, s) != cudaSuccess) return GCVT_ERR_CUDA;
  if (launch_rows(b, 0, s) != cudaSuccess) return GCVT_ERR_CUDA;
  int herr = 0;  // host stack: the only readback, no allocation
  if (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GCVT_ERR_CUDA;
  return herr ? GCVT_ERR_INPUT : GCVT_OK;
}
