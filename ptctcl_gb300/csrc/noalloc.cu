// noalloc.cu -- hora_gb_has_deadlock_noalloc: the deadlock predicate without any device allocation.
//
// Who needs this: a caller whose device memory is already owned by another allocator (a framework
// pool or arena that reserved the device up front, so a raw cudaMalloc would fail or break that
// allocator's accounting), and a caller in a latency-critical loop that cannot afford the implicit
// device synchronisation cudaMalloc/cudaFree bring. Such a caller hands in device buffers it
// already owns for the states and the answers; everything else the kernel needs -- the compiled
// network tables, their view and the error counters -- lives in the one fixed-size array below.
//
// The array is a file-scope __device__ variable, so every GPU that loads this library holds
// kNoAllocScratchBytes of it until the process exits. Host code cannot use its name as a device
// address: the address is fetched once per device with cudaGetSymbolAddress (with that device
// current) the first time this entry point runs on it, and passed to the kernel as a pointer.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"
#include "level_kernels.cuh"

namespace hgb {

// Stated maximum: the network tables, their view and the counters must fit in 1 MiB.
constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;
constexpr size_t kNoAllocCtlOffset = 0;      // Ctl counters (cleared on every call)
constexpr size_t kNoAllocViewOffset = 256;   // one NetView
constexpr size_t kNoAllocBlobOffset = 1024;  // the instance's int32 tables

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static_assert(sizeof(Ctl) <= kNoAllocViewOffset - kNoAllocCtlOffset, "Ctl must fit its slot");
static_assert(sizeof(NetView) <= kNoAllocBlobOffset - kNoAllocViewOffset, "NetView must fit its slot");

static std::mutex g_noalloc_mu;
static std::vector<unsigned char*> g_noalloc_ptr;   // per device: device address of the array

// Device address of the array on the current device (set up once per device).
static int noalloc_scratch(unsigned char** out, std::string& err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { err = std::string("CUDA: cudaGetDevice: ") + cudaGetErrorString(e); return HORA_E_CUDA; }
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if ((int)g_noalloc_ptr.size() <= dev) g_noalloc_ptr.resize(dev + 1, nullptr);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      err = std::string("CUDA: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return HORA_E_CUDA;
    }
    g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return HORA_OK;
}

#define HGB_FOR_DIMS_NA(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(17)

}  // namespace hgb

using namespace hgb;

extern "C" const char* hora_gb_last_error(void);
namespace hgb { void set_last_error(const std::string& m); }

extern "C" HORA_GB_API int32_t hora_gb_has_deadlock_noalloc(const hora_net_desc* net, int32_t n,
                                                            const int32_t* d_locs, const int32_t* d_ints,
                                                            const int32_t* d_zones, int32_t* d_out) {
  std::string err;
  set_last_error("");
  if (n < 0 || (n > 0 && (!d_locs || !d_zones || !d_out))) { set_last_error("bad arguments"); return HORA_E_INVALID; }
  HostNet H;
  int rc = compile_net(net, HORA_Q_DEADLOCK, nullptr, nullptr, H, err);
  if (rc) { set_last_error(err); return rc; }
  if (H.nints > 0 && n > 0 && !d_ints) { set_last_error("bad arguments: null integer states"); return HORA_E_INVALID; }
  std::vector<int32_t> blob;
  std::vector<size_t> offs;
  build_blob(H, blob, offs);
  if (kNoAllocBlobOffset + blob.size() * 4 > kNoAllocScratchBytes) {
    set_last_error("network tables (" + std::to_string(blob.size() * 4) + " bytes) exceed the " +
                   std::to_string(kNoAllocScratchBytes - kNoAllocBlobOffset) +
                   "-byte static scratch of the allocation-free entry point");
    return HORA_E_INVALID;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) { set_last_error("no CUDA device visible"); return HORA_E_NO_DEVICE; }
  unsigned char* base = nullptr;
  if ((rc = noalloc_scratch(&base, err))) { set_last_error(err); return rc; }
  if (n == 0) return HORA_OK;
  const NetView V = make_view(H, reinterpret_cast<const int32_t*>(base + kNoAllocBlobOffset), offs, 63);
  // Legacy default stream, synchronous copies: the call owns the array for its whole duration.
  cudaError_t e = cudaMemcpy(base + kNoAllocBlobOffset, blob.data(), blob.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + kNoAllocViewOffset, &V, sizeof(NetView), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(base + kNoAllocCtlOffset, 0, sizeof(Ctl));
  if (e != cudaSuccess) { set_last_error(std::string("CUDA: ") + cudaGetErrorString(e)); return HORA_E_CUDA; }
  const NetView* views = reinterpret_cast<const NetView*>(base + kNoAllocViewOffset);
  Ctl* ctl = reinterpret_cast<Ctl*>(base + kNoAllocCtlOffset);
  switch (H.dim) {
#define HGB_CASE(D) case D: Level<D>::has_deadlock(views, d_locs, d_ints, d_zones, n, d_out, ctl, 0); break;
    HGB_FOR_DIMS_NA(HGB_CASE)
#undef HGB_CASE
    default: set_last_error("unsupported DBM dimension"); return HORA_E_NOT_SUPPORTED;
  }
  e = cudaGetLastError();
  Ctl h;
  if (e == cudaSuccess) e = cudaMemcpy(&h, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { set_last_error(std::string("CUDA: ") + cudaGetErrorString(e)); return HORA_E_CUDA; }
  if (h.err) { set_last_error("deadlock test exceeded its escape table"); return (int32_t)h.err; }
  return HORA_OK;
}
