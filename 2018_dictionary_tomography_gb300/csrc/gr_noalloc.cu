// Forward projection that needs no workspace from the caller.
//
// gr_radproj needs a device workspace for its per-(angle, tile) atom
// bitmaps and loss partials, which the caller allocates.  Some callers cannot
// allocate device memory: a host application that owns the whole GPU memory
// budget and hands plug-ins only the buffers they must fill, a binding from a
// language that can pass device pointers but has no device allocator of its
// own, or a hot loop that must not call cudaMalloc/cudaFree because those
// calls synchronise the device.  For them, gr_radproj_noalloc runs the same
// kernels on a fixed scratch area compiled into this library.
//
// The scratch is a file-scope __device__ array of kNoAllocScratchBytes
// (4 MiB).  Every GPU that loads this library holds it until the process
// exits.  All calls share it and it keeps the contents of the last call; the
// projection clears the bitmap part itself before use and overwrites the rest,
// so nothing carries over between calls.  Calls whose GPU work overlaps (two
// streams, or two host threads, at the same time) race on the scratch and
// must be serialised by the caller.
//
// Host code cannot use the array's name as a device address (on the host it
// names a host-side stand-in).  The first call on each device therefore looks
// the address up with cudaGetSymbolAddress, with that device current, and
// caches it; make that first call before any stream capture on the device.
// The address belongs to the module loaded in one CUDA context: the cache is
// keyed by the context's process-unique id (cuCtxGetId), so a call made
// under another context of the device (a context the caller created, or the
// primary context re-created after cudaDeviceReset) looks the address up
// again instead of reusing one that is no longer valid.
#include <cuda.h>

#include <mutex>

#include "gauss_radon.h"
#include "gr_kernels.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;

// Driver entry points, found through the runtime (the library links only
// the CUDA runtime, so that it loads on machines without a driver).
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

bool driver_entry_points() {
  if (g_ctx_get_current && g_ctx_get_id) return true;
  void *a = nullptr, *b = nullptr;
  cudaDriverEntryPointQueryResult qa, qb;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) !=
          cudaSuccess ||
      cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) !=
          cudaSuccess ||
      qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b) {
    cudaGetLastError();
    return false;
  }
  g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(a);
  g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(b);
  return true;
}

struct ScratchAddr {
  unsigned long long ctx_id;  // 0: not looked up yet
  void *ptr;
};
ScratchAddr g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch in the current context of the current
// device (looked up once per device and context).  Returns nullptr on failure.
void *noalloc_scratch_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!driver_entry_points()) return nullptr;
  }
  void *ptr = nullptr;
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return nullptr;
  if (ctx == nullptr) {
    // no context current on this thread yet: the runtime makes the device's
    // primary context current on its first call, this lookup
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || ptr == nullptr) {
      cudaGetLastError();  // reset the runtime's last-error slot left by the failure
      return nullptr;
    }
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return nullptr;
  }
  unsigned long long id = 0;
  if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS || id == 0) return nullptr;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  ScratchAddr &c = g_noalloc_addr[dev];
  if (c.ctx_id != id || c.ptr == nullptr) {
    if (ptr == nullptr &&
        (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || ptr == nullptr)) {
      cudaGetLastError();
      return nullptr;
    }
    c.ctx_id = id;
    c.ptr = ptr;
  }
  return c.ptr;
}

}  // namespace

extern "C" int gr_radproj_noalloc(const gr_atoms *atoms, const gr_geometry *geom,
                                  float *R, void *stream) {
  using namespace gr;
  if (!atoms || !geom || !R) return GR_ERR_ARG;
  const size_t need = gr_workspace_bytes(GR_OP_PROJECT, atoms, geom);
  if (need == 0) return GR_ERR_ARG;  // invalid atoms or geometry
  if (need > kNoAllocScratchBytes) return GR_ERR_TOO_LARGE;
  void *ws = noalloc_scratch_for_current_device();
  if (ws == nullptr) return GR_ERR_LAUNCH;
  return gr_radproj(atoms, geom, R, ws, kNoAllocScratchBytes, stream);
}
