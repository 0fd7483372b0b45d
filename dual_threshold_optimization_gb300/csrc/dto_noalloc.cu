// dto_noalloc.cu -- device scratch for dto_run_range_noalloc, the entry point
// that allocates nothing.
//
// Some callers cannot call cudaMalloc at the moment they want a permutation
// null: a process whose memory manager owns every device allocation (a
// framework's pool with a fixed budget, an embedding host that hands device
// memory out itself), or a host runtime that forbids allocation on its
// request path.  For them, the intermediates of the run (permutation labels,
// the task counter, per-task optima) live in one file-scope device array of
// fixed size, kNoAllocBytes.  Every GPU that loads libdto.so holds that array
// until the process exits.
//
// Host code cannot use the array's name as a device address: in host code it
// names a host-side stand-in.  The device address is obtained once per
// device, with that device current, by cudaGetSymbolAddress, and passed to the
// kernels.  The cached address belongs to the device's primary context (every
// call makes the device current with cudaSetDevice, which selects it); after
// cudaDeviceReset, or under another context of the same device, the cache is
// not valid, and those uses are not supported.  All calls share the array and
// it keeps the last call's contents; the task counter is cleared by every
// call.  Calls whose GPU work overlaps (two streams, or two host threads with
// contexts on one device) race on the array.
#include <cuda_runtime.h>

#include <mutex>

#include "dto_internal.h"

namespace dto {

constexpr size_t kNoAllocBytes = (size_t)32 << 20;  // 32 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_ptr[kMaxDevices] = {};
}  // namespace

// Device address of the scratch array on `device` (which must be current, in
// its primary context).  The first call on a device resolves it, so that first
// call should come before any stream capture.
cudaError_t noalloc_scratch(int device, void** ptr, size_t* bytes) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_ptr[device] = p;
  }
  *ptr = g_ptr[device];
  *bytes = kNoAllocBytes;
  return cudaSuccess;
}

__global__ void noalloc_copy_p(const TaskResult* __restrict__ r, double* __restrict__ out, int n) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = r[t].p;
}

cudaError_t launch_noalloc_copy_p(const TaskResult* r, double* out, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  noalloc_copy_p<<<(n + 255) / 256, 256, 0, s>>>(r, out, n);
  return cudaGetLastError();
}

}  // namespace dto
