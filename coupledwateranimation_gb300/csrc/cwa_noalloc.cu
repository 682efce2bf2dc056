// cwa_noalloc.cu — exclusive scan for callers that cannot allocate device
// memory.
//
// cwa_exclusive_scan_i32 asks the caller for a workspace (the scan's
// look-back needs one status word per tile of 8192 elements plus a ticket
// counter).  Some callers cannot provide one: code that runs inside a host
// application which owns the whole device-memory budget and hands out no
// allocations, and real-time loops that must not call cudaMalloc / cudaFree
// because those calls can block on or synchronise with the device.  This
// entry point serves them from a fixed scratch array that the library
// declares at file scope, so it allocates nothing itself.
//
// Limits and rules:
//   * n <= CWA_NOALLOC_SCAN_MAX_N (2^24 elements); larger n is rejected with
//     CWA_ERR_CAPACITY before anything is launched.
//   * The scratch array (66,048 bytes) lives on every GPU that loads the
//     library until the process exits.
//   * Each call made outside a stream capture looks up the array's device
//     address on the current device (so a cudaDeviceReset in between is
//     harmless); a call inside a capture uses the address the last
//     uncaptured call on that device found, so make one call before any
//     stream capture.
//   * All calls on a device share the one array, so calls whose kernels
//     overlap on the GPU race: issue them on one stream, or order them.
//     Overlapping calls give wrong sums (and may time out), but their
//     writes stay inside the array.  Each call clears the parts of the array
//     that must start at zero.
//   * A look-back that gives up sets a status word in the array;
//     cwa_scan_noalloc_status reads it after the call.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "cwa_internal.h"

namespace cwa {
namespace {

constexpr int32_t kNoAllocMaxN = CWA_NOALLOC_SCAN_MAX_N;
// ticket + tile states for kNoAllocMaxN elements (256 + 8 per tile; sized
// for 2048-element tiles, four times what the 8192-element tiles use), then one
// status word in its own 256-byte line
constexpr size_t kNoAllocScratchBytes = 256 + (size_t)(kNoAllocMaxN / 2048) * 8 + 256;
constexpr size_t kNoAllocStatusOffset = kNoAllocScratchBytes - 256;
static_assert(256 + (size_t)((kNoAllocMaxN + kScanTileItems - 1) / kScanTileItems) * 8 <= kNoAllocStatusOffset,
              "the scratch array must hold the ticket and every tile state of the largest scan");

static __device__ __align__(256) unsigned char g_scan_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (the array's
// host-side name is not a device address).  Outside a stream capture it is
// looked up on every call, so an address cached before a cudaDeviceReset is
// never used; inside a capture the last address found on this device is
// used, and a capture before any uncaptured call is an error.
cwa_status scratch_on_current_device(cudaStream_t stream, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    cudaGetLastError();  // clear a non-sticky error for the next call
    return CWA_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal above the no-allocation scan's table");
    return CWA_ERR_CAPACITY;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) {
    set_error(std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
    cudaGetLastError();  // clear a non-sticky error for the next call
    return CWA_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scan_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("cudaGetSymbolAddress(scan scratch): ") + cudaGetErrorString(e));
      cudaGetLastError();  // clear a non-sticky error for the next call
      return CWA_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  } else if (!g_scratch_addr[dev]) {
    set_error("no-allocation scan first called inside a stream capture: call it once before capturing");
    return CWA_ERR_INVALID_ARG;
  }
  *out = g_scratch_addr[dev];
  return CWA_OK;
}

}  // namespace
}  // namespace cwa

extern "C" cwa_status cwa_exclusive_scan_i32_noalloc(const int32_t* d_in, int32_t* d_out, int32_t n,
                                                     void* stream) {
  using namespace cwa;
  if (n < 0) {
    set_error("n < 0");
    return CWA_ERR_INVALID_ARG;
  }
  if (n > kNoAllocMaxN) {
    set_error("n above CWA_NOALLOC_SCAN_MAX_N (16,777,216): use cwa_exclusive_scan_i32 with a workspace");
    return CWA_ERR_CAPACITY;
  }
  if (n == 0) return CWA_OK;
  if (!d_in || !d_out) {
    set_error("null device pointer");
    return CWA_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  void* base = nullptr;
  cwa_status st = scratch_on_current_device(s, &base);
  if (st != CWA_OK) return st;
  if (scan_workspace_bytes(n) > kNoAllocStatusOffset) {  // guaranteed by the static_assert; kept as a guard
    set_error("no-allocation scan: scratch array too small for n");
    return CWA_ERR_CAPACITY;
  }
  ScanWorkspace ws;
  scan_bind_workspace(base, n, &ws);
  int32_t* status = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(base) + kNoAllocStatusOffset);
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int32_t), s);  // the look-back time-out flag
  if (e == cudaSuccess) e = scan_launch(d_in, d_out, n, n, false, ws, status, s, nullptr);
  if (e != cudaSuccess) {
    set_error(std::string("no-allocation scan: ") + cudaGetErrorString(e));
    cudaGetLastError();  // clear a non-sticky error for the next call
    return CWA_ERR_CUDA;
  }
  return CWA_OK;
}

extern "C" cwa_status cwa_scan_noalloc_status(void* stream) {
  using namespace cwa;
  cudaStream_t s = (cudaStream_t)stream;
  void* base = nullptr;
  cwa_status st = scratch_on_current_device(s, &base);
  if (st != CWA_OK) return st;
  int32_t v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, reinterpret_cast<char*>(base) + kNoAllocStatusOffset, sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error(std::string("no-allocation scan status: ") + cudaGetErrorString(e));
    cudaGetLastError();  // clear a non-sticky error for the next call
    return CWA_ERR_CUDA;
  }
  return status_from_bits(v);
}
