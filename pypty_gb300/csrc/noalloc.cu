// pty_fft2_noalloc: the batched window FFT of pty_fft2 without a caller-provided workspace.
//
// Some callers cannot allocate device memory: a host application that owns every device
// allocation through its own pool and forbids direct cudaMalloc, code that runs while a
// CUDA graph is being captured (cudaMalloc is not permitted during stream capture), or a
// real-time loop that must not pay for an allocation. pty_fft2 needs a small workspace for
// its twiddle tables; this entry point keeps those tables in a fixed array of device memory
// that belongs to the library instead. The array is created when the library is loaded on a
// device and stays allocated on every GPU that loads the library until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "plan.h"

namespace {

using pty::Geo;

// Twiddle tables of both supported windows, side by side: W = 64 at offset 0, W = 128
// after it. 128 + 256 complex64 values = 3 KiB, the whole static scratch.
constexpr int kTw64 = Geo<64>::TW1 + Geo<64>::TW2;
constexpr int kTw128 = Geo<128>::TW1 + Geo<128>::TW2;
constexpr int kScratchEntries = kTw64 + kTw128;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float2 g_fft_scratch[kScratchEntries];

std::mutex g_setup_mutex;
float2* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_fft_scratch on the current device. In host code the array's name is
// only a stand-in for the symbol, never a device address, so the address is looked up once
// per device (with that device current) and cached.
int scratch_for_current_device(float2** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PTY_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return PTY_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_fft_scratch) != cudaSuccess || p == nullptr) return PTY_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<float2*>(p);
  }
  *out = g_scratch_ptr[dev];
  return PTY_OK;
}

}  // namespace

extern "C" int pty_fft2_noalloc(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse,
                                int32_t shift, void* stream) {
  // The static scratch holds twiddle tables for windows of 64 and 128 only.
  if (window != 64 && window != 128) return PTY_ERR_UNSUPPORTED;
  if (!in || !out || batch <= 0) return PTY_ERR_INVALID;
  float2* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != PTY_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const float2* src = static_cast<const float2*>(in);
  float2* dst = static_cast<float2*>(out);
  // Every call rewrites the whole table it uses before reading it, so nothing has to start
  // at zero and the previous call's contents are never read.
  if (window == 64) return pty::run_fft2<64>(src, dst, batch, inverse, shift, scratch, st);
  return pty::run_fft2<128>(src, dst, batch, inverse, shift, scratch + kTw64, st);
}
