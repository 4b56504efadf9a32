// common.cuh -- shared runtime pieces of libgputools_gb300: status codes,
// the thread-local error message, per-device streams and the grow-only
// device workspace that replaces the reference's per-call cudaMalloc/cudaFree
// (src/distance.cpp:277-316, src/correlation.cpp:83-160, src/kendall.cpp:13-55).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdio>

#include "gputools_gb300.h"

namespace gt {

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const char *fmt, ...);
// Clears the calling thread's last error.
void clear_error();
const char *last_error();

// CUDA runtime call -> GT_ECUDA with the call site in the message.
#define GT_CUDA(expr)                                                          \
  do {                                                                         \
    cudaError_t _e = (expr);                                                   \
    if (_e != cudaSuccess)                                                     \
      return ::gt::fail(GT_ECUDA, "%s failed: %s (%s:%d)", #expr,              \
                        cudaGetErrorString(_e), __FILE__, __LINE__);           \
  } while (0)

#define GT_TRY(expr)                                                           \
  do {                                                                         \
    int _s = (expr);                                                           \
    if (_s != GT_OK) return _s;                                                \
  } while (0)

// Library-private non-blocking stream of the current device (created once).
cudaStream_t lib_stream();

// Synchronises a stream when it goes out of scope.  A host entry that queues
// copies from or to the caller's memory holds one, so that no return path
// -- an error after the first copy included -- leaves copies running on
// memory the caller owns again.
class StreamSyncGuard {
 public:
  explicit StreamSyncGuard(cudaStream_t s) : s_(s) {}
  ~StreamSyncGuard() { cudaStreamSynchronize(s_); }
  StreamSyncGuard(const StreamSyncGuard &) = delete;
  StreamSyncGuard &operator=(const StreamSyncGuard &) = delete;

 private:
  cudaStream_t s_;
};

// Named slots of the per-device workspace.  Each slot is a grow-only device
// buffer kept across calls and released by gt_release_workspace().
enum WsSlot {
  WS_IN_A = 0, WS_IN_B, WS_OUT0, WS_OUT1, WS_OUT2, WS_SCRATCH0, WS_SCRATCH1,
  WS_SCRATCH2, WS_SCRATCH3, WS_SCRATCH4,
  // the distance adjoint's own slots (it calls the Euclid path, which uses
  // WS_SCRATCH0..3, in between)
  WS_ADJ0, WS_ADJ1, WS_ADJ2,
  WS_TILES,  // tile tables of banded launches
  WS_NSLOTS
};
// Device buffer of at least `bytes` for `slot` on the current device.
int ws_get(int slot, size_t bytes, void **ptr);
void ws_release_all();
// Page-locked host buffer of at least `bytes` for the current device
// (grow-only, kept across calls, released with the device workspace).
int host_ws_get(size_t bytes, void **ptr);

// Counts kernel launches (gt_kernel_launches); call once per launch.
void count_launch(int n = 1);

// Event timing of one launch on its stream (enabled by gt_profile_enable).
class ProfScope {
 public:
  ProfScope(const char *name, cudaStream_t st);
  ~ProfScope();
  ProfScope(const ProfScope &) = delete;
  ProfScope &operator=(const ProfScope &) = delete;

 private:
  const char *name_;
  cudaStream_t st_;
  cudaEvent_t e0_ = nullptr;
};

// Device-usable address through which kernels may write the host buffer
// `host` directly (page-locked memory, reached over NVLink-C2C or PCIe), or
// nullptr when the buffer must be staged through device memory: pageable
// pages, even where the GPU can reach them, may be unpopulated and fault one
// by one.  GT_DIRECT_HOST=0 disables it.
void *host_direct_ptr(void *host);

// Device-usable address of a host output buffer of a synchronous entry
// (`bytes` long), or nullptr when it must be staged through device memory:
//  * page-locked memory is written in place by the kernels;
//  * pageable memory (what R's .C passes) is written in place too where the
//    device reaches the host's page tables (cudaDevAttrPageableMemoryAccess,
//    GB300 over NVLink-C2C) and every page of the buffer is resident: the
//    kernels' writes then overlap the computation.  A page that is not yet
//    populated would be faulted in one at a time (measured: 2.2 GB/s against
//    125 GB/s on resident pages), so buffers with non-resident pages, and
//    buffers below kDirectMin bytes, are staged;
//  * anything else is staged.
// GT_DIRECT_HOST=0 disables writing in place, GT_DIRECT_PAGEABLE=0 only the
// pageable case.  (Page-locking the caller's buffer for the call,
// cudaHostRegister, measured slower than either: 8 to 105 ms per 1.6 GB.)
void *host_output_ptr(void *host, size_t bytes);
constexpr size_t kDirectMin = size_t(1) << 20;

// Per-device error word of the kernels with bounded waits (allocated and
// zeroed on first use, kept until gt_release_workspace).  Kernels only set it;
// device_error_check() reads and clears it.
int device_error_word(int **p);
// Synchronises `s`, reads the current device's error word and clears it;
// *failed is set when a bounded wait inside a kernel gave up since the last
// check on this device.
int device_error_check(cudaStream_t s, bool *failed);

// Limit of each bounded device-side wait, in nanoseconds (2 s unless changed
// by gt_set_wait_limit_ns), and the sleep hint that goes with it.
uint64_t wait_limit_ns();
uint32_t wait_sleep_hint_ns();

// Host-side reads of the device the library runs on.
int current_device(int *dev);
int sm_count();

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace gt
