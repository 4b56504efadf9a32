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
  WS_SCRATCH2, WS_SCRATCH3, WS_SCRATCH4, WS_NSLOTS
};
// Device buffer of at least `bytes` for `slot` on the current device.
int ws_get(int slot, size_t bytes, void **ptr);
void ws_release_all();

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

// A host output buffer of a synchronous entry, as its kernels reach it.
// map() returns the device-usable address of `host` (`bytes` long), or
// nullptr when it must be staged through device memory:
//  * page-locked memory is written in place;
//  * pageable memory from kRegisterMin bytes on (R's .C vectors are such) is
//    page-locked for the call with cudaHostRegister and written in place --
//    on GB300 this costs ~1.6 ms per GB and the kernels then write at the
//    host link's rate, where a staged pageable copy runs at half of it;
//  * anything else (small, or not registrable) is staged.
// The registration is released by the destructor: declare the object before
// the StreamSyncGuard of the call, so that the stream is synchronised first.
// GT_DIRECT_HOST=0 disables writing in place, GT_REGISTER_HOST=0 only the
// registration.
class HostOutput {
 public:
  static constexpr size_t kRegisterMin = size_t(1) << 20;
  HostOutput() = default;
  ~HostOutput();
  HostOutput(const HostOutput &) = delete;
  HostOutput &operator=(const HostOutput &) = delete;
  void *map(void *host, size_t bytes);
  bool registered() const { return reg_ != nullptr; }

 private:
  void *reg_ = nullptr;
};

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
