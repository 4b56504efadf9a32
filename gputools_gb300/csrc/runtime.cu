// runtime.cu -- error reporting, per-device streams and workspace, device
// selection.  The reference allocates and frees every device buffer per call
// (src/distance.cpp:277-316, src/correlation.cpp:83-160,
// src/kendall.cpp:13-55) and reports errors by longjmp-ing through R's
// error() (src/cuseful.cpp:95-102), which leaks what was allocated.  Here
// buffers are grow-only per-device slots reused across calls, and every
// failure is a status code plus a thread-local message.
#include "common.cuh"

#include <cstdarg>
#include <sys/mman.h>
#include <unistd.h>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

namespace gt {

namespace {
thread_local char t_err[1024] = {0};

constexpr int kMaxDevices = 64;

struct DeviceState {
  cudaStream_t stream = nullptr;
  void *slot[WS_NSLOTS] = {};
  size_t bytes[WS_NSLOTS] = {};
  int *err = nullptr;  // error word of the kernels with bounded waits
  void *host = nullptr;  // page-locked staging of host outputs
  size_t host_bytes = 0;
  int sms = 0;
};

constexpr uint64_t kDefaultWaitNs = 2000000000ull;  // 2 s per barrier wait
std::atomic<uint64_t> g_wait_ns{kDefaultWaitNs};

std::mutex g_mu;
DeviceState g_dev[kMaxDevices];
std::atomic<unsigned long long> g_launches{0};
}  // namespace

void count_launch(int n) { g_launches.fetch_add((unsigned long long)n); }

namespace {
struct ProfRecord {
  std::string name;
  cudaEvent_t e0, e1;
};
std::atomic<int> g_prof_on{0};
std::mutex g_prof_mu;
std::vector<ProfRecord> g_prof_pending;
struct ProfTotal {
  std::string name;
  double ms;
  unsigned long long count;
};
std::vector<ProfTotal> g_prof_totals;

void prof_drain_locked() {
  for (auto &r : g_prof_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.e1) == cudaSuccess && cudaEventElapsedTime(&ms, r.e0, r.e1) == cudaSuccess) {
      bool found = false;
      for (auto &t : g_prof_totals)
        if (t.name == r.name) { t.ms += ms; t.count++; found = true; break; }
      if (!found) g_prof_totals.push_back({r.name, double(ms), 1});
    }
    cudaEventDestroy(r.e0);
    cudaEventDestroy(r.e1);
  }
  g_prof_pending.clear();
}
}  // namespace

ProfScope::ProfScope(const char *name, cudaStream_t st) : name_(name), st_(st) {
  if (!g_prof_on.load()) return;
  if (cudaEventCreate(&e0_) != cudaSuccess) { e0_ = nullptr; return; }
  cudaEventRecord(e0_, st_);
}

ProfScope::~ProfScope() {
  if (!e0_) return;
  cudaEvent_t e1 = nullptr;
  if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0_); return; }
  cudaEventRecord(e1, st_);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_pending.push_back({name_, e0_, e1});
}

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err, sizeof(t_err), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { t_err[0] = 0; }
const char *last_error() { return t_err; }

int current_device(int *dev) {
  cudaError_t e = cudaGetDevice(dev);
  if (e != cudaSuccess)
    return fail(GT_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
  if (*dev < 0 || *dev >= kMaxDevices)
    return fail(GT_ENODEV, "device ordinal %d out of range", *dev);
  return GT_OK;
}

cudaStream_t lib_stream() {
  int dev = 0;
  if (current_device(&dev) != GT_OK) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState &d = g_dev[dev];
  if (!d.stream) cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking);
  return d.stream;
}

void *host_direct_ptr(void *host) {
  static int enabled = -1;
  if (enabled < 0) {
    const char *e = std::getenv("GT_DIRECT_HOST");
    enabled = (e && e[0] == '0') ? 0 : 1;
  }
  if (!enabled || !host) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

namespace {
// Whether every page of [p, p + bytes) is resident (mincore).
bool pages_resident(const void *p, size_t bytes) {
  const long pg = sysconf(_SC_PAGESIZE);
  if (pg <= 0) return false;
  const uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(pg - 1);
  const uintptr_t e = reinterpret_cast<uintptr_t>(p) + bytes;
  const size_t npages = (e - a + size_t(pg) - 1) / size_t(pg);
  std::vector<unsigned char> vec(npages);
  if (mincore(reinterpret_cast<void *>(a), e - a, vec.data()) != 0) return false;
  for (unsigned char v : vec)
    if (!(v & 1)) return false;
  return true;
}

int pageable_access() {
  static int cached[kMaxDevices];
  static bool init[kMaxDevices];
  int dev = 0;
  if (current_device(&dev) != GT_OK) return 0;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!init[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    cached[dev] = v;
    init[dev] = true;
  }
  return cached[dev];
}
}  // namespace

void *host_output_ptr(void *host, size_t bytes) {
  static int pageable_enabled = -1;
  if (pageable_enabled < 0) {
    const char *e = std::getenv("GT_DIRECT_PAGEABLE");
    pageable_enabled = (e && e[0] == '1') ? 1 : 0;
  }
  if (!host || bytes == 0) return nullptr;
  if (void *d = host_direct_ptr(host)) return d;
  const char *e = std::getenv("GT_DIRECT_HOST");
  if ((e && e[0] == '0') || !pageable_enabled || bytes < kDirectMin) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeUnregistered || !pageable_access()) return nullptr;
  return pages_resident(host, bytes) ? host : nullptr;
}

int sm_count() {
  int dev = 0;
  if (current_device(&dev) != GT_OK) return 148;
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState &d = g_dev[dev];
  if (!d.sms) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    d.sms = v > 0 ? v : 148;
  }
  return d.sms;
}

int ws_get(int slot, size_t bytes, void **ptr) {
  if (slot < 0 || slot >= WS_NSLOTS) return fail(GT_EINVAL, "bad workspace slot");
  int dev = 0;
  GT_TRY(current_device(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState &d = g_dev[dev];
  if (bytes == 0) bytes = 256;
  if (d.bytes[slot] < bytes) {
    if (d.slot[slot]) {
      // The slot may still be read by work queued earlier on any stream.
      cudaDeviceSynchronize();
      cudaFree(d.slot[slot]);
      d.slot[slot] = nullptr;
      d.bytes[slot] = 0;
    }
    // Round up so that slowly growing requests do not reallocate each call.
    size_t want = bytes + bytes / 8;
    want = (want + (1u << 20) - 1) & ~size_t((1u << 20) - 1);
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(GT_ENOMEM, "device workspace of %zu bytes unavailable: %s", want,
                  cudaGetErrorString(e));
    }
    d.slot[slot] = p;
    d.bytes[slot] = want;
  }
  *ptr = d.slot[slot];
  return GT_OK;
}

int host_ws_get(size_t bytes, void **ptr) {
  int dev = 0;
  GT_TRY(current_device(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState &d = g_dev[dev];
  if (d.host_bytes < bytes) {
    if (d.host) {
      cudaDeviceSynchronize();
      cudaFreeHost(d.host);
      d.host = nullptr;
      d.host_bytes = 0;
    }
    size_t want = bytes + bytes / 8;
    want = (want + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
    void *p = nullptr;
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(GT_ENOMEM, "page-locked staging of %zu bytes unavailable: %s", want,
                  cudaGetErrorString(e));
    }
    d.host = p;
    d.host_bytes = want;
  }
  *ptr = d.host;
  return GT_OK;
}

int device_error_word(int **p) {
  int dev = 0;
  GT_TRY(current_device(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState &d = g_dev[dev];
  if (!d.err) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, 256);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(GT_ENOMEM, "device error word unavailable: %s", cudaGetErrorString(e));
    }
    e = cudaMemset(q, 0, 256);
    if (e != cudaSuccess) {
      cudaFree(q);
      return fail(GT_ECUDA, "clearing the device error word: %s", cudaGetErrorString(e));
    }
    d.err = static_cast<int *>(q);
  }
  *p = d.err;
  return GT_OK;
}

int device_error_check(cudaStream_t s, bool *failed) {
  *failed = false;
  int *err = nullptr;
  GT_TRY(device_error_word(&err));
  int h = 0;
  GT_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaStreamSynchronize(s));
  if (h) {
    *failed = true;
    GT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    GT_CUDA(cudaStreamSynchronize(s));
  }
  return GT_OK;
}

uint64_t wait_limit_ns() { return g_wait_ns.load(); }

uint32_t wait_sleep_hint_ns() {
  // a suspending wait may outlast a short limit: below 1 ms the waits poll
  return g_wait_ns.load() < 1000000ull ? 0u : 100000u;
}

void ws_release_all() {
  std::lock_guard<std::mutex> lk(g_mu);
  int cur = -1;
  cudaGetDevice(&cur);
  for (int dev = 0; dev < kMaxDevices; dev++) {
    DeviceState &d = g_dev[dev];
    bool any = d.err != nullptr || d.host != nullptr;
    for (int s = 0; s < WS_NSLOTS; s++) any |= d.slot[s] != nullptr;
    if (!any) continue;
    cudaSetDevice(dev);
    cudaDeviceSynchronize();
    for (int s = 0; s < WS_NSLOTS; s++) {
      if (d.slot[s]) cudaFree(d.slot[s]);
      d.slot[s] = nullptr;
      d.bytes[s] = 0;
    }
    if (d.err) cudaFree(d.err);
    d.err = nullptr;
    if (d.host) cudaFreeHost(d.host);
    d.host = nullptr;
    d.host_bytes = 0;
  }
  if (cur >= 0) cudaSetDevice(cur);
}

}  // namespace gt

extern "C" {

const char *gt_last_error(void) { return gt::last_error(); }

int gt_version(void) { return 10000; }

uint64_t gt_kernel_launches(void) { return gt::g_launches.load(); }

void gt_release_workspace(void) { gt::ws_release_all(); }

int gt_device_status(void *stream) {
  gt::clear_error();
  bool failed = false;
  GT_TRY(gt::device_error_check(static_cast<cudaStream_t>(stream), &failed));
  if (failed) return gt::fail(GT_ETIMEOUT, "a bounded wait inside a device kernel timed out");
  return GT_OK;
}

int gt_set_wait_limit_ns(uint64_t ns) {
  gt::clear_error();
  gt::g_wait_ns.store(ns == 0 ? gt::kDefaultWaitNs : ns);
  return GT_OK;
}

void gt_profile_enable(int on) { gt::g_prof_on.store(on ? 1 : 0); }

void gt_profile_reset(void) {
  std::lock_guard<std::mutex> lk(gt::g_prof_mu);
  gt::prof_drain_locked();
  gt::g_prof_totals.clear();
}

int gt_profile_kernel_ms(const char *name, double *total_ms, uint64_t *launches) {
  gt::clear_error();
  if (!name) return gt::fail(GT_EINVAL, "null kernel name");
  std::lock_guard<std::mutex> lk(gt::g_prof_mu);
  gt::prof_drain_locked();
  double ms = 0.0;
  unsigned long long c = 0;
  for (auto &t : gt::g_prof_totals)
    if (t.name == name) { ms = t.ms; c = t.count; }
  if (total_ms) *total_ms = ms;
  if (launches) *launches = c;
  return GT_OK;
}

}  // extern "C"
