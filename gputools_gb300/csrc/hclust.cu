// hclust.cu -- gpuHclust / gpuDistClust: hierarchical clustering of a
// device-resident distance matrix.
//
// Reference: R/gpuHclust.R:41-146 -> Rhcluster / Rdistclust
// (src/rinterface.cpp) -> hclusterPreparedDistances (src/hcluster.cpp:40-201)
// with the kernels of inst/cuda/hcluster.cu: n - 1 times, every active row's
// minimum over columns 0..row (find_min1_kernel, a full scan of the lower
// triangle), the smallest of those (find_min2_kernel), then the linkage
// update of the merged row and column (single, complete, wpgma, average,
// median, centroid, flexible_group, flexible, ward, mcquitty).  That is
// O(n^3) work and 3 (n - 1) launches.
//
// Here every row keeps its minimum (value and column) from one scan; a merge
// of columns c < r changes only row r, the entries (x, r) and (x, c) of the
// rows below, and makes row c inactive, so after the update a row is scanned
// again only if its kept minimum sat in column c or r (and row r always); the
// other rows below r compare their kept minimum with the new (x, r).  Ties
// are broken as the reference's 32-lane strided scan and tree reduction break
// them (value, then column mod 32, then column; rows likewise), so the merges
// are the reference's.  One CTA runs all merges (no inter-CTA waits: the
// per-merge work is O(n) and latency-bound), after a multi-CTA kernel that
// initialises the kept minima.  The linkage expressions are evaluated as the
// reference writes them (float, with its double promotions), each operation
// rounded on its own.
#include "common.cuh"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace gt {

namespace {

constexpr int kHcThreads = 1024;
enum { HC_SINGLE = 0, HC_COMPLETE, HC_WPGMA, HC_AVERAGE, HC_MEDIAN, HC_CENTROID,
       HC_FLEXIBLE_GROUP, HC_FLEXIBLE, HC_WARD, HC_MCQUITTY };

// getClusterEnum (src/rinterface.cpp): exact names, anything else single
// linkage -- including R's "flexible group", which the reference compares
// with "flexible_group".
int hc_method(const char *name) {
  static const char *names[] = {"complete", "wpgma", "average", "median", "centroid",
                                "flexible_group", "flexible", "ward", "mcquitty"};
  static const int ids[] = {HC_COMPLETE, HC_WPGMA, HC_AVERAGE, HC_MEDIAN, HC_CENTROID,
                            HC_FLEXIBLE_GROUP, HC_FLEXIBLE, HC_WARD, HC_MCQUITTY};
  for (int i = 0; i < 9; i++)
    if (name && std::strcmp(name, names[i]) == 0) return ids[i];
  return HC_SINGLE;
}

// (v1, c1) before (v2, c2): value, then index mod 32, then index; NaN never.
__device__ __forceinline__ bool hc_before(float v1, int c1, float v2, int c2) {
  if (v1 < v2) return true;
  if (!(v1 == v2)) return false;
  if ((c1 & 31) != (c2 & 31)) return (c1 & 31) < (c2 & 31);
  return c1 < c2;
}

// The linkage update of inst/cuda/hcluster.cu:108-401 for one column: top =
// the merged-away row's entry, bot = the kept row's, nr / np the kept and the
// merged-away cluster sizes (after the merge), nk the column's size, val the
// merge height.  Intrinsics keep every operation separately rounded.
__device__ float hc_update(int method, float top, float bot, float nr, float np, float nk,
                           float val, float lambda, float beta) {
  const float nq = __fsub_rn(nr, np);
  switch (method) {
    case HC_COMPLETE: return fmaxf(bot, top);
    case HC_WPGMA:
    case HC_MCQUITTY: return float(__ddiv_rn(double(__fadd_rn(bot, top)), 2.0));
    case HC_AVERAGE:
      return __fdiv_rn(__fadd_rn(__fmul_rn(top, np), __fmul_rn(bot, nq)), nr);
    case HC_MEDIAN:
      return float(__dsub_rn(__ddiv_rn(double(__fadd_rn(bot, top)), 2.0),
                             __ddiv_rn(double(val), 4.0)));
    case HC_CENTROID: {
      const float t1 = __fdiv_rn(__fadd_rn(__fmul_rn(top, np), __fmul_rn(bot, nq)), nr);
      const float t2 = __fdiv_rn(__fmul_rn(__fmul_rn(np, nq), val), __fmul_rn(nr, nr));
      return __fsub_rn(t1, t2);
    }
    case HC_FLEXIBLE_GROUP: {
      const double l1 = __dsub_rn(1.0, double(lambda));
      const double a = __dmul_rn(__dmul_rn(double(bot), l1), double(np));
      const double b = __dmul_rn(__dmul_rn(double(top), l1), double(nq));
      return float(__dadd_rn(__ddiv_rn(__dadd_rn(a, b), double(nr)),
                             double(__fmul_rn(beta, val))));
    }
    case HC_FLEXIBLE: {
      const double l1 = __dsub_rn(1.0, double(lambda));
      const double a = __dmul_rn(double(bot), l1), b = __dmul_rn(double(top), l1);
      return float(__dadd_rn(__ddiv_rn(__dadd_rn(a, b), 2.0), double(__fmul_rn(beta, val))));
    }
    case HC_WARD: {
      const float a = __fmul_rn(bot, __fadd_rn(np, nk)), b = __fmul_rn(top, __fadd_rn(nq, nk));
      float v = __fdiv_rn(__fsub_rn(__fadd_rn(a, b), __fmul_rn(val, nk)), __fadd_rn(nr, nk));
      if (isinf(v)) v = INFINITY;
      return v;
    }
    default: return fminf(bot, top);
  }
}

// Diagonal to +inf (convert_kernel), unit counts, and every row's minimum
// over columns 0..row: one warp per row, lanes strided by 32 as the reference.
__global__ void __launch_bounds__(256)
hc_init_kernel(float *__restrict__ D, int64_t n, float *__restrict__ count,
               float *__restrict__ minv, int *__restrict__ minc) {
  const unsigned FULL = 0xffffffffu;
  const int64_t row = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (row >= n) return;
  const int lane = threadIdx.x & 31;
  float *p = D + row * n;
  if (lane == 0) {
    p[row] = INFINITY;
    count[row] = 1.f;
  }
  __syncwarp();
  float v = INFINITY;
  int c = 0;
  for (int64_t col = lane; col <= row; col += 32) {
    const float t = p[col];
    if (hc_before(t, int(col), v, c)) { v = t; c = int(col); }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(FULL, v, o);
    const int oc = __shfl_xor_sync(FULL, c, o);
    if (hc_before(ov, oc, v, c)) { v = ov; c = oc; }
  }
  if (lane == 0) {
    minv[row] = v;
    minc[row] = c;
  }
}

// Block-wide smallest (v, c) by hc_before; every thread gets the result.
__device__ __forceinline__ void hc_block_min(float &v, int &c, float *sv, int *sc) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(FULL, v, o);
    const int oc = __shfl_xor_sync(FULL, c, o);
    if (hc_before(ov, oc, v, c)) { v = ov; c = oc; }
  }
  if (lane == 0) { sv[w] = v; sc[w] = c; }
  __syncthreads();
  if (w == 0) {
    v = sv[lane];
    c = sc[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(FULL, v, o);
      const int oc = __shfl_xor_sync(FULL, c, o);
      if (hc_before(ov, oc, v, c)) { v = ov; c = oc; }
    }
    if (lane == 0) { sv[32] = v; sc[32] = c; }
  }
  __syncthreads();
  v = sv[32];
  c = sc[32];
  __syncthreads();  // sv / sc may be reused at once
}

// All n - 1 merges in one CTA.
__global__ void __launch_bounds__(kHcThreads, 1)
hc_loop_kernel(float *__restrict__ D, int64_t n, int method, float lambda, float beta,
               float *__restrict__ count, float *__restrict__ minv, int *__restrict__ minc,
               float *__restrict__ scratch, int *__restrict__ list, int *__restrict__ sub,
               int *__restrict__ sup, float *__restrict__ val) {
  __shared__ float sv[33];
  __shared__ int sc[33];
  __shared__ int nlist;
  const int tid = threadIdx.x;
  for (int64_t it = 0; it + 1 < n; it++) {
    // the smallest kept minimum over the active rows (find_min2_kernel)
    float v = INFINITY;
    int rw = 0;
    for (int64_t x = tid; x < n; x += kHcThreads)
      if (count[x] > 0.f && hc_before(minv[x], int(x), v, rw)) { v = minv[x]; rw = int(x); }
    hc_block_min(v, rw, sv, sc);
    const int r = rw, c = minc[r];
    __syncthreads();  // every thread has read minc[r] before it changes
    if (tid == 0) {
      sub[it] = c;
      sup[it] = r;
      val[it] = v;
      // hcluster.cpp's statement order, which also fixes the sizes when an
      // all-infinite row makes c == r
      count[r] += count[c];
      count[c] = -count[c];
      sv[0] = count[r];
      sv[1] = -count[c];
      minv[c] = INFINITY;
      minc[c] = 0;
      nlist = 0;
    }
    __syncthreads();
    const float nr = sv[0], np = sv[1];
    __syncthreads();
    // the kept row's new entries
    for (int64_t col = tid; col < n; col += kHcThreads) {
      float nv;
      const float nk = count[col];
      if (col == c || col == r || (method == HC_WARD && nr == -nk))
        nv = INFINITY;
      else
        nv = hc_update(method, D[int64_t(c) * n + col], D[int64_t(r) * n + col], nr, np, nk, v,
                       lambda, beta);
      scratch[col] = nv;
    }
    __syncthreads();
    for (int64_t col = tid; col < n; col += kHcThreads) {
      const float nv = scratch[col];
      D[int64_t(r) * n + col] = nv;
      D[col * n + r] = nv;
      D[int64_t(c) * n + col] = INFINITY;
      D[col * n + c] = INFINITY;
    }
    __syncthreads();
    // kept minima: rows below c that lost their minimum's column, rows below
    // r that may gain the new (x, r)
    for (int64_t x = int64_t(c) + 1 + tid; x < n; x += kHcThreads) {
      if (x == r || !(count[x] > 0.f)) continue;
      const int mc = minc[x];
      if (mc == c || (x > r && mc == r)) {
        list[atomicAdd(&nlist, 1)] = int(x);
      } else if (x > r) {
        const float t = scratch[x];
        if (hc_before(t, r, minv[x], mc)) { minv[x] = t; minc[x] = r; }
      }
    }
    if (tid == 0) list[atomicAdd(&nlist, 1)] = r;
    __syncthreads();
    const int cnt = nlist;
    for (int e = 0; e < cnt; e++) {
      const int x = list[e];
      const float *p = D + int64_t(x) * n;
      float bv = INFINITY;
      int bc = 0;
      // lanes strided by 32 within each 1024-column stretch: the key order
      // is total, so any partition gives the reference's result
      for (int64_t col = tid; col <= x; col += kHcThreads) {
        const float t = p[col];
        if (hc_before(t, int(col), bv, bc)) { bv = t; bc = int(col); }
      }
      hc_block_min(bv, bc, sv, sc);
      if (tid == 0) {
        minv[x] = bv;
        minc[x] = bc;
      }
    }
    __syncthreads();
  }
}

// formatClustering (src/rinterface.cpp:241-290) in O(n alpha(n)).  The
// reference replaces, for each step i, every later entry equal to one of
// step i's two entries by i + 1; an entry therefore ends up as the last step
// before it whose cluster (the union of everything merged with the index so
// far) contains the index, or -(index + 1) if there is none.  Union-find
// keeps those clusters.  A point comes before a cluster, clusters in step
// order, two points as merged.  The order is the reference's depth-first
// walk (right subtree first, filled from the end), on an explicit stack.
// Returns false for a step list that is not a tree over len + 1 points.
bool format_clustering(int len, const int *sub, const int *sup, int *merge, int *order) {
  const int nidx = len + 1;
  for (int j = 0; j < len; j++)
    if (sub[j] < 0 || sub[j] >= nidx || sup[j] < 0 || sup[j] >= nidx) return false;
  std::vector<int> parent(static_cast<size_t>(nidx)), step(static_cast<size_t>(nidx), 0);
  for (int i = 0; i < nidx; i++) parent[size_t(i)] = i;
  auto find = [&](int x) {
    while (parent[size_t(x)] != x) {
      parent[size_t(x)] = parent[size_t(parent[size_t(x)])];
      x = parent[size_t(x)];
    }
    return x;
  };
  for (int j = 0; j < len; j++) {
    const int a = find(sub[j]), b = find(sup[j]);
    int va = step[size_t(a)] ? step[size_t(a)] : -(sub[j] + 1);
    int vb = step[size_t(b)] ? step[size_t(b)] : -(sup[j] + 1);
    if ((vb < 0 && va > 0) || (va > 0 && vb > 0 && va > vb)) std::swap(va, vb);
    merge[j] = va;
    merge[j + len] = vb;
    parent[size_t(a)] = b;
    step[size_t(b)] = j + 1;
  }
  if (len < 1) return true;
  // a leaf -(p + 1) is pushed as -(p + 2), a step s as s - 1: both "entry - 1"
  std::vector<int> stack;
  stack.reserve(size_t(2 * len + 2));
  int otop = len, visits = 0;
  stack.push_back(len - 1);
  while (!stack.empty()) {
    const int level = stack.back();
    stack.pop_back();
    if (++visits > len) return false;  // a step reached twice: not a tree
    stack.push_back(merge[level] - 1);
    stack.push_back(merge[level + len] - 1);
    while (!stack.empty() && stack.back() < 0) {
      if (otop < 0) return false;
      order[otop--] = -(stack.back() + 1);
      stack.pop_back();
    }
  }
  return true;
}

}  // namespace

// Clusters the full n x n matrix dD in place (it is overwritten); sub / sup
// / val (host, n - 1 each) receive the merges.
int hclust_device(float *dD, int64_t n, const char *method, int *sub, int *sup, float *val,
                  cudaStream_t s) {
  if (n < 2) return fail(GT_EINVAL, "must have n >= 2 objects to cluster");
  if (n > 2147483647LL / 2) return fail(GT_EINVAL, "too many objects");
  const int m = hc_method(method);
  void *pw = nullptr;
  const size_t bytes = size_t(n) * (3 * sizeof(float) + 2 * sizeof(int)) +
                       size_t(n - 1) * (2 * sizeof(int) + sizeof(float)) + 64;
  GT_TRY(ws_get(WS_SCRATCH3, bytes, &pw));
  float *count = static_cast<float *>(pw);
  float *minv = count + n, *scratch = minv + n;
  int *minc = reinterpret_cast<int *>(scratch + n), *list = minc + n;
  int *dsub = list + n, *dsup = dsub + (n - 1);
  float *dval = reinterpret_cast<float *>(dsup + (n - 1));
  {
    ProfScope prof("hclust", s);
    hc_init_kernel<<<unsigned(cdiv(n, 8)), 256, 0, s>>>(dD, n, count, minv, minc);
    hc_loop_kernel<<<1, kHcThreads, 0, s>>>(dD, n, m, 0.5f, 0.5f, count, minv, minc, scratch,
                                            list, dsub, dsup, dval);
    count_launch(2);
    GT_CUDA(cudaGetLastError());
  }
  GT_CUDA(cudaMemcpyAsync(sub, dsub, size_t(n - 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaMemcpyAsync(sup, dsup, size_t(n - 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaMemcpyAsync(val, dval, size_t(n - 1) * sizeof(float), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaStreamSynchronize(s));
  return GT_OK;
}

int hclust_format(int len, const int *sub, const int *sup, int *merge, int *order) {
  if (!format_clustering(len, sub, sup, merge, order))
    return fail(GT_EINVAL, "the merge steps do not form a tree over %d points", len + 1);
  return GT_OK;
}

}  // namespace gt

extern "C" int gt_hclust_format(int len, const int *sub, const int *sup, int *merge,
                                int *order) {
  gt::clear_error();
  if (len < 0 || (len > 0 && (!sub || !sup || !merge || !order)))
    return gt::fail(GT_EINVAL, "bad arguments");
  return gt::hclust_format(len, sub, sup, merge, order);
}

extern "C" int gt_hclust_device(float *d_dist, int64_t n, const char *method, int *merge,
                                int *order, float *height, void *stream) {
  gt::clear_error();
  if (!d_dist || !merge || !order || !height) return gt::fail(GT_EINVAL, "null pointer");
  std::vector<int> sub(size_t(n > 1 ? n - 1 : 1)), sup(sub.size());
  GT_TRY(gt::hclust_device(d_dist, n, method, sub.data(), sup.data(), height,
                           static_cast<cudaStream_t>(stream)));
  return gt::hclust_format(int(n - 1), sub.data(), sup.data(), merge, order);
}

extern "C" int gt_hclust(const float *dist, int64_t n, const char *method, int *merge, int *order,
                         float *height) {
  gt::clear_error();
  if (n < 2) return gt::fail(GT_EINVAL, "must have n >= 2 objects to cluster");
  if (!dist) return gt::fail(GT_EINVAL, "null pointer");
  cudaStream_t s = gt::lib_stream();
  void *dd = nullptr;
  const size_t bytes = size_t(n) * size_t(n) * 4;
  GT_TRY(gt::ws_get(gt::WS_IN_A, bytes, &dd));
  GT_CUDA(cudaMemcpyAsync(dd, dist, bytes, cudaMemcpyHostToDevice, s));
  return gt_hclust_device(static_cast<float *>(dd), n, method, merge, order, height, s);
}

extern "C" int gt_distclust(const float *points, int64_t n, int64_t dim, int dist_method,
                            const char *method, int *merge, int *order, float *height) {
  gt::clear_error();
  if (n < 2) return gt::fail(GT_EINVAL, "must have n >= 2 objects to cluster");
  if (!points) return gt::fail(GT_EINVAL, "null pointer");
  cudaStream_t s = gt::lib_stream();
  void *dp = nullptr, *dd = nullptr;
  const size_t pbytes = size_t(n) * size_t(dim) * 4, dbytes = size_t(n) * size_t(n) * 4;
  GT_TRY(gt::ws_get(gt::WS_IN_A, pbytes, &dp));
  GT_TRY(gt::ws_get(gt::WS_OUT0, dbytes, &dd));
  GT_CUDA(cudaMemcpyAsync(dp, points, pbytes, cudaMemcpyHostToDevice, s));
  // the distance matrix never leaves the device (distanceLeaveOnGpu)
  GT_TRY(gt_distances_device(static_cast<float *>(dp), n, dim, static_cast<float *>(dd),
                             GT_LAYOUT_FULL, dist_method, 2.f, s));
  return gt_hclust_device(static_cast<float *>(dd), n, method, merge, order, height, s);
}
