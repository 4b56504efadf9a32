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
// are the reference's.  All merges run in one launch of a thread-block
// cluster (up to 16 CTAs exchanging their candidates through distributed
// shared memory, one hardware cluster barrier per merge), after a multi-CTA
// kernel that initialises the kept minima.  The linkage expressions are
// evaluated as the reference writes them (float, with its double
// promotions), each operation rounded on its own; the reference compiles
// them with NVRTC --use_fast_math, so its own rounding is the compiler's
// choice of contractions.
#include "common.cuh"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace gt {

namespace {

constexpr int kHcThreads = 512;
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

__device__ __forceinline__ int64_t cdiv_d(int64_t a, int64_t b) { return (a + b - 1) / b; }

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

// Diagonal to +inf (convert_kernel) and every row's minimum
// over columns 0..row: one warp per row, lanes strided by 32 as the reference.
__global__ void __launch_bounds__(256)
hc_init_kernel(float *__restrict__ D, int64_t n, float *__restrict__ minv,
               int *__restrict__ minc) {
  const unsigned FULL = 0xffffffffu;
  const int64_t row = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (row >= n) return;
  const int lane = threadIdx.x & 31;
  float *p = D + row * n;
  if (lane == 0) p[row] = INFINITY;
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

// *asym = 1 unless D[i][j] == D[j][i] for every i, j (NaN counts as a
// difference): 32 x 32 tiles of the lower triangle against their transposes,
// both read coalesced through shared memory.
__global__ void __launch_bounds__(256)
hc_symmetry_kernel(const float *__restrict__ D, int64_t n, int *__restrict__ asym) {
  __shared__ float t[32][33];
  const int64_t nt = (n + 31) / 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int64_t b = blockIdx.x; b < nt * (nt + 1) / 2; b += gridDim.x) {
    // tile (bi, bj), bj <= bi, from the triangular index b
    int64_t bi = int64_t((sqrt(8.0 * double(b) + 1.0) - 1.0) / 2.0);
    while (bi * (bi + 1) / 2 > b) bi--;
    while ((bi + 1) * (bi + 2) / 2 <= b) bi++;
    const int64_t bj = b - bi * (bi + 1) / 2;
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {  // the transposed tile (bj, bi), row by row
      const int64_t row = bj * 32 + k, col = bi * 32 + tx;
      t[k][tx] = (row < n && col < n) ? D[row * n + col] : 0.f;
    }
    __syncthreads();
    bool diff = false;
    for (int k = ty; k < 32; k += 8) {
      const int64_t row = bi * 32 + k, col = bj * 32 + tx;
      if (row < n && col < n) diff |= !(D[row * n + col] == t[tx][k]);
    }
    if (__syncthreads_or(diff) && threadIdx.x == 0) atomicExch(asym, 1);
  }
}

// A candidate minimum: value, the index its ties are ordered by (column for
// a row's minimum, row for the smallest row minimum) and the other index.
struct alignas(16) HcCand {
  float v;
  int k;
  int a;
  int pad;
};
// What a CTA publishes after each merge: the smallest kept minimum of its
// rows (r and c excluded) and its part of the kept row r's new minimum.
struct alignas(32) HcSlot {
  HcCand x, rm;
};

constexpr int kHcWarps = kHcThreads / 32;
constexpr int kHcRescan = 2;  // rows scanned again within the step's reduction (hc_scan_rows: two)
constexpr int kHcCands = 2 + kHcRescan;
constexpr int kHcPre = 4;     // owned columns per thread loaded at once
constexpr int kHcMaxCtas = 16;

__device__ __forceinline__ HcCand hc_cand(float v, int k, int a) { return HcCand{v, k, a, 0}; }
__device__ __forceinline__ HcCand hc_none() { return HcCand{INFINITY, 0, 0, 0}; }
__device__ __forceinline__ void hc_take(HcCand &best, const HcCand &o) {
  if (hc_before(o.v, o.k, best.v, best.k)) best = o;
}
// Order-preserving keys: hc_before(v1, c1, v2, c2) <=> (vkey(v1), ikey(c1)) <
// (vkey(v2), ikey(c2)) lexicographically, for non-NaN values (-0 and +0 tie;
// a NaN, never chosen, maps above +inf).
__device__ __forceinline__ unsigned hc_vkey(float v) {
  if (v != v) return 0xffffffffu;
  const unsigned u = __float_as_uint(v == 0.f ? 0.f : v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned hc_ikey(int k) {
  const unsigned u = unsigned(k);
  return ((u & 31u) << 27) | (u >> 5);
}
// Warp-wide smallest candidate, for every lane: two redux.sync on the keys.
__device__ __forceinline__ void hc_warp_min(HcCand &c) {
  const unsigned FULL = 0xffffffffu;
  const unsigned vk = hc_vkey(c.v), ik = hc_ikey(c.k);
  const unsigned mv = __reduce_min_sync(FULL, vk);
  const unsigned mi = __reduce_min_sync(FULL, vk == mv ? ik : 0xffffffffu);
  const int src = __ffs(__ballot_sync(FULL, vk == mv && ik == mi)) - 1;
  c.v = __shfl_sync(FULL, c.v, src);
  c.k = __shfl_sync(FULL, c.k, src);
  c.a = __shfl_sync(FULL, c.a, src);
}

// Block-wide smallest of c[0..nc) (nc block-uniform); every thread gets the
// results.  s: kHcCands * (kHcWarps + 1) candidates, alternated between
// consecutive calls (two barriers apart, so no barrier is needed after).
__device__ __forceinline__ void hc_block_min(HcCand (&c)[kHcCands], int nc, HcCand *s) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kHcCands; j++)
    if (j < nc) hc_warp_min(c[j]);
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < kHcCands; j++)
      if (j < nc) s[j * kHcWarps + w] = c[j];
  }
  __syncthreads();
  if (w < nc) {
    HcCand t = lane < kHcWarps ? s[w * kHcWarps + lane] : hc_none();
    hc_warp_min(t);
    if (lane == 0) s[kHcCands * kHcWarps + w] = t;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kHcCands; j++)
    if (j < nc) c[j] = s[kHcCands * kHcWarps + j];
}

// Thread-block cluster primitives: this CTA's rank, the cluster barrier
// (release / acquire), and accesses to another CTA's shared memory.
__device__ __forceinline__ int hc_cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return int(r);
}
__device__ __forceinline__ void hc_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned hc_dsmem(const void *p, int rank) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(p));
  unsigned out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(a), "r"(rank));
  return out;
}
__device__ __forceinline__ void hc_st_dsmem4(unsigned addr, float4 v) {
  asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w)
               : "memory");
}
__device__ __forceinline__ float hc_ld_dsmem(unsigned addr) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
  return v;
}

// This thread's part of the minima of rows row0 and row1 (row1 < 0: none)
// over columns 0..row, columns c and r left out (the caller accounts for
// them).  The two rows' loads are issued together; read through L2.
__device__ __forceinline__ void hc_scan_rows(const float *__restrict__ D, int64_t n, int64_t row0,
                                             int64_t row1, int c, int r, HcCand &b0, HcCand &b1) {
  const int tid = threadIdx.x;
  const float4 inf4 = make_float4(INFINITY, INFINITY, INFINITY, INFINITY);
  const float *p0 = D + row0 * n, *p1 = D + (row1 < 0 ? 0 : row1) * n;
  const int64_t len0 = row0 + 1, len1 = row1 + 1;  // len1 = 0 for no row
  auto head = [&](const float *p, int64_t len) {
    const int64_t mis = int64_t(reinterpret_cast<uintptr_t>(p) >> 2) & 3;
    return len < ((4 - mis) & 3) ? len : ((4 - mis) & 3);
  };
  const int64_t h0 = head(p0, len0), h1 = head(p1, len1);
  const int64_t m0 = (len0 - h0) >> 2, m1 = (len1 - h1) >> 2;
  const float4 *q0 = reinterpret_cast<const float4 *>(p0 + h0);
  const float4 *q1 = reinterpret_cast<const float4 *>(p1 + h1);
  auto take = [&](HcCand &best, float t, int64_t col) {
    if (col != c && col != r) hc_take(best, hc_cand(t, int(col), 0));
  };
  if (tid < h0) take(b0, __ldcg(p0 + tid), tid);
  if (tid < h1) take(b1, __ldcg(p1 + tid), tid);
  const int64_t mm = m0 > m1 ? m0 : m1;
  for (int64_t base = 0; base < mm; base += 4 * kHcThreads) {
    float4 f0[4], f1[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int64_t j = base + u * kHcThreads + tid;
      f0[u] = j < m0 ? __ldcg(q0 + j) : inf4;
      f1[u] = j < m1 ? __ldcg(q1 + j) : inf4;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int64_t j = base + u * kHcThreads + tid;
      if (j < m0) {
        const int64_t c0 = h0 + 4 * j;
        take(b0, f0[u].x, c0);
        take(b0, f0[u].y, c0 + 1);
        take(b0, f0[u].z, c0 + 2);
        take(b0, f0[u].w, c0 + 3);
      }
      if (j < m1) {
        const int64_t c1 = h1 + 4 * j;
        take(b1, f1[u].x, c1);
        take(b1, f1[u].y, c1 + 1);
        take(b1, f1[u].z, c1 + 2);
        take(b1, f1[u].w, c1 + 3);
      }
    }
  }
  const int64_t t0 = h0 + 4 * m0 + tid, t1 = h1 + 4 * m1 + tid;
  if (t0 < len0) take(b0, __ldcg(p0 + t0), t0);
  if (t1 < len1) take(b1, __ldcg(p1 + t1), t1);
}

// Writes this CTA's slot into slot [buf][b] of every CTA of the cluster.
__device__ __forceinline__ void hc_push(HcSlot (*slots)[kHcMaxCtas], int buf, int b, int G,
                                        const HcCand &x, const HcCand &rm) {
  const int tid = threadIdx.x;
  if (tid < G) {
    const unsigned a = hc_dsmem(&slots[buf][b], tid);
    hc_st_dsmem4(a, make_float4(x.v, __int_as_float(x.k), __int_as_float(x.a), 0.f));
    hc_st_dsmem4(a + 16, make_float4(rm.v, __int_as_float(rm.k), __int_as_float(rm.a), 0.f));
  }
}

// All n - 1 merges in one thread-block cluster of G <= 16 CTAs (one launch,
// its CTAs co-scheduled by the hardware).  CTA b owns the indices [lo, hi) =
// [n b / G, n (b + 1) / G): their columns in each update and their rows'
// kept minima, in its shared memory.  Counts: with REP every CTA keeps all n
// (updated by each merge), otherwise each CTA its own, read by the others
// from its shared memory.  Step t:
//   A. every warp reduces the G slots that the CTAs wrote into this CTA's
//      shared memory in the previous step to the merge (v, r, c) and to the
//      previous kept row's new minimum;
//   B. list the owned rows whose minimum sat in column c or r; load rows c
//      and r at the owned columns and the listed rows (columns c and r left
//      out) together; write the new row / column r, row / column c = +inf;
//      compare the other owned rows' kept minima with the new (x, r); one
//      block reduction gives the owned rows' smallest minimum, the owned part
//      of row r's minimum and the listed rows' minima;
//   C. write the slot into every CTA (double-buffered) and pass the cluster
//      barrier (release / acquire), which also orders the D writes before
//      any other CTA's reads of them (through L2).
template <bool REP>
__global__ void __launch_bounds__(kHcThreads, 1)
hc_loop_kernel(float *__restrict__ D, int64_t n, int method, float lambda, float beta,
               const float *__restrict__ minv0, const int *__restrict__ minc0,
               const int *__restrict__ asym, int *__restrict__ sub, int *__restrict__ sup,
               float *__restrict__ val) {
  extern __shared__ __align__(16) float hc_smem[];
  __shared__ HcSlot s_slots[2][kHcMaxCtas];
  __shared__ HcCand sred[2][kHcCands * (kHcWarps + 1)];
  __shared__ int nlist;
  const int G = int(gridDim.x), b = hc_cluster_rank(), tid = threadIdx.x, lane = tid & 31;
  const int64_t lo = n * b / G, hi = n * (b + 1) / G, smax = cdiv_d(n, G);
  float *s_minv = hc_smem;
  int *s_minc = reinterpret_cast<int *>(s_minv + smax);
  int *s_list = s_minc + smax;
  float *s_cnt = reinterpret_cast<float *>(s_list + smax);  // n (REP) or smax entries
  auto cnt_own = [&](int64_t i) -> float & { return REP ? s_cnt[i] : s_cnt[i - lo]; };
  int sb = 0;

  HcCand cand[kHcCands];
#pragma unroll
  for (int j = 0; j < kHcCands; j++) cand[j] = hc_none();
  if (REP) {
    for (int64_t i = tid; i < n; i += kHcThreads) s_cnt[i] = 1.f;
  }
  for (int64_t i = lo + tid; i < hi; i += kHcThreads) {
    const float mv = minv0[i];
    const int mc = minc0[i];
    s_minv[i - lo] = mv;
    s_minc[i - lo] = mc;
    if (!REP) s_cnt[i - lo] = 1.f;
    hc_take(cand[0], hc_cand(mv, int(i), mc));
  }
  if (tid == 0) nlist = 0;
  hc_block_min(cand, 2, sred[sb]);
  sb ^= 1;
  hc_cluster_sync();  // every CTA has started before shared memory is written remotely
  hc_push(s_slots, 0, b, G, cand[0], cand[1]);
  hc_cluster_sync();
  int pr = -1, pc = -1;
  float prf = 0.f, pcf = 0.f;  // the previous merge's rows and their counts after it
  // a symmetric matrix stays symmetric (every update writes both halves)
  const bool symmetric = *asym == 0;

  for (int64_t it = 0; it + 1 < n; it++) {
    // A. the merge
    const int par = int(it & 1);
    HcCand x = hc_none(), y = hc_none();
    if (lane < G) {
      const HcSlot &sl = s_slots[par][lane];
      x = sl.x;
      y = sl.rm;
    }
    hc_warp_min(x);
    hc_warp_min(y);
    if (pr >= 0 && prf > 0.f) hc_take(x, hc_cand(y.v, pr, y.k));
    const float v = x.v;
    const int r = x.k, c = x.a;
    auto cnt_any = [&](int64_t i) -> float {
      if (REP) return s_cnt[i];
      if (i == pc) return pcf;  // their owners store these now
      if (i == pr) return prf;
      const int o = int(((i + 1) * G - 1) / n);
      return o == b ? s_cnt[i - lo] : hc_ld_dsmem(hc_dsmem(&s_cnt[i - n * o / G], o));
    };
    // counts as src/hcluster.cpp updates them (cnt[r] += cnt[c]; cnt[c] = -cnt[c])
    const float cr0 = cnt_any(r), cc0 = cnt_any(c);
    const float a = cr0 + cc0;
    const float cfin = -(c == r ? a : cc0);
    const float rfin = c == r ? cfin : a;
    const float nr = rfin, np = -cfin;
    if (tid == 0) {
      if (pr >= lo && pr < hi) {
        s_minv[pr - lo] = y.v;
        s_minc[pr - lo] = y.k;
        if (!REP) s_cnt[pr - lo] = prf;
      }
      if (!REP && pc >= lo && pc < hi) s_cnt[pc - lo] = pcf;  // after pr: pc == pr keeps pcf
      if (b == 0) {
        sub[it] = c;
        sup[it] = r;
        val[it] = v;
      }
    }

    // B. rows to scan again (pr's values from registers: stored just now).
    // Single linkage on a symmetric matrix: the new (i, r) is min(old (i, r),
    // old (i, c)), never above the old minimum's entry; when the row's
    // minimum sat in column r it stays there, and when it sat in column c
    // with r ordered before c (r <= i), (i, r) is the new minimum: no scan.
    const bool single_short = method == HC_SINGLE && symmetric && c != r;
    const bool r_before_c = hc_before(0.f, r, 0.f, c);
    auto rescan = [&](int64_t i, int mc) {
      if (!(mc == c || (i > r && mc == r))) return false;
      if (single_short && (mc == r || (r <= i && r_before_c))) return false;
      return true;
    };
    for (int64_t i = lo + tid; i < hi; i += kHcThreads) {
      if (i <= c || i == r) continue;
      const float ci = (!REP && i == pc) ? pcf : (!REP && i == pr) ? prf : cnt_own(i);
      if (!(ci > 0.f)) continue;
      const int mc = i == pr ? y.k : s_minc[i - lo];
      if (rescan(i, mc)) s_list[atomicAdd(&nlist, 1)] = int(i);
    }
    __syncthreads();
    const int L = nlist, L1 = L < kHcRescan ? L : kHcRescan;
#pragma unroll
    for (int j = 0; j < kHcCands; j++) cand[j] = hc_none();
    for (int64_t base = lo; base < hi; base += int64_t(kHcPre) * kHcThreads) {
      float top[kHcPre], bot[kHcPre];
#pragma unroll
      for (int u = 0; u < kHcPre; u++) {
        const int64_t i = base + u * kHcThreads + tid;
        top[u] = i < hi ? __ldcg(D + int64_t(c) * n + i) : 0.f;
        bot[u] = i < hi ? __ldcg(D + int64_t(r) * n + i) : 0.f;
      }
      if (base == lo && L1 > 0)
        hc_scan_rows(D, n, s_list[0], L1 > 1 ? s_list[1] : -1, c, r, cand[2], cand[3]);
#pragma unroll
      for (int u = 0; u < kHcPre; u++) {
        const int64_t i = base + u * kHcThreads + tid;
        if (i >= hi) continue;
        const float nk = cnt_own(i);
        float nv;
        if (i == c || i == r || (method == HC_WARD && nr == -nk))
          nv = INFINITY;
        else
          nv = hc_update(method, top[u], bot[u], nr, np, nk, v, lambda, beta);
        if (i <= r) hc_take(cand[1], hc_cand(nv, int(i), 0));
        D[int64_t(r) * n + i] = nv;
        D[i * n + r] = nv;
        D[int64_t(c) * n + i] = INFINITY;
        D[i * n + c] = INFINITY;
        if (i == r || i == c || !(nk > 0.f)) continue;
        float mv = s_minv[i - lo];
        int mc = s_minc[i - lo];
        if (i > c && rescan(i, mc)) {
#pragma unroll
          for (int e = 0; e < kHcRescan; e++)
            if (e < L1 && s_list[e] == i && r <= i) hc_take(cand[2 + e], hc_cand(nv, r, 0));
        } else {
          if (i > c && mc == c) {  // single linkage, see above: (i, r) is the minimum
            mv = nv;
            mc = r;
            s_minv[i - lo] = mv;
            s_minc[i - lo] = mc;
          } else if (i > r && hc_before(nv, r, mv, mc)) {
            mv = nv;
            mc = r;
            s_minv[i - lo] = mv;
            s_minc[i - lo] = mc;
          }
          hc_take(cand[0], hc_cand(mv, int(i), mc));
        }
      }
    }
    hc_block_min(cand, 2 + L1, sred[sb]);
    sb ^= 1;
    HcCand best = cand[0];
    const HcCand rmin = cand[1];
#pragma unroll
    for (int e = 0; e < kHcRescan; e++) {
      if (e < L1) {
        const int row = s_list[e];
        if (tid == 0) {
          s_minv[row - lo] = cand[2 + e].v;
          s_minc[row - lo] = cand[2 + e].k;
        }
        hc_take(best, hc_cand(cand[2 + e].v, row, cand[2 + e].k));
      }
    }
    for (int e0 = kHcRescan; e0 < L; e0 += kHcRescan) {  // more rows: further rounds
#pragma unroll
      for (int j = 0; j < kHcCands; j++) cand[j] = hc_none();
      hc_scan_rows(D, n, s_list[e0], e0 + 1 < L ? s_list[e0 + 1] : -1, c, r, cand[0], cand[1]);
#pragma unroll
      for (int e = 0; e < kHcRescan; e++) {
        if (e0 + e < L) {
          const int row = s_list[e0 + e];
          // (row, r) was written by this CTA in this step
          if (tid == 0 && r <= row) hc_take(cand[e], hc_cand(__ldcg(D + int64_t(row) * n + r), r, 0));
        }
      }
      const int m = L - e0 < kHcRescan ? L - e0 : kHcRescan;
      hc_block_min(cand, m, sred[sb]);
      sb ^= 1;
#pragma unroll
      for (int e = 0; e < kHcRescan; e++) {
        if (e < m) {
          const int row = s_list[e0 + e];
          if (tid == 0) {
            s_minv[row - lo] = cand[e].v;
            s_minc[row - lo] = cand[e].k;
          }
          hc_take(best, hc_cand(cand[e].v, row, cand[e].k));
        }
      }
    }

    // C. publish
    if (tid == 0) {
      nlist = 0;
      if (REP) {
        s_cnt[r] = rfin;
        s_cnt[c] = cfin;  // after r: c == r keeps cfin
      }
    }
    hc_push(s_slots, par ^ 1, b, G, best, rmin);
    pr = r;
    pc = c;
    prf = rfin;
    pcf = cfin;
    hc_cluster_sync();
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
  int m = hc_method(method);
  // one cluster of up to 16 CTAs, at least ~64 indices each
  int G = int(std::min<int64_t>(kHcMaxCtas, cdiv(n, 64)));
  if (const char *e = std::getenv("GT_HCLUST_CTAS")) G = std::max(1, std::min(G, std::atoi(e)));
  // shared memory: kept minima, rescan list, counts (all n when they fit)
  const size_t cap = size_t(200) * 1024;
  auto smem_of = [&](int g, bool rep) {
    return size_t(cdiv(n, g)) * 12 + (rep ? size_t(n) : size_t(cdiv(n, g))) * 4;
  };
  bool rep = smem_of(G, true) <= cap;
  if (const char *e = std::getenv("GT_HCLUST_COUNTS"))  // "owned": the large-n layout at any n
    if (std::strcmp(e, "owned") == 0) rep = false;
  auto kern = rep ? hc_loop_kernel<true> : hc_loop_kernel<false>;
  GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  for (;; G /= 2) {  // the largest cluster that the device can place
    const size_t smem = G >= 1 ? smem_of(G, rep) : 0;
    if (G < 1 || smem > cap)
      return fail(GT_EUNSUPPORTED, "no thread-block cluster large enough for %lld objects",
                  static_cast<long long>(n));
    GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(kHcThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    GT_CUDA(cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg));
    if (nclusters >= 1) break;
  }
  void *pw = nullptr;
  const size_t bytes = 256 + size_t(n) * 8 + size_t(n - 1) * 12 + 256;
  GT_TRY(ws_get(WS_SCRATCH3, bytes, &pw));
  int *asym = static_cast<int *>(pw);
  float *minv = reinterpret_cast<float *>(static_cast<char *>(pw) + 256);
  int *minc = reinterpret_cast<int *>(minv + n);
  int *dsub = minc + n, *dsup = dsub + (n - 1);
  float *dval = reinterpret_cast<float *>(dsup + (n - 1));
  {
    ProfScope prof("hclust", s);
    // single linkage's shortcut needs a symmetric matrix (R's as.matrix(dist)
    // is); other methods never look at the flag
    GT_CUDA(cudaMemsetAsync(asym, 0, sizeof(int), s));
    if (m == HC_SINGLE) {
      const int64_t tiles = cdiv(n, 32) * (cdiv(n, 32) + 1) / 2;
      hc_symmetry_kernel<<<unsigned(std::min<int64_t>(tiles, int64_t(sm_count()) * 8)), 256, 0,
                           s>>>(dD, n, asym);
      count_launch();
    } else {
      GT_CUDA(cudaMemsetAsync(asym, 0xff, sizeof(int), s));
    }
    hc_init_kernel<<<unsigned(cdiv(n, 8)), 256, 0, s>>>(dD, n, minv, minc);
    GT_CUDA(cudaGetLastError());
    GT_CUDA(cudaLaunchKernelEx(&cfg, kern, dD, n, m, 0.5f, 0.5f,
                               static_cast<const float *>(minv), static_cast<const int *>(minc),
                               static_cast<const int *>(asym), dsub, dsup, dval));
    count_launch(2);
  }
  GT_CUDA(cudaMemcpyAsync(sub, dsub, size_t(n - 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaMemcpyAsync(sup, dsup, size_t(n - 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaMemcpyAsync(val, dval, size_t(n - 1) * sizeof(float), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaStreamSynchronize(s));
  return GT_OK;
}

int hclust_format(int len, const int *sub, const int *sup, int *merge, int *order) {
  try {
    if (!format_clustering(len, sub, sup, merge, order))
      return fail(GT_EINVAL, "the merge steps do not form a tree over %d points", len + 1);
  } catch (const std::bad_alloc &) {
    return fail(GT_ENOMEM, "host memory for the merge formatting");
  }
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
  std::vector<int> sub, sup;
  try {
    sub.resize(size_t(n > 1 ? n - 1 : 1));
    sup.resize(sub.size());
  } catch (const std::bad_alloc &) {
    return gt::fail(GT_ENOMEM, "host memory for %lld merge steps", static_cast<long long>(n));
  }
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
  gt::StreamSyncGuard guard(s);
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
  gt::StreamSyncGuard guard(s);
  void *dp = nullptr, *dd = nullptr;
  const size_t pbytes = size_t(n) * size_t(dim) * 4, dbytes = size_t(n) * size_t(n) * 4;
  GT_TRY(gt::ws_get(gt::WS_IN_A, pbytes, &dp));
  GT_TRY(gt::ws_get(gt::WS_OUT0, dbytes, &dd));
  GT_CUDA(cudaMemcpyAsync(dp, points, pbytes, cudaMemcpyHostToDevice, s));
  // the distance matrix never leaves the device (distanceLeaveOnGpu)
  GT_TRY(gt_distances_device(static_cast<float *>(dp), n, dim, static_cast<float *>(dd),
                             GT_LAYOUT_FULL, dist_method, 2.f, s));
  bool failed = false;
  GT_TRY(gt::device_error_check(s, &failed));
  if (failed) return gt::fail(GT_ETIMEOUT, "a tensor-core kernel wait timed out");
  return gt_hclust_device(static_cast<float *>(dd), n, method, merge, order, height, s);
}
