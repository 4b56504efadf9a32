// batch.cu -- plans for batches of independent correlation problems: many
// uneven gpuCor problems computed by one persistent launch per phase,
// replayed from a captured CUDA graph.  No counterpart in the reference,
// which handles one problem per .C call (src/correlation.cpp:66-161,
// src/kendall.cpp:13-55).
//
// A plan fixes the problems (pointers and shapes), owns its device buffers
// (descriptors, operand planes or pair masks, per-CTA tile lists), balances
// the tiles over the CTAs on the host (longest-processing-time first: tiles
// sorted by cost, each given to the least loaded CTA), and captures the
// launches into a graph that gt_batch_plan_launch replays.
#include "common.cuh"
#include "kernels.cuh"

#include <sys/stat.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <functional>
#include <queue>
#include <vector>

struct gt_batch_plan {
  int kind = 0;  // 0 = pearson, 1 = kendall
  int device = 0;
  std::vector<void *> bufs;
  std::function<int(cudaStream_t)> run;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t tiles = 0, ctas = 0;
  int *err = nullptr;  // the device error word, when the plan runs tensor-core kernels
  double config_ms = 0.0;
  char config[160] = {0};
};

namespace gt {

namespace {

int plan_alloc(gt_batch_plan *p, size_t bytes, void **ptr) {
  if (bytes == 0) bytes = 256;
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(GT_ENOMEM, "batch plan: %zu bytes unavailable: %s", bytes, cudaGetErrorString(e));
  }
  p->bufs.push_back(q);
  *ptr = q;
  return GT_OK;
}

template <class T>
int plan_upload(gt_batch_plan *p, const std::vector<T> &v, T **dptr) {
  void *q = nullptr;
  GT_TRY(plan_alloc(p, v.size() * sizeof(T), &q));
  if (!v.empty()) GT_CUDA(cudaMemcpy(q, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  *dptr = static_cast<T *>(q);
  return GT_OK;
}

// Longest-processing-time-first assignment of tiles (given their costs) to
// `ncta` CTAs; returns the tile ids grouped by CTA and the group offsets.
void lpt_assign(const std::vector<int64_t> &cost, int64_t ncta, std::vector<int64_t> &tiles,
                std::vector<int64_t> &off) {
  const int64_t nt = int64_t(cost.size());
  std::vector<int64_t> order(nt);
  for (int64_t i = 0; i < nt; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return cost[a] > cost[b]; });
  using Item = std::pair<int64_t, int64_t>;  // (load, cta)
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
  for (int64_t c = 0; c < ncta; c++) heap.push({0, c});
  std::vector<std::vector<int64_t>> lists(ncta);
  for (int64_t t : order) {
    Item it = heap.top();
    heap.pop();
    lists[it.second].push_back(t);
    it.first += cost[t] > 0 ? cost[t] : 1;
    heap.push(it);
  }
  tiles.clear();
  off.assign(ncta + 1, 0);
  for (int64_t c = 0; c < ncta; c++) {
    off[c] = int64_t(tiles.size());
    tiles.insert(tiles.end(), lists[c].begin(), lists[c].end());
  }
  off[ncta] = int64_t(tiles.size());
}

// Runs the plan once eagerly (validates it), then captures it into a graph.
int plan_finalize(gt_batch_plan *p, int flags) {
  cudaStream_t s = nullptr;
  GT_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  int st = p->run(s);
  if (st == GT_OK) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = fail(GT_ECUDA, "batch plan first run: %s", cudaGetErrorString(e));
  }
  if (st == GT_OK && p->err) {
    bool failed = false;
    st = device_error_check(s, &failed);
    if (st == GT_OK && failed)
      st = fail(GT_ETIMEOUT, "batch plan first run: a tensor-core kernel wait timed out");
  }
  if (st == GT_OK && !(flags & GT_BATCH_NO_GRAPH)) {
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      st = p->run(s);
      cudaGraph_t g = nullptr;
      e = cudaStreamEndCapture(s, &g);
      if (st == GT_OK && e == cudaSuccess) {
        p->graph = g;
        e = cudaGraphInstantiate(&p->exec, g, 0);
        if (e != cudaSuccess) st = fail(GT_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
      } else if (st == GT_OK) {
        st = fail(GT_ECUDA, "graph capture: %s", cudaGetErrorString(e));
      }
    } else {
      st = fail(GT_ECUDA, "begin capture: %s", cudaGetErrorString(e));
    }
  }
  cudaStreamDestroy(s);
  return st;
}

void plan_free(gt_batch_plan *p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  for (void *b : p->bufs) cudaFree(b);
  delete p;
}

}  // namespace

int kendall_batch_plan(const gt_kendall_problem *probs, int64_t count, int flags,
                       gt_batch_plan **out) {
  if (count < 0 || (count > 0 && !probs)) return fail(GT_EINVAL, "bad problem list");
  auto *p = new gt_batch_plan();
  p->kind = 1;
  cudaGetDevice(&p->device);
  std::vector<KendallBatchProblem> hp;
  std::vector<int64_t> var_prefix{0}, tile_prefix{0}, tile_cost;
  int64_t mask_words = 0, vars = 0;
  for (int64_t i = 0; i < count; i++) {
    const gt_kendall_problem &q = probs[i];
    if (q.p < 0 || q.n < 0 || q.n > 65536) {
      plan_free(p);
      return fail(GT_EINVAL, "problem %lld: bad shape (p=%lld, n=%lld)", (long long)i,
                  (long long)q.p, (long long)q.n);
    }
    if (q.p == 0) continue;
    if (!q.X || !q.out) {
      plan_free(p);
      return fail(GT_EINVAL, "problem %lld: null pointer", (long long)i);
    }
    KendallBatchProblem b;
    b.X = q.X;
    b.p = q.p;
    b.n = q.n;
    b.Dr = q.n / 2;
    b.Wn = cdiv(q.n, 32);
    b.K = b.Dr * b.Wn;
    b.mask_off = mask_words;
    b.var_off = vars;
    b.out = q.out;
    hp.push_back(b);
    mask_words += b.K * b.p;
    vars += b.p;
    var_prefix.push_back(vars);
    const int64_t m = cdiv(q.p, 64), nt = m * (m + 1) / 2;
    tile_prefix.push_back(tile_prefix.back() + nt);
    for (int64_t t = 0; t < nt; t++) tile_cost.push_back(b.K + 16);
  }
  const int64_t nprob = int64_t(hp.size());
  const int64_t ntiles = tile_prefix.back();
  int64_t ncta = int64_t(sm_count()) * 6;
  if (ncta > ntiles) ncta = ntiles;
  std::vector<int64_t> cta_tiles, cta_off;
  lpt_assign(tile_cost, ncta, cta_tiles, cta_off);
  KendallBatchProblem *d_probs = nullptr;
  int64_t *d_vp = nullptr, *d_tp = nullptr, *d_ct = nullptr, *d_co = nullptr;
  void *d_m = nullptr, *d_t = nullptr;
  int st = GT_OK;
  if ((st = plan_upload(p, hp, &d_probs)) || (st = plan_upload(p, var_prefix, &d_vp)) ||
      (st = plan_upload(p, tile_prefix, &d_tp)) || (st = plan_upload(p, cta_tiles, &d_ct)) ||
      (st = plan_upload(p, cta_off, &d_co)) ||
      (st = plan_alloc(p, size_t(mask_words) * sizeof(uint2), &d_m)) ||
      (st = plan_alloc(p, size_t(vars) * 16, &d_t))) {  // untied counts, then their roots
    plan_free(p);
    return st;
  }
  p->tiles = ntiles;
  p->ctas = ncta;
  std::snprintf(p->config, sizeof(p->config), "kendall 64x64 tiles, %lld ctas", (long long)ncta);
  auto *masks = static_cast<uint2 *>(d_m);
  auto *T = static_cast<unsigned long long *>(d_t);
  p->run = [=](cudaStream_t s) {
    return kendall_batch_launch(d_probs, d_vp, nprob, vars, d_tp, d_ct, d_co, ncta, masks, T, s);
  };
  st = plan_finalize(p, flags);
  if (st != GT_OK) {
    plan_free(p);
    return st;
  }
  *out = p;
  return GT_OK;
}

// ----------------------------------------------------------------- autotuner
// Candidate tile configurations of the batched Pearson contraction, timed on
// the batch itself when GT_BATCH_AUTOTUNE is given; the winner is cached in a
// small text file (GT_AUTOTUNE_CACHE, default ~/.cache/gputools_gb300/
// autotune.txt) keyed by the batch's shape, and reused by later plans.
struct TileConfig {
  int bk;
  int64_t chunk;
  const char *name;
};

const TileConfig kX3Configs[] = {{64, 256, "bk64-chunk256"}, {32, 256, "bk32-chunk256"},
                                 {64, 512, "bk64-chunk512"}, {32, 512, "bk32-chunk512"}};
const TileConfig kX6Configs[] = {{32, 256, "bk32-chunk256"}, {32, 128, "bk32-chunk128"}};

std::string cache_path() {
  const char *e = std::getenv("GT_AUTOTUNE_CACHE");
  if (e && *e) return e;
  const char *h = std::getenv("HOME");
  return std::string(h ? h : "/tmp") + "/.cache/gputools_gb300/autotune.txt";
}

int cache_lookup(const std::string &key) {
  std::ifstream f(cache_path());
  std::string k;
  int v;
  int found = -1;
  while (f >> k >> v)
    if (k == key) found = v;
  return found;
}

void cache_store(const std::string &key, int v) {
  const std::string path = cache_path();
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) {
    std::string dir = path.substr(0, slash);
    for (size_t i = 1; i <= dir.size(); i++)
      if (i == dir.size() || dir[i] == '/') ::mkdir(dir.substr(0, i).c_str(), 0755);
  }
  std::ofstream f(path, std::ios::app);
  if (f) f << key << " " << v << "\n";
}

const char *kind_name(int kind) {
  return kind == GT_GRAM_TC_BF16X6 ? "bf16x6" : (kind == GT_GRAM_TC_F16X3 ? "f16x3" : "bf16x3");
}

int build_pearson(const gt_cor_problem *probs, int64_t count, int kind, const TileConfig &cfg,
                  gt_batch_plan **out) {
  auto *p = new gt_batch_plan();
  p->kind = 0;
  cudaGetDevice(&p->device);
  auto alloc = [p](size_t bytes, void **ptr) { return plan_alloc(p, bytes, ptr); };
  int st = pearson_batch_prepare(probs, count, kind, cfg.bk, cfg.chunk, alloc, &p->run,
                                 &p->tiles, &p->ctas, &p->err);
  if (st != GT_OK) {
    plan_free(p);
    return st;
  }
  std::snprintf(p->config, sizeof(p->config), "%s %s, %lld tiles on %lld ctas", kind_name(kind),
                cfg.name, (long long)p->tiles, (long long)p->ctas);
  *out = p;
  return GT_OK;
}

int time_plan(gt_batch_plan *p, double *ms) {
  cudaStream_t s = nullptr;
  GT_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int st = p->run(s);  // warm
  if (st == GT_OK) {
    cudaEventRecord(e0, s);
    for (int i = 0; i < 3 && st == GT_OK; i++) st = p->run(s);
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    float f = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&f, e0, e1);
    else st = fail(GT_ECUDA, "autotune timing: %s", cudaGetErrorString(e));
    *ms = f / 3.0;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  return st;
}

int pearson_batch_plan(const gt_cor_problem *probs, int64_t count, int flags,
                       gt_batch_plan **out) {
  if (count < 0 || (count > 0 && !probs)) return fail(GT_EINVAL, "bad problem list");
  const int path = gt_get_gram_path();
  if (path == GT_GRAM_FP32)
    return fail(GT_EUNSUPPORTED, "batched Pearson runs on the tensor-core Gram paths");
  if (path == GT_GRAM_TC_F16X6)
    return fail(GT_EUNSUPPORTED,
                "batched Pearson runs the f16x3, bf16x3 and bf16x6 splits, not f16x6");
  const bool x6 = path == GT_GRAM_TC_BF16X6;
  const TileConfig *cands = x6 ? kX6Configs : kX3Configs;
  const int ncand = x6 ? int(sizeof(kX6Configs) / sizeof(kX6Configs[0]))
                       : int(sizeof(kX3Configs) / sizeof(kX3Configs[0]));
  double work = 0.0;
  for (int64_t i = 0; i < count; i++) work += double(probs[i].p) * double(probs[i].p) * double(probs[i].n);
  char key[128];
  std::snprintf(key, sizeof(key), "pearson:%s:%lld:%.3e", kind_name(path), (long long)count,
                work);
  int choice = 0;
  if (flags & GT_BATCH_AUTOTUNE) {
    gt_batch_plan *best = nullptr;
    double best_ms = 0.0;
    for (int c = 0; c < ncand; c++) {
      gt_batch_plan *cand = nullptr;
      GT_TRY(build_pearson(probs, count, path, cands[c], &cand));
      double ms = 0.0;
      int st = time_plan(cand, &ms);
      if (st != GT_OK) {
        plan_free(cand);
        plan_free(best);
        return st;
      }
      if (!best || ms < best_ms) {
        plan_free(best);
        best = cand;
        best_ms = ms;
        choice = c;
      } else {
        plan_free(cand);
      }
    }
    cache_store(key, choice);
    best->config_ms = best_ms;
    char tmp[sizeof(best->config) + 64];
    std::snprintf(tmp, sizeof(tmp), "%s, tuned %.3f ms", best->config, best_ms);
    std::snprintf(best->config, sizeof(best->config), "%.*s", int(sizeof(best->config) - 1), tmp);
    int st = plan_finalize(best, flags);
    if (st != GT_OK) {
      plan_free(best);
      return st;
    }
    *out = best;
    return GT_OK;
  }
  const int cached = cache_lookup(key);
  if (cached >= 0 && cached < ncand) choice = cached;
  gt_batch_plan *p = nullptr;
  GT_TRY(build_pearson(probs, count, path, cands[choice], &p));
  int st = plan_finalize(p, flags);
  if (st != GT_OK) {
    plan_free(p);
    return st;
  }
  *out = p;
  return GT_OK;
}

}  // namespace gt

extern "C" int gt_pmcc_batch_plan_create(const gt_cor_problem *problems, int64_t count, int flags,
                                         gt_batch_plan **plan) {
  gt::clear_error();
  if (!plan) return gt::fail(GT_EINVAL, "null plan pointer");
  *plan = nullptr;
  return gt::pearson_batch_plan(problems, count, flags, plan);
}

extern "C" int gt_kendall_batch_plan_create(const gt_kendall_problem *problems, int64_t count,
                                            int flags, gt_batch_plan **plan) {
  gt::clear_error();
  if (!plan) return gt::fail(GT_EINVAL, "null plan pointer");
  *plan = nullptr;
  return gt::kendall_batch_plan(problems, count, flags, plan);
}

extern "C" int gt_batch_plan_launch(gt_batch_plan *plan, void *stream) {
  gt::clear_error();
  if (!plan) return gt::fail(GT_EINVAL, "null plan");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != plan->device)
    return gt::fail(GT_EINVAL, "plan was created on device %d, current device is %d", plan->device,
                    dev);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (plan->exec) {
    GT_CUDA(cudaGraphLaunch(plan->exec, s));
    return GT_OK;
  }
  return plan->run(s);
}

extern "C" const char *gt_batch_plan_describe(const gt_batch_plan *plan) {
  return plan ? plan->config : "";
}

extern "C" void gt_batch_plan_destroy(gt_batch_plan *plan) { gt::plan_free(plan); }
