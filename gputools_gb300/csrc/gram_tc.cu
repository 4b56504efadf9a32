// gram_tc.cu -- placeholder until the tcgen05 path lands.
#include "common.cuh"
#include "kernels.cuh"
namespace gt {
int pearson_tc_prologue(const float *, int64_t, int64_t, int, int, int, void **, int64_t *,
                        cudaStream_t) {
  return fail(GT_EUNSUPPORTED, "tensor-core path not built");
}
int pearson_tc(const void *, int64_t, const void *, int64_t, int64_t, int, const PearsonOut &,
               cudaStream_t) {
  return fail(GT_EUNSUPPORTED, "tensor-core path not built");
}
int euclid_tc(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout,
              cudaStream_t st) {
  return dist_simt(d_pts, n, dim, d_out, layout, GT_EUCLIDEAN, 2.f, st);
}
}  // namespace gt
