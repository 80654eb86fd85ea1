// sdg_screen.cu -- the screened candidate engine (see sdg_screen.h).
#include "sdg_kernels.h"
#include "sdg_screen.h"

namespace sdg {
namespace {

__global__ void k_check_rows(DevCsc M, int* err) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= M.ncol) return;
  int32_t prev = -1;
  for (int64_t a = M.p[j]; a < M.p[j + 1]; ++a) {
    const int32_t r = M.i[a];
    if (r <= prev || r >= M.nrow) { atomicOr(err, 1); return; }
    prev = r;
  }
}

}  // namespace

void launch_check_rows(const DevCsc& M, int* err, cudaStream_t s) {
  if (M.ncol > 0) k_check_rows<<<(unsigned)((M.ncol + 127) / 128), 128, 0, s>>>(M, err);
}

bool screen_supported(int, int) { return false; }

int screen_knn(cudaStream_t, const ScreenRun&, const DevCsc&, const ColAux&, ScreenCache*,
               const DevCsc&, const ColAux&, ScreenCache*, int32_t*, double*, int64_t*,
               const std::function<void()>&) {
  return (int)cudaErrorNotSupported;
}

void screen_cache_free(ScreenCache* c, cudaStream_t s) {
  if (c && c->blob) cudaFreeAsync(c->blob, s);
  if (c) *c = ScreenCache();
}

}  // namespace sdg
