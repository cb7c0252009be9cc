// Tile-wise sum of two arrays of the same tiling into a third, for sm_103a:
// the tile operation of TiledArray's AddEngine (expressions/add_engine.h) as
// used by `C("i,j") += A("i,k") * B("k,j")` (expressions/tsr_expr.h:146-152).
// Where both argument tiles exist the result is c + p (one rounding); where
// one is absent the other is copied unchanged (signed zeros included).
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

__global__ void __launch_bounds__(256) add_tiles_kernel(const AddChunk* __restrict__ chunks,
                                                        int64_t nchunks,
                                                        const double* __restrict__ C,
                                                        const double* __restrict__ P,
                                                        double* __restrict__ R) {
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const AddChunk k = chunks[ch];
    double* r = R + k.r;
    if (k.c >= 0 && k.p >= 0) {
      const double* c = C + k.c;
      const double* p = P + k.p;
      for (int64_t i = threadIdx.x; i < k.len; i += blockDim.x) r[i] = __dadd_rn(c[i], p[i]);
    } else {
      const double* s = k.c >= 0 ? C + k.c : P + k.p;
      for (int64_t i = threadIdx.x; i < k.len; i += blockDim.x) r[i] = s[i];
    }
  }
}

}  // namespace

void launch_add_tiles(cudaStream_t s, const AddChunk* chunks, int64_t nchunks, const double* C,
                      const double* P, double* R) {
  if (nchunks <= 0) return;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t grid = nchunks < (int64_t)sms * 16 ? nchunks : (int64_t)sms * 16;
  add_tiles_kernel<<<(unsigned)grid, 256, 0, s>>>(chunks, nchunks, C, P, R);
  count_launch();
}

}  // namespace tagpu
