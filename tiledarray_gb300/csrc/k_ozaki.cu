// Kernel (d), emulated FP64 form (Ozaki scheme on the tcgen05 tensor cores).
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {

tagpu_status ozaki_run(cudaStream_t, const GemmView&, int, int, size_t*, double*, double*,
                       int64_t*, std::string* err) {
  *err = "emulated FP64 form not built yet";
  return TAGPU_ERR_UNSUPPORTED;
}

}  // namespace tagpu
