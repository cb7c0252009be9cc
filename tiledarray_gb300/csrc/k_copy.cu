// Host <-> device copies of array storage driven by the SMs, for sm_103a on
// a coherent host link (Grace + NVLink-C2C): the kernel reads or writes the
// registered host buffer through its device-visible address.  On GB300 this
// reaches the same ~210 GB/s (H2D) and ~193 GB/s (D2H) as the copy engines,
// and it does not depend on which copy engine a stream is given.
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

// 16-byte vectors where both ends are 16-byte aligned, 8-byte words
// otherwise; four independent vectors in flight per thread.
__global__ void __launch_bounds__(256) link_copy_kernel(uint8_t* __restrict__ dst,
                                                        const uint8_t* __restrict__ src,
                                                        size_t bytes) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t done = 0;
  if ((((uintptr_t)dst | (uintptr_t)src) & 15) == 0) {
    const size_t n16 = bytes / 16;
    uint4* d = reinterpret_cast<uint4*>(dst);
    const uint4* s = reinterpret_cast<const uint4*>(src);
    size_t i = tid;
    for (; i + 3 * stride < n16; i += 4 * stride) {
      const uint4 a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
      d[i] = a;
      d[i + stride] = b;
      d[i + 2 * stride] = c;
      d[i + 3 * stride] = e;
    }
    for (; i < n16; i += stride) d[i] = s[i];
    done = n16 * 16;
  } else if ((((uintptr_t)dst | (uintptr_t)src) & 7) == 0) {
    const size_t n8 = bytes / 8;
    uint64_t* d = reinterpret_cast<uint64_t*>(dst);
    const uint64_t* s = reinterpret_cast<const uint64_t*>(src);
    for (size_t i = tid; i < n8; i += stride) d[i] = s[i];
    done = n8 * 8;
  }
  for (size_t i = done + tid; i < bytes; i += stride) dst[i] = src[i];
}

}  // namespace

bool link_copy_usable(const void* host) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  int host_ptr = 0, coherent = 0;
  cudaDeviceGetAttribute(&host_ptr, cudaDevAttrCanUseHostPointerForRegisteredMem, dev);
  cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
  if (!host_ptr || !coherent) return false;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost && at.devicePointer == host;
}

void launch_link_copy(cudaStream_t s, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (bytes + 4095) / 4096;   // one 256-thread block per 4 KB at most
  const unsigned grid = (unsigned)(want < (size_t)sms * 4 ? want : (size_t)sms * 4);
  link_copy_kernel<<<grid, 256, 0, s>>>(static_cast<uint8_t*>(dst),
                                         static_cast<const uint8_t*>(src), bytes);
  count_launch();
}

}  // namespace tagpu
