// fvc_gather.cu -- value upload for a loaded structure: fills the SELL-32
// value slots from the caller's raw arrays with the slot map built once per
// structure, so a new SIMPLE outer iteration moves only the values.
#include "fvc_internal.h"

namespace fvc {

namespace {

// src code: >= 0 index into a1; -1 padding (0.0); <= -2 index -code-2 in a2
__global__ void gather_values(int64_t slots, const int32_t *__restrict__ src,
                              const double *__restrict__ a1, const double *__restrict__ a2,
                              double *__restrict__ val) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < slots;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = src[q];
    val[q] = (c >= 0) ? a1[c] : ((c == -1) ? 0.0 : a2[-(int64_t)c - 2]);
  }
}

}  // namespace

int32_t launch_gather_values(int64_t slots, const int32_t *src, const double *a1,
                             const double *a2, double *val, cudaStream_t stream) {
  if (slots <= 0) return FVC_OK;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t want = (slots + 255) / 256;
  int blocks = (int)std::min<int64_t>(want, (int64_t)sms * 16);
  gather_values<<<blocks, 256, 0, stream>>>(slots, src, a1, a2, val);
  count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

}  // namespace fvc
