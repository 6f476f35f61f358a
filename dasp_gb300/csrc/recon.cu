// Consumer of the centroids: the reconstructor matrix-vector step of DASP's
// tomoRecon (science/tomoRecon.py:1077-1107 decay, :1196-1223 MVM):
//   act[i] = decay_i * act[i] - gain_i * sum_j R[i, j] x[j]
// with R (nacts x ncents, row-major float32) resident in HBM.  The step is
// bound by reading R once: one warp per actuator row, 16-byte loads, eight
// in flight per lane, x read through L1 (every row reads it), float32
// accumulation as the reference's float32 dot, decay and gain fused into the
// same pass.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>

#include "../../include/shwfs.h"
#include "engine_internal.h"

namespace shwfs {

namespace {

constexpr int kMvmThreads = 256;
constexpr int kMvmUnroll = 8;  // 16-byte loads of R in flight per lane

__global__ void __launch_bounds__(kMvmThreads) mvm_update_kernel(const float* __restrict__ R, int nacts, int ncents,
                                                                 const float* __restrict__ x,
                                                                 const float* __restrict__ gains, float gain,
                                                                 const float* __restrict__ decay, float decay_s,
                                                                 float* __restrict__ act, bool vec) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < nacts; row += warps) {
    const float* r = R + (long long)row * ncents;
    float acc = 0.f;
    if (vec) {
      // 16-byte chunks, kMvmUnroll per lane per pass
      const int nq = ncents >> 2;
      const float4* r4 = reinterpret_cast<const float4*>(r);
      const float4* x4 = reinterpret_cast<const float4*>(x);
      int q = lane;
      for (; q + 32 * (kMvmUnroll - 1) < nq; q += 32 * kMvmUnroll) {
        float4 a[kMvmUnroll];
#pragma unroll
        for (int u = 0; u < kMvmUnroll; u++) a[u] = __ldcs(r4 + q + 32 * u);
#pragma unroll
        for (int u = 0; u < kMvmUnroll; u++) {
          const float4 b = x4[q + 32 * u];
          acc += a[u].x * b.x + a[u].y * b.y + a[u].z * b.z + a[u].w * b.w;
        }
      }
      for (; q < nq; q += 32) {
        const float4 a0 = __ldcs(r4 + q), b0 = x4[q];
        acc += a0.x * b0.x + a0.y * b0.y + a0.z * b0.z + a0.w * b0.w;
      }
    } else {
      for (int j = lane; j < ncents; j += 32) acc += __ldcs(r + j) * x[j];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const float d = decay ? decay[row] : decay_s;
      const float g = gains ? gains[row] : gain;
      act[row] = d * act[row] - g * acc;
    }
  }
}

}  // namespace

}  // namespace shwfs

extern "C" shwfs_status shwfs_mvm_update(int nacts, int ncents, const float* R, const float* x, const float* gains,
                                         float gain, const float* decay, float decay_scalar, float* act,
                                         void* stream) {
  if (nacts < 1 || ncents < 1 || !R || !x || !act)
    return shwfs::engine_fail(SHWFS_ERR_INVALID, "mvm_update: bad arguments");
  const bool vec = (ncents & 3) == 0 && ((uintptr_t)R & 15) == 0 && ((uintptr_t)x & 15) == 0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int warpsPerCta = shwfs::kMvmThreads / 32;
  const int grid = std::max(1, std::min((nacts + warpsPerCta - 1) / warpsPerCta, sms * 8));
  cudaStream_t st = (cudaStream_t)stream;
  shwfs::mvm_update_kernel<<<grid, shwfs::kMvmThreads, 0, st>>>(R, nacts, ncents, x, gains, gain, decay, decay_scalar,
                                                                act, vec);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return shwfs::engine_fail(SHWFS_ERR_CUDA, (std::string("mvm_update: ") + cudaGetErrorString(e)).c_str());
  return SHWFS_OK;
}
