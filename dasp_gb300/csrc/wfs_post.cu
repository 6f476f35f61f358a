// Noise, threshold and post stages of the GEMM-DFT form.
//
// The tensor-core kernel (wfs_gemm.cu) leaves each lit subaperture-frame's
// normalised pre-noise image in bimg; this kernel adds the counter-based
// Poisson and read noise, thresholds (cmod/src/centmodule.c:1874-1882,
// 785-817) and runs the shared post stages (post_tile: brightest pixels,
// pixel power, bimg write, centroids, calibration, references).  Each pixel
// draws from the same (seed, frame, subaperture, pixel) stream as in the
// fused FP32 kernel, so equal pre-noise images give equal noisy images.
//
// A separate launch rather than a stage of the tensor-core kernel: the noise
// samplers are latency-bound scalar code that wants many resident warps,
// while the tensor-core kernel holds one 576-thread CTA per SM.
#include "gemm_form.h"
#include "wfs_plain.cuh"

namespace shwfs {

namespace {

constexpr int kPostThreads = 256;
constexpr int kPostMaxTS = 64;

__global__ void __launch_bounds__(kPostThreads, 4) wfs_post_kernel(const WfsArgs a) {
  extern __shared__ float smem_post[];
  __shared__ int s_subap[kPostMaxTS];
  __shared__ int s_frame[kPostMaxTS];
  __shared__ unsigned char s_pflag[kPostMaxTS];
  const int tid = threadIdx.x;
  const int mm = a.m * a.m;
  const bool cw2d = a.centWeightDim == 2;
  float* s_cw = smem_post;
  float* imgs = smem_post + (cw2d ? mm : 0);
  if (cw2d)
    for (int k = tid; k < mm; k += blockDim.x) s_cw[k] = a.centWeight[k];
  const int TS = a.TS;
  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + TS - 1) / TS;
  const bool noise = a.mode & kNoiseCounter;
  const bool pois = a.addPoisson == 1 && a.calsource == 0;
  const float rn = a.calsource == 0 ? a.readNoise : 0.f;
  const unsigned long long fbase = frame_base(a);

  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long w0 = tile * TS;
    const int ns = (int)min((long long)TS, nwork - w0);
    __syncthreads();  // previous tile fully consumed
    for (int s = tid; s < ns; s += blockDim.x) {
      const long long w = w0 + s;
      const int i = a.lit[w % a.nlit];
      s_frame[s] = (int)(w / a.nlit);
      s_subap[s] = i;
      s_pflag[s] = a.totsig[i] > 0.f || a.sky * a.frac[i] > 0.f || a.skyArr;
    }
    __syncthreads();
    const float inv_mm = 1.0f / (float)mm;
    for (int w = tid; w < ns * mm; w += blockDim.x) {
      const int s = div_small(w, mm, inv_mm), pix = w - s * mm;
      const int i = s_subap[s];
      float v = a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)i * mm + pix];
      if (noise) {
        // one stream per pixel: the read-noise normal takes the first two
        // uniforms, the Poisson sampler continues from the third
        CounterStream st(a.seed, fbase + s_frame[s], i, pix, 0);
        const float g = rn != 0.f ? normal_counter(st) : 0.f;
        if (pois && s_pflag[s]) v = poisson_counter(st, v);
        if (rn != 0.f)
          v += rn * g + a.readBg;
        else
          v += a.readBg;
        v = threshold_px(v, a.floorv, a.threshType);
      }
      imgs[s * mm + pix] = v;
    }
    __syncthreads();
    post_tile(a, ns, s_subap, s_frame, s_cw, [&](int s) { return imgs + s * mm; }, [&](int) { return mm; });
  }
}

}  // namespace

cudaError_t launch_post(const WfsArgs& a0, int numSMs, cudaStream_t stream) {
  WfsArgs a = a0;
  const int mm = a.m * a.m;
  const long long nwork = (long long)a.nlit * a.nframes;
  if (nwork == 0) return cudaSuccess;
  a.TS = mm > 0 ? (8192 / mm < 1 ? 1 : (8192 / mm > kPostMaxTS ? kPostMaxTS : 8192 / mm)) : 1;
  const int smem = (a.TS * mm + (a.centWeightDim == 2 ? mm : 0)) * (int)sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(wfs_post_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int ctas = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, wfs_post_kernel, kPostThreads, smem);
  if (e != cudaSuccess) return e;
  if (ctas < 1) return cudaErrorInvalidConfiguration;
  const long long ntiles = (nwork + a.TS - 1) / a.TS;
  const long long cap = (long long)numSMs * ctas;
  const int grid = (int)(ntiles < cap ? ntiles : cap);
  wfs_post_kernel<<<grid, kPostThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace shwfs
