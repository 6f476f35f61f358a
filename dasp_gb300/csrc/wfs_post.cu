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
constexpr int kPostBright = 512;  // queued bright pixels per tile (overflow: drawn in place)

__global__ void __launch_bounds__(kPostThreads, 4) wfs_post_kernel(const WfsArgs a, const PoisTab* __restrict__ tab) {
  extern __shared__ __align__(16) float smem_post[];
  __shared__ int s_subap[kPostMaxTS];
  __shared__ int s_frame[kPostMaxTS];
  __shared__ unsigned char s_pflag[kPostMaxTS];
  __shared__ int s_nbright;
  __shared__ int s_bright[kPostBright];
  __shared__ float s_brightv[kPostBright];
  const int tid = threadIdx.x;
  const int mm = a.m * a.m;
  const bool cw2d = a.centWeightDim == 2;
  const bool useTab = tab != nullptr;
  PoisTab* s_tab = reinterpret_cast<PoisTab*>(smem_post);
  float* s_cw = smem_post + (useTab ? sizeof(PoisTab) / sizeof(float) : 0);
  float* imgs = s_cw + (cw2d ? mm : 0);
  if (useTab) {
    const int4* src = reinterpret_cast<const int4*>(tab);
    int4* dst = reinterpret_cast<int4*>(s_tab);
    for (int k = tid; k < (int)(sizeof(PoisTab) / sizeof(int4)); k += blockDim.x) dst[k] = src[k];
  }
  if (cw2d)
    for (int k = tid; k < mm; k += blockDim.x) s_cw[k] = a.centWeight[k];
  const int TS = a.TS;
  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + TS - 1) / TS;
  const bool noise = a.mode & kNoiseCounter;
  const bool pois = a.addPoisson == 1 && a.calsource == 0;
  const float rn = a.calsource == 0 ? a.readNoise : 0.f;
  const unsigned long long fbase = frame_base(a);
  // the common configuration (window CoG, no brightest-pixel selection, no
  // fit) takes a lean path; everything else runs post_tile
  const bool simple = !(a.calsource == 0 && (a.useBrightest != 0 || a.useBrightestArr)) && a.opticalBinning != 1 &&
                      a.fitSize == 0 && a.gaussianFit <= 0 && a.cob == 0;

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
    if (tid == 0) s_nbright = 0;
    __syncthreads();  // the tile's subaperture list is complete
    const float inv_mm = 1.0f / (float)mm;
    // the tile's pre-noise pixels into shared memory with asynchronous
    // copies: every load is in flight at once instead of one per iteration
    for (int w = tid; w < ns * mm; w += blockDim.x) {
      const int s = div_small(w, mm, inv_mm);
      const float* src = a.bimg + (long long)s_frame[s] * a.bimgFrameStride + (long long)s_subap[s] * mm + (w - s * mm);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(imgs + w)),
                   "l"(src)
                   : "memory");
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    // noise, threshold [, power, bimg write] of pixel w of the tile
    auto pixel = [&](int w, float v) {
      const int s = div_small(w, mm, inv_mm), pix = w - s * mm;
      const int i = s_subap[s];
      if (noise) {
        // one stream per pixel: the read-noise normal takes the first two
        // uniforms, the Poisson sampler continues from the third
        CounterStream st(a.seed, fbase + s_frame[s], i, pix, 0);
        const float g = rn != 0.f ? normal_counter(st) : 0.f;
        if (pois && s_pflag[s]) v = poisson_counter_tab(st, v, *s_tab);
        if (rn != 0.f)
          v += rn * g + a.readBg;
        else
          v += a.readBg;
        v = threshold_px(v, a.floorv, a.threshType);
      }
      if (simple) {
        // pixel power and the bimg write of post_tile's stage 8, here
        if (a.pxlPower == 2.f)
          v = v * v;
        else if (a.pxlPower != 1.f && a.pxlPower != 0.f)
          v = powf(v, a.pxlPower);
        a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)i * mm + pix] = v;
      }
      imgs[s * mm + pix] = v;
    };
    // Pixels whose Poisson mean needs the rejection sampler (lambda >= 64)
    // are queued and drawn afterwards with the whole CTA, so that one bright
    // pixel does not hold the other 31 lanes of its warp (same streams, same
    // draws).
    for (int w = tid; w < ns * mm; w += blockDim.x) {
      const int s = div_small(w, mm, inv_mm);
      const float v = imgs[w];
      if (noise && pois && s_pflag[s] && v >= kModalMaxLam) {
        const int slot = atomicAdd(&s_nbright, 1);
        if (slot < kPostBright) {
          s_bright[slot] = w;
          s_brightv[slot] = v;
          continue;
        }
      }
      pixel(w, v);
    }
    __syncthreads();
    const int nb = min(s_nbright, kPostBright);
    for (int k = tid; k < nb; k += blockDim.x) pixel(s_bright[k], s_brightv[k]);
    __syncthreads();
    if (!simple) {
      post_tile(a, ns, s_subap, s_frame, s_cw, [&](int s) { return imgs + s * mm; }, [&](int) { return mm; });
      continue;
    }
    if (a.imageOnly != 0 || a.skipCents) continue;
    // centred-window CoG (post_tile's stage 9, same summation order): one
    // warp per subaperture, lanes over the window pixels
    const int warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
    const int m = a.m, ncen = a.ncen, sx0 = (m - ncen) / 2, nwin = ncen * ncen;
    const float inv_nc = 1.0f / (float)ncen;
    for (int s = warp; s < ns; s += nwarps) {
      const float* img = imgs + s * mm;
      const int i = s_subap[s];
      const float* wt = cw2d ? s_cw : (a.centWeightDim == 4 ? a.centWeight + (long long)i * mm : nullptr);
      float sum = 0.f, sxv = 0.f, syv = 0.f;
      for (int k = lane; k < nwin; k += 32) {
        const int rr = div_small(k, ncen, inv_nc);
        const int r = sx0 + rr, c = sx0 + (k - rr * ncen);
        float t = img[r * m + c];
        if (wt) t *= wt[r * m + c];
        sum += t;
        sxv += t * c;
        syv += t * r;
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        sxv += __shfl_xor_sync(0xffffffffu, sxv, o);
        syv += __shfl_xor_sync(0xffffffffu, syv, o);
      }
      if (lane == 0) {
        float cx = 0.f, cy = 0.f;
        if (sum > 0.f) {
          cx = sxv / sum - 0.5f * (float)(m - 1);
          cy = syv / sum - 0.5f * (float)(m - 1);
        }
        calibrate_and_store(a, i, s_frame[s], cx, cy);
      }
    }
  }
}

}  // namespace

cudaError_t launch_post(const WfsArgs& a0, int numSMs, cudaStream_t stream) {
  WfsArgs a = a0;
  const int mm = a.m * a.m;
  const long long nwork = (long long)a.nlit * a.nframes;
  if (nwork == 0) return cudaSuccess;
  a.TS = mm > 0 ? (8192 / mm < 1 ? 1 : (8192 / mm > kPostMaxTS ? kPostMaxTS : 8192 / mm)) : 1;
  const bool pois = (a.mode & kNoiseCounter) && a.addPoisson == 1 && a.calsource == 0;
  const PoisTab* tab = nullptr;
  if (pois) {
    cudaError_t et = pois_table_device(&tab);
    if (et != cudaSuccess) return et;
  }
  const int smem = (a.TS * mm + (a.centWeightDim == 2 ? mm : 0)) * (int)sizeof(float) +
                   (pois ? (int)sizeof(PoisTab) : 0);
  cudaError_t e = cudaFuncSetAttribute(wfs_post_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int ctas = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, wfs_post_kernel, kPostThreads, smem);
  if (e != cudaSuccess) return e;
  if (ctas < 1) return cudaErrorInvalidConfiguration;
  const long long ntiles = (nwork + a.TS - 1) / a.TS;
  const long long cap = (long long)numSMs * ctas;
  const int grid = (int)(ntiles < cap ? ntiles : cap);
  wfs_post_kernel<<<grid, kPostThreads, smem, stream>>>(a, tab);
  return cudaGetLastError();
}

}  // namespace shwfs
