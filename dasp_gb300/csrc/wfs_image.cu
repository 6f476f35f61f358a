// Image-input path of the WFS step (runSlope): centroids from a detector
// image instead of phase (cmod/src/centmodule.c:1987-2127).
//
// Per lit subaperture: the subaperture window is cut from the 2-D detector
// image (default tiling by nimg, or the caller's subapLocation rows/cols) or
// taken from a 4-D (nsubx,nsubx,nimg,nimg) image; as in the reference the
// window lands in the top-left of the nimg x nimg image and pixels outside it
// keep their previous bimg values.  Then, for a science source, readCCD with
// no noise (threshold only) over the first nexposed pixels in storage order,
// and the shared post stages (brightest pixels, power, bimg, centroids).
#include "wfs_plain.cuh"

namespace shwfs {

__device__ __forceinline__ void subap_window(const WfsArgs& a, const int* loc, int i, int& r0, int& r1, int& c0,
                                             int& c1) {
  if (loc) {
    r0 = loc[i * 4];
    r1 = loc[i * 4 + 1];
    c0 = loc[i * 4 + 2];
    c1 = loc[i * 4 + 3];
  } else {
    r0 = (i / a.nsubx) * a.m;
    r1 = r0 + a.m;
    c0 = (i % a.nsubx) * a.m;
    c1 = c0 + a.m;
  }
}

__global__ void __launch_bounds__(kThreads)
    wfs_image_kernel(const WfsArgs a, const float* img, int dims, int npxlx, const int* loc) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int tid = threadIdx.x;
  const int m = a.m, mm = m * m;
  const bool cw2d = a.centWeightDim == 2;
  float* s_cw = smem;
  float* s_sub0 = smem + (((cw2d ? mm : 0) + 3) & ~3);
  const int persub = (mm + 3) & ~3;
  __shared__ int s_subap[64];
  __shared__ int s_frame[64];
  __shared__ int s_nexp[64];
  if (cw2d)
    for (int k = tid; k < mm; k += blockDim.x) s_cw[k] = a.centWeight[k];
  const int TS = a.TS;
  const int ntiles = (a.nlit + TS - 1) / TS;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int w0 = tile * TS;
    const int ns = min(TS, a.nlit - w0);
    __syncthreads();
    for (int s = tid; s < ns; s += blockDim.x) {
      const int i = a.lit[w0 + s];
      s_subap[s] = i;
      s_frame[s] = 0;
      if (dims == 4) {
        s_nexp[s] = mm;
      } else {
        int r0, r1, c0, c1;
        subap_window(a, loc, i, r0, r1, c0, c1);
        s_nexp[s] = (r1 - r0) * (c1 - c0);
      }
    }
    __syncthreads();
    for (int w = tid; w < ns * mm; w += blockDim.x) {
      const int s = w / mm, pix = w - s * mm;
      const int i = s_subap[s];
      float v;
      if (dims == 4) {
        v = img[(long long)i * mm + pix];
      } else {
        int r0, r1, c0, c1;
        subap_window(a, loc, i, r0, r1, c0, c1);
        const int j = pix / m, k = pix - j * m;
        if (j < r1 - r0 && k < c1 - c0)
          v = img[(long long)(r0 + j) * npxlx + c0 + k];
        else
          v = a.bimg[(long long)i * mm + pix];
      }
      if (a.calsource == 0 && pix < s_nexp[s]) v = threshold_px(v + 0.f, a.floorv, a.threshType);
      s_sub0[s * persub + pix] = v;
    }
    __syncthreads();
    post_tile(a, ns, s_subap, s_frame, s_cw, [&](int s) { return s_sub0 + s * persub; },
              [&](int s) { return s_nexp[s]; });
  }
}

cudaError_t launch_image(const WfsArgs& a, const float* img, int dims, int npxlx, const int* loc, int numSMs,
                         cudaStream_t stream) {
  const int mm = a.m * a.m;
  const int smem = ((((a.centWeightDim == 2 ? mm : 0) + 3) & ~3) + a.TS * ((mm + 3) & ~3)) * 4;
  cudaError_t e = kernel_smem_setup((const void*)wfs_image_kernel, smem, kThreads, nullptr);
  if (e != cudaSuccess) return e;
  const int ntiles = (a.nlit + a.TS - 1) / a.TS;
  const int grid = ntiles < numSMs * 8 ? (ntiles > 0 ? ntiles : 1) : numSMs * 8;
  wfs_image_kernel<<<grid, kThreads, smem, stream>>>(a, img, dims, npxlx, loc);
  return cudaGetLastError();
}

}  // namespace shwfs
