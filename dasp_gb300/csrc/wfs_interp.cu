// Phase interpolation (interpolatePhase, cmod/src/centmodule.c:1628-1758):
// when the phase array is not nsubx*phasesize square, each readout first
// resamples it to that size with the reference's bicubic (Catmull-Rom)
// convolution, and the pipeline then runs on the resampled array.  The
// reference does this per subaperture inside its worker loop (:1795-1804);
// here one kernel resamples the whole array (every output sample depends on
// its position only), one thread per output sample.
//
// Arithmetic follows the C code in float with its operation order and no
// contraction (explicit _rn intrinsics): the sample position t = scale*X,
// the weights 0.5*(1, t, t^2, t^3), four basis-row sums over four input rows
// per input column, the y weighting, the basis rows over the four column
// values and the x weighting.  Input rows and columns outside the array
// repeat the edge (:1685-1728); the last output sample of each axis uses
// t = 1 from input sample n-3 (:1663-1666).
#include <algorithm>

#include "wfs_plain.cuh"

namespace shwfs {

namespace {

__device__ __forceinline__ float dot4c(float c0, float c1, float c2, float c3, const float (&v)[4]) {
  float s = __fmul_rn(c0, v[0]);
  s = __fadd_rn(s, __fmul_rn(c1, v[1]));
  s = __fadd_rn(s, __fmul_rn(c2, v[2]));
  return __fadd_rn(s, __fmul_rn(c3, v[3]));
}

// basis row k of the Catmull-Rom matrix applied to v
__device__ __forceinline__ float basis_row(int k, const float (&v)[4]) {
  switch (k) {
    case 0: return dot4c(0.f, 2.f, 0.f, 0.f, v);
    case 1: return dot4c(-1.f, 0.f, 1.f, 0.f, v);
    case 2: return dot4c(2.f, -5.f, 4.f, -1.f, v);
    default: return dot4c(-1.f, 3.f, -3.f, 1.f, v);
  }
}

__device__ __forceinline__ void cubic_axis(int X, int nin, int nout, float scale, int& i0, float (&w)[4]) {
  float t = __fmul_rn(scale, (float)X);
  i0 = (int)floorf(t);
  t = __fsub_rn(t, (float)i0);
  i0--;
  if (X == nout - 1) {
    t = 1.f;
    i0 = nin - 3;
  }
  w[0] = 0.5f;
  w[1] = __fmul_rn(0.5f, t);
  w[2] = __fmul_rn(w[1], t);
  w[3] = __fmul_rn(w[2], t);
}

__global__ void interp_phase_kernel(const float* __restrict__ in, long long inStride, int nin, float* __restrict__ out,
                                    long long outStride, int nout, float scale, int nframes) {
  const long long per = (long long)nout * nout, total = per * nframes;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(idx / per);
    const long long rem = idx - (long long)f * per;
    const int Y = (int)(rem / nout), X = (int)(rem - (long long)Y * nout);
    int iy, ix;
    float wy[4], wx[4];
    cubic_axis(Y, nin, nout, scale, iy, wy);
    cubic_axis(X, nin, nout, scale, ix, wx);
    const float* src = in + (long long)f * inStride;
    int rows[4];
#pragma unroll
    for (int j = 0; j < 4; j++) rows[j] = min(max(iy + j, 0), nin - 1);
    float pc[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int c = min(max(ix + i, 0), nin - 1);
      float fv[4], tmp[4];
#pragma unroll
      for (int j = 0; j < 4; j++) fv[j] = src[(long long)rows[j] * nin + c];
#pragma unroll
      for (int k = 0; k < 4; k++) tmp[k] = basis_row(k, fv);
      pc[i] = dot4c(wy[0], wy[1], wy[2], wy[3], tmp);
    }
    float t2[4];
#pragma unroll
    for (int i = 0; i < 4; i++) t2[i] = basis_row(i, pc);
    out[(long long)f * outStride + rem] = dot4c(wx[0], wx[1], wx[2], wx[3], t2);
  }
}

// p x p blocks of the lit subapertures from src (W x W) to dst (W x W)
__global__ void copy_lit_blocks_kernel(const float* __restrict__ src, float* __restrict__ dst, const int* __restrict__ lit,
                                       int nlit, int nsubx, int p) {
  const int W = nsubx * p, pp = p * p;
  const long long total = (long long)nlit * pp;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(idx / pp), k = (int)(idx - (long long)l * pp);
    const int s = lit[l], sy = s / nsubx, sx = s - sy * nsubx;
    const long long o = (long long)(sy * p + k / p) * W + sx * p + k % p;
    dst[o] = src[o];
  }
}

}  // namespace

cudaError_t launch_interp_phase(const float* in, long long inStride, int nin, float* out, long long outStride, int nout,
                                int nframes, cudaStream_t stream) {
  const long long total = (long long)nout * nout * nframes;
  if (total == 0) return cudaSuccess;
  const float scale = (float)((nin - 1.0) / (nout - 1));
  const long long blocks = std::min<long long>((total + 255) / 256, 152LL * 16);
  interp_phase_kernel<<<(int)blocks, 256, 0, stream>>>(in, inStride, nin, out, outStride, nout, scale, nframes);
  return cudaGetLastError();
}

cudaError_t launch_copy_lit_blocks(const float* src, float* dst, const int* lit, int nlit, int nsubx, int p,
                                   cudaStream_t stream) {
  const long long total = (long long)nlit * p * p;
  if (total == 0) return cudaSuccess;
  const long long blocks = std::min<long long>((total + 255) / 256, 152LL * 8);
  copy_lit_blocks_kernel<<<(int)blocks, 256, 0, stream>>>(src, dst, lit, nlit, nsubx, p);
  return cudaGetLastError();
}

}  // namespace shwfs
