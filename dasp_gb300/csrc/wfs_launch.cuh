// Registry of the compiled (fftsize, psfsize) instantiations of the fused
// kernel.  Each wfs_inst_*.cu translation unit instantiates a few sizes and
// registers host-side launchers at load time; the engine looks them up by
// size when a handle is created.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <utility>

#include "wfs_plain.cuh"

namespace shwfs {

struct PlainEntry {
  cudaError_t (*launch)(const WfsArgs&, int grid, int smem, cudaStream_t);
  // several handles of this instantiation in one launch (grid = m.ctaStart[m.n])
  cudaError_t (*launch_multi)(const PlainMulti& m, int smem, cudaStream_t);
  cudaError_t (*occupancy_multi)(int* ctas_per_sm, int smem);
  cudaError_t (*occupancy)(int* ctas_per_sm, int smem);
  cudaError_t (*psf_spectra)(const float* psf, int npsf, float2* out, cudaStream_t);
};

inline std::map<std::pair<int, int>, PlainEntry>& plain_registry() {
  static std::map<std::pair<int, int>, PlainEntry> r;
  return r;
}

// r2c spectrum of each PSF after the reference's quadrant swap
// (flipArray(...,1,...) then fftwf r2c, cmod/src/centmodule.c:2348-2373).
// One CTA per PSF; out is [npsf][P][P/2+1].
template <int P>
__global__ void psf_spectrum_kernel(const float* psf, int npsf, float2* out) {
  constexpr int HS = P / 2 + 1;
  __shared__ float2 rows[P * HS];
  const int k = blockIdx.x;
  if (k >= npsf) return;
  const float* src = psf + (long long)k * P * P;
  for (int r = threadIdx.x; r < P; r += blockDim.x) {
    float2 y[P];
    const int sr = (r + P / 2) % P;
#pragma unroll
    for (int n = 0; n < P; n++) y[n] = make_float2(src[sr * P + (n + P / 2) % P], 0.f);
    fft<P, -1>(y);
#pragma unroll
    for (int c = 0; c < HS; c++) rows[r * HS + c] = y[c];
  }
  __syncthreads();
  for (int c = threadIdx.x; c < HS; c += blockDim.x) {
    float2 y[P];
#pragma unroll
    for (int r = 0; r < P; r++) y[r] = rows[r * HS + c];
    fft<P, -1>(y);
#pragma unroll
    for (int r = 0; r < P; r++) out[(long long)k * P * HS + r * HS + c] = y[r];
  }
}

template <int N, int P>
cudaError_t plain_launch(const WfsArgs& a, int grid, int smem, cudaStream_t stream) {
  cudaError_t e = kernel_smem_setup((const void*)wfs_plain_kernel<N, P>, smem, kThreads, nullptr);
  if (e != cudaSuccess) return e;
  wfs_plain_kernel<N, P><<<grid, kThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

template <int N, int P>
cudaError_t plain_launch_multi(const PlainMulti& m, int smem, cudaStream_t stream) {
  cudaError_t e = kernel_smem_setup((const void*)wfs_plain_multi_kernel<N, P>, smem, kThreads, nullptr);
  if (e != cudaSuccess) return e;
  wfs_plain_multi_kernel<N, P><<<m.ctaStart[m.n], kThreads, smem, stream>>>(m);
  return cudaGetLastError();
}

template <int N, int P>
cudaError_t plain_occupancy_multi(int* ctas, int smem) {
  return kernel_smem_setup((const void*)wfs_plain_multi_kernel<N, P>, smem, kThreads, ctas);
}

template <int N, int P>
cudaError_t plain_occupancy(int* ctas, int smem) {
  return kernel_smem_setup((const void*)wfs_plain_kernel<N, P>, smem, kThreads, ctas);
}

template <int P>
cudaError_t psf_spectra_launch(const float* psf, int npsf, float2* out, cudaStream_t stream) {
  if constexpr (P > 0) {
    psf_spectrum_kernel<P><<<npsf, 64, 0, stream>>>(psf, npsf, out);
    return cudaGetLastError();
  } else {
    return cudaErrorInvalidValue;
  }
}

template <int N, int P>
struct PlainRegistrar {
  PlainRegistrar() {
    plain_registry()[{N, P}] =
        PlainEntry{&plain_launch<N, P>, &plain_launch_multi<N, P>, &plain_occupancy_multi<N, P>,
                   &plain_occupancy<N, P>, &psf_spectra_launch<P>};
  }
};

#define SHWFS_REGISTER_PLAIN(N, P) static ::shwfs::PlainRegistrar<N, P> shwfs_reg_##N##_##P;

}  // namespace shwfs
