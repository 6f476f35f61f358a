// Reference-stream noise: the reference's own generators on the GPU.
//
// In SHWFS_NOISE_REFERENCE mode the fused kernel stops after the sky stage
// and leaves the pre-noise images in bimg; this kernel then walks each
// reference worker thread's contiguous subaperture range in order, exactly
// as workerFunc/centroidsFromPhase do (cmod/src/centmodule.c:1791-1881,
// 2535-2563), drawing from
//   * PCG32 (cmod/src/centmodule.c:70-98) through rk_poisson (:680-782), and
//   * MT19937 with GSL seeding through the Marsaglia polar gaussian (GSL's
//     gsl_ran_gaussian, third-party; restated from the published method)
// and applying readCCD's read noise and threshold (:785-817).  One GPU thread
// per reference thread: the streams are sequential by construction.
//
// This file is compiled with -fmad=false so every float/double operation is
// rounded exactly where the reference's C expression rounds it.
#include <stdint.h>

#include "refnoise.h"
#include "shwfs_dev.cuh"

namespace shwfs {

__device__ __forceinline__ uint32_t pcg32_next(RefRng& r) {
  uint64_t old = r.pcg_state;
  r.pcg_state = old * 6364136223846793005ULL + r.pcg_inc;
  uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((-rot) & 31));
}

__device__ __forceinline__ float rk_float(RefRng& r) {
  return (float)((double)pcg32_next(r) * 2.3283064365386963e-10);
}

__device__ double loggam_ref(double x) {
  float x0, x2, xp, gl, gl0;
  long k, n;
  const float a[10] = {(float)8.333333333333333e-02, (float)-2.777777777777778e-03,
                       (float)7.936507936507937e-04, (float)-5.952380952380952e-04,
                       (float)8.417508417508418e-04, (float)-1.917526917526918e-03,
                       (float)6.410256410256410e-03, (float)-2.955065359477124e-02,
                       (float)1.796443723688307e-01, (float)-1.39243221690590e+00};
  x0 = (float)x;
  n = 0;
  if ((x == 1.0) || (x == 2.0)) return 0.0;
  if (x <= 7.0) {
    n = (long)(7 - x);
    x0 = (float)(x + n);
  }
  x2 = (float)(1.0 / (double)(x0 * x0));
  xp = (float)(2 * 3.14159265358979323846);
  gl0 = a[9];
  for (k = 8; k >= 0; k--) {
    gl0 *= x2;
    gl0 += a[k];
  }
  gl = (float)((double)(gl0 / x0) + 0.5 * (double)logf(xp) + ((double)x0 - 0.5) * (double)logf(x0) - (double)x0);
  if (x <= 7.0) {
    for (k = 1; k <= n; k++) {
      gl -= logf((float)((double)x0 - 1.0));
      x0 = (float)((double)x0 - 1.0);
    }
  }
  return gl;
}

__device__ long poisson_ptrs_ref(RefRng& st, float lam, int* guard) {
  long k;
  float U, V, slam, loglam, a, b, invalpha, vr, us;
  slam = sqrtf(lam);
  loglam = logf(lam);
  b = (float)(0.931 + 2.53 * (double)slam);
  a = (float)(-0.059 + 0.02483 * (double)b);
  invalpha = (float)(1.1239 + 1.1328 / ((double)b - 3.4));
  vr = (float)(0.9277 - 3.6224 / (double)(b - 2.0f));
  for (int it = 0; it < 100000; it++) {
    U = (float)((double)rk_float(st) - 0.5);
    V = rk_float(st);
    us = (float)(0.5 - (double)fabsf(U));
    k = (long)floorf((float)((double)((2 * a / us + b) * U + lam) + 0.43));
    if (((double)us >= 0.07) && (V <= vr)) return k;
    if ((k < 0) || (((double)us < 0.013) && (V > us))) continue;
    if ((double)(logf(V) + logf(invalpha) - logf(a / (us * us) + b)) <=
        (double)(-lam + (float)k * loglam) - loggam_ref((double)(k + 1)))
      return k;
  }
  *guard = 1;  // iteration limit reached: reported to the host
  return (long)lam;
}

__device__ long poisson_ref(RefRng& st, float lam, int* guard) {
  if (lam >= 10) return poisson_ptrs_ref(st, lam, guard);
  if (lam == 0) return 0;
  long X = 0;
  float prod = 1.f, enlam = expf(-lam);
  do {
    prod *= rk_float(st);
    X++;
  } while (prod > enlam && X < 100000);
  return X - 1;
}

__device__ uint32_t mt_next(RefRng& s) {
  const uint32_t UPPER = 0x80000000u, LOWER = 0x7fffffffu;
  uint32_t y;
  if (s.mti >= kMtN) {
    int kk;
    for (kk = 0; kk < kMtN - kMtM; kk++) {
      y = (s.mt[kk] & UPPER) | (s.mt[kk + 1] & LOWER);
      s.mt[kk] = s.mt[kk + kMtM] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    for (; kk < kMtN - 1; kk++) {
      y = (s.mt[kk] & UPPER) | (s.mt[kk + 1] & LOWER);
      s.mt[kk] = s.mt[kk + (kMtM - kMtN)] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    y = (s.mt[kMtN - 1] & UPPER) | (s.mt[0] & LOWER);
    s.mt[kMtN - 1] = s.mt[kMtM - 1] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    s.mti = 0;
  }
  y = s.mt[s.mti++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

__device__ double gaussian_ref(RefRng& s, double sigma) {
  double x, y, r2;
  int it = 0;
  do {
    double u;
    do { u = (double)mt_next(s) / 4294967296.0; } while (u == 0);
    x = -1 + 2 * u;
    do { u = (double)mt_next(s) / 4294967296.0; } while (u == 0);
    y = -1 + 2 * u;
    r2 = x * x + y * y;
  } while ((r2 > 1.0 || r2 == 0) && ++it < 100000);
  return sigma * y * sqrt(-2.0 * log(r2) / r2);
}

__device__ void readccd_ref(RefRng& s, float* d, int n, float mean, float rn, float fl, int tt) {
  for (int i = 0; i < n; i++) {
    float v = d[i];
    if (rn == 0) {
      v += mean;
    } else {
      v += (float)gaussian_ref(s, (double)rn) + mean;
    }
    if (tt == 0)
      v = v < fl ? 0.f : v - fl;
    else if (tt == 1)
      v = v < fl ? 0.f : v;
    d[i] = v;
  }
}

__global__ void refnoise_walker_kernel(RefNoiseArgs a, RefRng* rng, int* status) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.nthreads) return;
  RefRng& st = rng[t];
  const int mm = a.m * a.m;
  const float rn = a.calsource == 0 ? a.readNoise : 0.f;
  const bool pois = a.addPoisson == 1 && a.calsource == 0;
  int guard = 0;
  for (int i = a.subapStart[t]; i < a.subapStart[t + 1]; i++) {
    float* img = a.bimg + (long long)i * mm;
    if (a.subflag[i] == 1) {
      // centroidsFromImage: readCCD without noise on lit subapertures (no draws)
      if (a.imageInput) continue;
      if (pois && a.poisFlag[i])
        for (int k = 0; k < a.nexp; k++) img[k] = (float)poisson_ref(st, img[k], &guard);
      readccd_ref(st, img, a.nexp, a.readBg, rn, a.floorv, a.threshType);
    } else if (a.imageOnly != 0) {
      for (int k = 0; k < mm; k++) img[k] = 0.f;
      readccd_ref(st, img, mm, a.readBg, rn, a.floorv, a.threshType);
    }
  }
  if (guard) atomicOr(status, 1);
}

cudaError_t launch_refnoise(const RefNoiseArgs& a, RefRng* rng, int* status, cudaStream_t stream) {
  const int threads = 32;
  const int blocks = (a.nthreads + threads - 1) / threads;
  refnoise_walker_kernel<<<blocks, threads, 0, stream>>>(a, rng, status);
  return cudaGetLastError();
}

__global__ void pois_flag_kernel(int nsubaps, const float* __restrict__ totsig, const float* __restrict__ frac,
                                 float sky, int skyArr, unsigned char* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nsubaps) flag[i] = totsig[i] > 0.f || sky * frac[i] > 0.f || skyArr != 0;
}

cudaError_t launch_pois_flag(int nsubaps, const float* totsig, const float* frac, float sky, int skyArr,
                             unsigned char* poisFlag, cudaStream_t stream) {
  pois_flag_kernel<<<(nsubaps + 255) / 256, 256, 0, stream>>>(nsubaps, totsig, frac, sky, skyArr, poisFlag);
  return cudaGetLastError();
}

__global__ void inject_noise_kernel(const InjectArgs a) {
  const long long mm = (long long)a.m * a.m;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= mm * a.nsubaps) return;
  const int i = (int)(k / mm);
  const float rn = a.calsource == 0 ? a.readNoise : 0.f;
  float v;
  if (a.subflag[i] == 1) {
    v = a.bimg[k];
    if (a.addPoisson == 1 && a.calsource == 0 && a.poisFlag[i]) v = a.shot[k];
  } else if (a.imageOnly != 0) {
    v = 0.f;
  } else {
    return;
  }
  // readCCD: data += (float)gaussian + noiseMean, or data += noiseMean
  if (rn == 0.f)
    v += a.readBg;
  else
    v += a.readn[k] + a.readBg;
  if (a.threshType == 0)
    v = v < a.floorv ? 0.f : v - a.floorv;
  else if (a.threshType == 1)
    v = v < a.floorv ? 0.f : v;
  a.bimg[k] = v;
}

cudaError_t launch_inject_noise(const InjectArgs& a, cudaStream_t stream) {
  const long long n = (long long)a.m * a.m * a.nsubaps;
  if (n == 0) return cudaSuccess;
  inject_noise_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace shwfs
