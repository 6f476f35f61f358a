// Unlit-subaperture kernel of the WFS step.
#include <algorithm>
#include <cstring>

#include "wfs_plain.cuh"

namespace shwfs {

// Unlit subapertures on a readout frame (cmod/src/centmodule.c:1964-1981):
// centroids zeroed, or with imageOnly a noise-only image.
__global__ void wfs_unlit_kernel(const WfsArgs a, const int* unlit, int nunlit) {
  const int mm = a.m * a.m;
  const long long total = (long long)nunlit * a.nframes * (a.imageOnly ? mm : 1);
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < total;
       w += (long long)gridDim.x * blockDim.x) {
    if (!a.imageOnly) {
      const int f = (int)(w / nunlit), i = unlit[w % nunlit];
      float* c = a.cents + (long long)f * a.centsFrameStride;
      c[2 * i] = 0.f;
      c[2 * i + 1] = 0.f;
    } else {
      const long long q = w / mm;
      const int pix = (int)(w - q * mm);
      const int f = (int)(q / nunlit), i = unlit[q % nunlit];
      float v = a.readBg;
      const float rn = a.calsource == 0 ? a.readNoise : 0.f;
      if (rn != 0.f) {
        CounterStream st(a.seed, frame_base(a) + f, i, pix, 1);
        v = rn * normal_counter(st) + a.readBg;
      }
      a.bimg[(long long)f * a.bimgFrameStride + (long long)i * mm + pix] = threshold_px(v, a.floorv, a.threshType);
    }
  }
}

// Copy the images of the listed subapertures from the device mirror to the
// caller's host array (pinned and mapped, written through its device alias).
__global__ void publish_subaps_kernel(const float* __restrict__ src, float* dst, const int* __restrict__ list, int n,
                                      int mm) {
  const long long total = (long long)n * mm;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < total;
       w += (long long)gridDim.x * blockDim.x) {
    const long long k = w / mm;
    const long long off = (long long)list[k] * mm + (w - k * mm);
    dst[off] = src[off];
  }
}

cudaError_t launch_publish(const float* src, float* dst, const int* list, int n, int mm, cudaStream_t stream) {
  const long long total = (long long)n * mm;
  if (total == 0) return cudaSuccess;
  const int blocks = (int)((total + 255) / 256 < 2048 ? (total + 255) / 256 : 2048);
  publish_subaps_kernel<<<blocks, 256, 0, stream>>>(src, dst, list, n, mm);
  return cudaGetLastError();
}

// advance the device frame counters of a graph's handles (one per handle)
__global__ void bump_counters_kernel(unsigned long long* const* ctrs, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ctrs[i][0] += 1ull;
}

cudaError_t launch_bump_counters(unsigned long long* const* ctrs, int n, cudaStream_t stream) {
  bump_counters_kernel<<<(n + 127) / 128, 128, 0, stream>>>(ctrs, n);
  return cudaGetLastError();
}

__global__ void set_counter_kernel(unsigned long long* ctr, unsigned long long v) { *ctr = v; }

cudaError_t launch_set_counter(unsigned long long* ctr, unsigned long long v, cudaStream_t stream) {
  set_counter_kernel<<<1, 1, 0, stream>>>(ctr, v);
  return cudaGetLastError();
}

// n draws of the counter-based noise, element i as the pipeline draws pixel
// i & 0xffff of subaperture i >> 16 in frame `frame` (one thread per quad of
// four elements): kind 1 its read-noise normal (quad_normals), kind 2 its
// Poisson(lam[i]) shot noise (quad_poisson below lambda 64, ptrs_pixel
// above); kind 0 Poisson(lam[i]) by the table-free modal inversion / PTRS
// from the element's own stream (seed, frame, i >> 16, i & 0xffff, purpose
// 2), an independent sampler kept to cross-check kind 2
__global__ void sample_noise_kernel(const float* __restrict__ lam, long long n, const PhiloxKeys keys,
                                    unsigned long long seed, unsigned long long frame, int kind,
                                    float* __restrict__ out, const PoisTab* __restrict__ tab) {
  const long long nq = (n + 3) >> 2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nq; t += (long long)gridDim.x * blockDim.x) {
    const long long i0 = 4 * t;
    const int np = (int)(n - i0 < 4 ? n - i0 : 4);
    const uint32_t subap = (uint32_t)(i0 >> 16), pix0 = (uint32_t)(i0 & 0xffff), fr = (uint32_t)frame;
    float v[4];
    if (kind == 0) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        v[k] = 0.f;
        if (k < np) {
          CounterStream st(seed, frame, (int)subap, (int)(pix0 + k), 2);
          v[k] = poisson_counter(st, lam[i0 + k]);
        }
      }
    } else if (kind == 1) {
      quad_normals(keys, fr, subap, pix0 >> 2, v);
    } else {
      unsigned bm = 0;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        v[k] = k < np ? lam[i0 + k] : 0.f;
        if (v[k] >= kModalMaxLam) bm |= 1u << k;
      }
      quad_poisson(keys, fr, subap, pix0 >> 2, *tab, v, bm);
#pragma unroll
      for (int k = 0; k < 4; k++)
        if ((bm >> k) & 1u) v[k] = ptrs_pixel(keys, fr, subap, pix0 + k, v[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (k < np) out[i0 + k] = v[k];
  }
}

cudaError_t launch_sample_noise(const float* lam, long long n, unsigned long long seed, unsigned long long frame,
                                int kind, float* out, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const PoisTab* tab = nullptr;
  if (kind == 2) {
    cudaError_t e = pois_table_device(&tab);
    if (e != cudaSuccess) return e;
  }
  WfsArgs tmp;
  memset(&tmp, 0, sizeof(tmp));
  tmp.seed = seed;
  set_philox_keys(tmp);
  const long long nq = (n + 3) / 4;
  const long long blocks = (nq + 255) / 256 < 152 * 16 ? (nq + 255) / 256 : 152 * 16;
  sample_noise_kernel<<<(int)blocks, 256, 0, stream>>>(lam, n, tmp.philoxKeys, seed, frame, kind, out, tab);
  return cudaGetLastError();
}

cudaError_t launch_unlit(const WfsArgs& a, const int* unlit, int nunlit, cudaStream_t stream) {
  const long long total = (long long)nunlit * a.nframes * (a.imageOnly ? a.m * a.m : 1);
  if (total == 0) return cudaSuccess;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  wfs_unlit_kernel<<<blocks, 256, 0, stream>>>(a, unlit, nunlit);
  return cudaGetLastError();
}

__global__ void accumulate_kernel(float* __restrict__ acc, const float* __restrict__ sub, long long n, int first,
                                  float scale) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    float v = first ? sub[k] : acc[k] + sub[k];
    if (scale != 1.0f) v *= scale;
    acc[k] = v;
  }
}

cudaError_t launch_accumulate(float* acc, const float* sub, long long n, int first, float scale, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = std::min<long long>((n + 255) / 256, 4096);
  accumulate_kernel<<<(unsigned)blocks, 256, 0, stream>>>(acc, sub, n, first, scale);
  return cudaGetLastError();
}

}  // namespace shwfs
