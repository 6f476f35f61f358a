// Noise, threshold and post stages of the GEMM-DFT form.
//
// The tensor-core kernel (wfs_gemm.cu) leaves each lit subaperture-frame's
// normalised pre-noise image in bimg; this kernel adds the counter-based
// Poisson and read noise, thresholds (cmod/src/centmodule.c:1874-1882,
// 785-817) and runs the shared post stages (post_tile: brightest pixels,
// pixel power, bimg write, centroids, calibration, references).  Each quad
// of pixels draws from the same (seed, frame, subaperture, quad) stream as
// in the fused FP32 kernel, so equal pre-noise images give equal noisy
// images.
//
// A separate launch rather than a stage of the tensor-core kernel: the noise
// samplers are latency-bound scalar code that wants many resident warps,
// while the tensor-core kernel holds one 608-thread CTA per SM.
#include <algorithm>

#include "gemm_form.h"
#include "wfs_plain.cuh"

namespace shwfs {

namespace {

constexpr int kPostThreads = 256;
constexpr int kPostMaxTS = 64;
constexpr int kPostBright = 512;  // queued bright pixels per tile (overflow: drawn in place)

// three CTAs per SM: a tile's images (up to 32 KB) and the Poisson table
// (22 KB) in shared memory allow no more
__global__ void __launch_bounds__(kPostThreads, 3) wfs_post_kernel(const WfsArgs a, const PoisTab* __restrict__ tab) {
  extern __shared__ __align__(16) float smem_post[];
  __shared__ int s_subap[kPostMaxTS];
  __shared__ int s_frame[kPostMaxTS];
  __shared__ unsigned char s_pflag[kPostMaxTS];
  __shared__ int s_nbright;
  __shared__ int s_bright[kPostBright];
  __shared__ float s_brightv[kPostBright];
  const int tid = threadIdx.x;
  // the image-formation kernel before this one has completed (stream order)
  if (a.statusOut && blockIdx.x == 0 && tid == 0) *(volatile int*)a.statusOut = *(const volatile int*)a.statusIn;
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
    // threshold [, power, bimg write] of pixel pix of tile item s, value v
    // after the noise
    auto store = [&](int s, int pix, float v) {
      if (simple) {
        // pixel power and the bimg write of post_tile's stage 8, here
        if (a.pxlPower == 2.f)
          v = v * v;
        else if (a.pxlPower != 1.f && a.pxlPower != 0.f)
          v = powf(v, a.pxlPower);
        a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)s_subap[s] * mm + pix] = v;
      }
      imgs[s * mm + pix] = v;
    };
    auto finish = [&](float v, float g) {
      if (noise) {
        v += rn * g + a.readBg;
        v = threshold_px(v, a.floorv, a.threshType);
      }
      return v;
    };
    // one lane per quad of pixels (quad_normals, quad_poisson).  Pixels
    // whose Poisson mean needs the rejection sampler (lambda >= 64) are
    // queued and drawn afterwards with the whole CTA, so that one bright
    // pixel does not hold the other 31 lanes of its warp (same streams, same
    // draws).
    const int nqi = (mm + 3) >> 2;
    const float inv_nqi = 1.0f / (float)nqi;
    for (int wq = tid; wq < ns * nqi; wq += blockDim.x) {
      const int s = div_small(wq, nqi, inv_nqi), qd = wq - s * nqi;
      const int p0 = 4 * qd, np = min(4, mm - p0);
      const int i = s_subap[s];
      const uint32_t fr = (uint32_t)(fbase + s_frame[s]);
      float v[4];
#pragma unroll
      for (int k = 0; k < 4; k++) v[k] = k < np ? imgs[s * mm + p0 + k] : 0.f;
      unsigned bm = 0;  // bright pixels, queued
      float g[4] = {0.f, 0.f, 0.f, 0.f};
      if (noise) {
        if (pois && s_pflag[s]) {
          unsigned inplace = 0;  // bright pixels past the queue's end
#pragma unroll
          for (int k = 0; k < 4; k++) {
            if (k < np && v[k] >= kModalMaxLam) {
              const int slot = atomicAdd(&s_nbright, 1);
              if (slot < kPostBright) {
                s_bright[slot] = s * mm + p0 + k;
                s_brightv[slot] = v[k];
                bm |= 1u << k;
              } else {
                inplace |= 1u << k;
              }
            }
          }
          quad_poisson(a.philoxKeys, fr, (uint32_t)i, (uint32_t)qd, *s_tab, v, bm | inplace);
#pragma unroll
          for (int k = 0; k < 4; k++)
            if ((inplace >> k) & 1u) v[k] = ptrs_pixel_cold(a.seed, fr, (uint32_t)i, (uint32_t)(p0 + k), v[k]);
        }
        if (rn != 0.f) quad_normals(a.philoxKeys, fr, (uint32_t)i, (uint32_t)qd, g);
      }
#pragma unroll
      for (int k = 0; k < 4; k++)
        if (k < np && !((bm >> k) & 1u)) store(s, p0 + k, finish(v[k], g[k]));
    }
    __syncthreads();
    const int nb = min(s_nbright, kPostBright);
    for (int k = tid; k < nb; k += blockDim.x) {
      const int w = s_bright[k];
      const int s = div_small(w, mm, inv_mm), pix = w - s * mm;
      const int i = s_subap[s];
      const uint32_t fr = (uint32_t)(fbase + s_frame[s]);
      const float g = rn != 0.f ? pixel_normal(a.philoxKeys, fr, (uint32_t)i, (uint32_t)pix) : 0.f;
      store(s, pix, finish(ptrs_pixel(a.philoxKeys, fr, (uint32_t)i, (uint32_t)pix, s_brightv[k]), g));
    }
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

constexpr int kWarpThreads = 256;  // 8 warps per CTA
constexpr int kWarpQ = 160;        // queued bright pixels per warp (at most 32 + one round's 128); even
constexpr int kWarpMaxK = 16;      // subaperture-frames per chunk

// Per-warp shared memory: two pixel buffers of bufPx floats (the chunk being
// drawn and the next one, copied in asynchronously), the chunk's item table
// for both buffers (per item an int4 {subaperture, noise frame index,
// Poisson flag, frame} and the 64-bit offset of its image in bimg), the
// window-row partial sums of the centroids and the bright-pixel queue
// (kWarpQ 16-bit indices into the chunk's buffer).
__host__ __device__ inline int warp_smem_floats(int bufPx, int ncen) {
  return 2 * bufPx + 2 * 6 * kWarpMaxK + 2 * kWarpMaxK * ncen + kWarpQ / 2;
}

// The common configuration (window CoG or image only; no brightest-pixel
// selection, fit or optical binning), one warp per chunk of K consecutive
// lit subaperture-frames: the chunk's pixels are drawn a quad (four
// consecutive pixels of one image) per lane, lanes over the chunk's
// flattened quad index (every lane busy whatever nimg is), with 16-byte
// loads and stores when nimg^2 is a multiple of 4.  Bright pixels
// (lambda >= 64, the rejection sampler) are queued and drawn by the whole
// warp after a round that left more than 32 in the queue and after the
// last, then the window centroids come from the chunk's images in shared
// memory.  Warps are independent (no block barrier after the table load);
// each copies its next chunk into shared memory with cp.async while it
// draws the current one.  Unlit subapertures are not visited; their
// centroids are zeroed at the end (zeroUnlit).  Pixels and streams are
// those of wfs_post_kernel and of the fused FP32 kernel (quad_normals,
// quad_poisson, ptrs_pixel), so equal pre-noise images give equal noisy
// images in every form.  RN (read noise on) and POIS (Poisson on) are
// compile-time.
template <bool RN, bool POIS>
__global__ void __launch_bounds__(kWarpThreads, 3)
    wfs_post_warp_kernel(const WfsArgs a, const PoisTab* __restrict__ tab, int K, int bufPx) {
  extern __shared__ __align__(16) float smem_post[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m = a.m, mm = m * m, ncen = a.ncen;
  const bool cw2d = a.centWeightDim == 2;
  PoisTab* s_tab = reinterpret_cast<PoisTab*>(smem_post);
  float* s_cw = smem_post + (POIS ? sizeof(PoisTab) / sizeof(float) : 0);
  float* wbase = s_cw + ((cw2d ? mm : 0) + 3) / 4 * 4 + warp * warp_smem_floats(bufPx, ncen);
  // buffer b: pixels wbase + b * bufPx, items item0 + b * kWarpMaxK, image
  // offsets off0 + b * kWarpMaxK
  int4* item0 = reinterpret_cast<int4*>(wbase + 2 * bufPx);
  long long* off0 = reinterpret_cast<long long*>(item0 + 2 * kWarpMaxK);
  float* s_rows = wbase + 2 * bufPx + 12 * kWarpMaxK;
  // queued pixels as 16-bit indices into the chunk's buffer (bufPx <= 3200:
  // the launcher's 200 KB bound on 16 buffers of bufPx floats)
  unsigned short* q_idx = reinterpret_cast<unsigned short*>(s_rows + 2 * kWarpMaxK * ncen);
  if constexpr (POIS) {
    const int4* src = reinterpret_cast<const int4*>(tab);
    int4* dst = reinterpret_cast<int4*>(s_tab);
    for (int k = tid; k < (int)(sizeof(PoisTab) / sizeof(int4)); k += blockDim.x) dst[k] = src[k];
  }
  if (cw2d)
    for (int k = tid; k < mm; k += blockDim.x) s_cw[k] = a.centWeight[k];
  __syncthreads();
  // launched programmatically behind the image-formation kernel: everything
  // above reads constants only; bimg is read after that grid has completed
  // and its writes are visible (a no-op for an ordinary launch)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (a.statusOut && blockIdx.x == 0 && tid == 0) *(volatile int*)a.statusOut = *(const volatile int*)a.statusIn;

  const long long items = (long long)a.nlit * a.nframes;
  const long long nchunks = (items + K - 1) / K;
  const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + warp, nw = (long long)gridDim.x * (blockDim.x >> 5);
  const bool noise = a.mode & kNoiseCounter;
  const float rn = a.readNoise;
  const unsigned long long fbase = frame_base(a);
  const bool vec = (mm & 3) == 0 && (a.bimgFrameStride & 3) == 0 && ((uintptr_t)a.bimg & 15) == 0;
  const bool cents = a.imageOnly == 0 && !a.skipCents;
  const int sx0 = (m - ncen) / 2;
  const float inv_mm = 1.0f / (float)mm, inv_nc = 1.0f / (float)ncen;
  // readCCD's threshold (cmod/src/centmodule.c:785-817) without branches:
  // type 0 subtracts the floor, type 1 keeps the value, other types leave
  // the pixel as it is
  const float thr = (a.threshType == 0 || a.threshType == 1) ? a.floorv : -INFINITY;
  const float tsub = a.threshType == 0 ? a.floorv : 0.f;
  const bool pw1 = a.pxlPower == 1.f || a.pxlPower == 0.f;
  const bool out2 = a.bimgOut != nullptr;
  // whole quads with 16-byte loads and stores
  const bool vec4 = (mm & 3) == 0 && (a.bimgFrameStride & 3) == 0 && ((uintptr_t)a.bimg & 15) == 0 &&
                    (!out2 || ((uintptr_t)a.bimgOut & 15) == 0);

  // item table of chunk c into buffer b's table (lanes < K), then its
  // pixels into buffer b with cp.async (one commit group per lane, empty
  // past the end)
  // the first item of this warp's current chunk as (frame cf, lit index
  // cl), advanced by whole strides of nw chunks without a division
  long long cf = (gw * K) / a.nlit;
  int cl = (int)(gw * K - cf * a.nlit);
  const long long strideItems = nw * (long long)K;
  const long long sf = strideItems / a.nlit;
  const int sl = (int)(strideItems - sf * a.nlit);
  auto issue = [&](long long c, int b, long long f0, int l0) {
    int4* itb = item0 + b * kWarpMaxK;
    long long* ofb = off0 + b * kWarpMaxK;
    if (c < nchunks) {
      const long long w0 = c * K;
      const int nk = (int)min((long long)K, items - w0);
      if (lane < nk) {
        int li = l0 + lane, f = (int)f0;
        while (li >= a.nlit) {
          li -= a.nlit;
          f++;
        }
        const int i = a.lit[li];
        const int pf = POIS ? (a.totsig[i] > 0.f || a.sky * a.frac[i] > 0.f || a.skyArr != nullptr) : 0;
        itb[lane] = make_int4(i, (int)(uint32_t)(fbase + (unsigned long long)f), pf, f);
        ofb[lane] = (long long)f * a.bimgFrameStride + (long long)i * mm;
      }
      __syncwarp();
      float* dst = wbase + b * bufPx;
      if (vec) {
        const int nq = nk * mm / 4, q4 = mm / 4;
        const float inv_q4 = 1.0f / (float)q4;
        for (int q = lane; q < nq; q += 32) {
          const int s = div_small(q, q4, inv_q4), r = q - s * q4;
          const float* src = a.bimg + ofb[s] + 4 * r;
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst + 4 * q)),
                       "l"(src)
                       : "memory");
        }
      } else {
        for (int g = lane; g < nk * mm; g += 32) {
          const int s = div_small(g, mm, inv_mm), pix = g - s * mm;
          const float* src = a.bimg + ofb[s] + pix;
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst + g)),
                       "l"(src)
                       : "memory");
        }
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  int b = 0;
  issue(gw, 0, cf, cl);
  for (long long c = gw; c < nchunks; c += nw, b ^= 1) {
    const long long w0 = c * K;
    const int nk = (int)min((long long)K, items - w0);
    cf += sf;  // the next chunk of this warp
    cl += sl;
    if (cl >= a.nlit) {
      cl -= a.nlit;
      cf++;
    }
    issue(c + nw, b ^ 1, cf, cl);  // the next chunk's copies, in flight while this one is drawn
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    __syncwarp();
    float* img = wbase + b * bufPx;
    const int4* items = item0 + b * kWarpMaxK;
    const long long* offs = off0 + b * kWarpMaxK;
    // noise, threshold, power and stores of one pixel (x: its mean; g: its
    // read-noise normal)
    auto finish = [&](float x, float g) {
      if constexpr (RN)
        x += rn * g + a.readBg;
      else
        x += a.readBg;
      x = x < thr ? 0.f : x - tsub;
      if (!pw1) x = a.pxlPower == 2.f ? x * x : powf(x, a.pxlPower);
      return x;
    };
    int nq = 0;  // bright pixels queued (warp-uniform)
    const int nqi = (mm + 3) >> 2, nqc = nk * nqi;  // quads per item, per chunk
    // this lane's quad Q = Q0 + lane of the chunk is quad q of item s
    int s = 0, q = lane;
    while (q >= nqi) {
      q -= nqi;
      s++;
    }
    // one round of 32 quads (the last may be partial)
    auto round = [&](int Q0) {
      const bool in = Q0 + lane < nqc;
      const int si = in ? s : 0;
      const int4 it = items[si];
      (void)it;  // unused without noise
      const int p0 = 4 * q, np = in ? min(4, mm - p0) : 0;
      float* src = img + si * mm + p0;
      float v[4];
      if (vec4 && in) {
        const float4 t = *reinterpret_cast<const float4*>(src);
        v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
      } else {
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = k < np ? src[k] : 0.f;
      }
      unsigned bmask = 0;  // pixels with lambda >= 64, queued
      if constexpr (POIS) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const bool br = noise && k < np && it.z && v[k] >= kModalMaxLam;
          const unsigned bm = __ballot_sync(0xffffffffu, br);
          if (bm) {
            if (br) {
              bmask |= 1u << k;
              const int slot = nq + __popc(bm & ((1u << lane) - 1u));
              q_idx[slot] = (unsigned short)(si * mm + p0 + k);
            }
            nq += __popc(bm);
          }
        }
      }
      if (noise && in) {
        float g[4] = {0.f, 0.f, 0.f, 0.f};
        if constexpr (RN) quad_normals(a.philoxKeys, (uint32_t)it.y, (uint32_t)it.x, (uint32_t)q, g);
        if constexpr (POIS) {
          if (it.z) {
            quad_poisson(a.philoxKeys, (uint32_t)it.y, (uint32_t)it.x, (uint32_t)q, *s_tab, v, bmask);
          }
        }
        // a queued pixel keeps its mean (in img too) until the drain
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float x = finish(v[k], g[k]);
          v[k] = ((bmask >> k) & 1u) ? v[k] : x;
        }
      } else if (!pw1) {
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = a.pxlPower == 2.f ? v[k] * v[k] : powf(v[k], a.pxlPower);
      }
      if (in) {
        const long long ob = offs[si] + p0;
        // (queued pixels too: the drain overwrites them after a __syncwarp)
        if (vec4) {
          const float4 t = make_float4(v[0], v[1], v[2], v[3]);
          *reinterpret_cast<float4*>(a.bimg + ob) = t;
          if (out2) *reinterpret_cast<float4*>(a.bimgOut + ob) = t;
          if (cents) *reinterpret_cast<float4*>(src) = t;
        } else {
#pragma unroll
          for (int k = 0; k < 4; k++) {
            if (k < np) {
              a.bimg[ob + k] = v[k];
              if (out2) a.bimgOut[ob + k] = v[k];
              if (cents) src[k] = v[k];
            }
          }
        }
      }
      q += 32;
      while (q >= nqi) {
        q -= nqi;
        s++;
      }
    };
    // the queued bright pixels, drawn by the whole warp: after a round that
    // left more than 32 (a round queues at most 128) and after the last round
    auto drain = [&]() {
      __syncwarp();
      for (int k = lane; k < nq; k += 32) {
        const int g = q_idx[k];
        const int sq = div_small(g, mm, inv_mm), pq = g - sq * mm;
        const int4 it = items[sq];
        float gn = 0.f;
        if constexpr (RN) gn = pixel_normal(a.philoxKeys, (uint32_t)it.y, (uint32_t)it.x, (uint32_t)pq);
        const float x = finish(ptrs_pixel(a.philoxKeys, (uint32_t)it.y, (uint32_t)it.x, (uint32_t)pq, img[g]), gn);
        a.bimg[offs[sq] + pq] = x;
        if (out2) a.bimgOut[offs[sq] + pq] = x;
        if (cents) img[g] = x;
      }
      nq = 0;
      __syncwarp();
    };
    // one copy of each in the loop: the samplers' code is large, and a
    // second copy of either (a separate last round, a drain after the loop)
    // overflowed the instruction cache
    for (int Q0 = 0; Q0 < nqc; Q0 += 32) {
      round(Q0);
      if constexpr (POIS)
        if (nq > kWarpQ - 128 || (nq && Q0 + 32 >= nqc)) drain();
    }
    if (cents) {
      __syncwarp();
      // centred-window CoG: sums of each window row (one lane per item
      // row), then of the rows (one lane per item), in a fixed order
      for (int t = lane; t < nk * ncen; t += 32) {
        const int s = div_small(t, ncen, inv_nc), rr = t - s * ncen;
        const int r = sx0 + rr;
        const float* row = img + s * mm + r * m + sx0;
        const float* wrow = cw2d ? s_cw + r * m + sx0
                                 : (a.centWeightDim == 4 ? a.centWeight + (long long)items[s].x * mm + r * m + sx0 : nullptr);
        float ps = 0.f, px = 0.f;
        if (wrow) {
          for (int c2 = 0; c2 < ncen; c2++) {
            const float v = row[c2] * wrow[c2];
            ps += v;
            px += v * (float)(sx0 + c2);
          }
        } else {
          for (int c2 = 0; c2 < ncen; c2++) {
            const float v = row[c2];
            ps += v;
            px += v * (float)(sx0 + c2);
          }
        }
        s_rows[2 * t] = ps;
        s_rows[2 * t + 1] = px;
      }
      __syncwarp();
      if (lane < nk) {
        float sum = 0.f, sxv = 0.f, syv = 0.f;
        for (int rr = 0; rr < ncen; rr++) {
          const float ps = s_rows[2 * (lane * ncen + rr)];
          sum += ps;
          sxv += s_rows[2 * (lane * ncen + rr) + 1];
          syv += ps * (float)(sx0 + rr);
        }
        float cx = 0.f, cy = 0.f;
        if (sum > 0.f) {
          cx = sxv / sum - 0.5f * (float)(m - 1);
          cy = syv / sum - 0.5f * (float)(m - 1);
        }
        calibrate_and_store(a, items[lane].x, items[lane].w, cx, cy);
      }
    }
    __syncwarp();  // every lane is done with buffer b before it is refilled
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (a.zeroUnlit) {
    // unlit subapertures: centroids 0 (cmod/src/centmodule.c:1964-1981)
    const long long nu = (long long)a.nunlit * a.nframes;
    for (long long u = (long long)blockIdx.x * blockDim.x + tid; u < nu; u += (long long)gridDim.x * blockDim.x) {
      const int f = (int)(u / a.nunlit), i = a.unlit[u - (long long)f * a.nunlit];
      float* c = a.cents + (long long)f * a.centsFrameStride + 2LL * i;
      c[0] = 0.f;
      c[1] = 0.f;
    }
  }
}

}  // namespace

cudaError_t launch_post(const WfsArgs& a0, int numSMs, cudaStream_t stream, unsigned* done) {
  WfsArgs a = a0;
  a.zeroUnlit = 0;
  if (done) *done = 0;
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
  const bool simple = !(a.calsource == 0 && (a.useBrightest != 0 || a.useBrightestArr)) && a.opticalBinning != 1 &&
                      a.fitSize == 0 && a.gaussianFit <= 0 && a.cob == 0;
  const int tabB = pois ? (int)sizeof(PoisTab) : 0;
  const int cwB = ((a.centWeightDim == 2 ? mm : 0) + 3) / 4 * 16;
  const int bufPx = (std::max(512, mm) + 3) / 4 * 4;
  const int warpB = warp_smem_floats(bufPx, a.ncen) * (int)sizeof(float);
  const int wsmem = tabB + cwB + (kWarpThreads / 32) * warpB;
  if (simple && a.ncen >= 1 && wsmem <= 200 * 1024) {
    const bool rnOn = a.calsource == 0 && a.readNoise != 0.f;
    auto kern = pois ? (rnOn ? wfs_post_warp_kernel<true, true> : wfs_post_warp_kernel<false, true>)
                     : (rnOn ? wfs_post_warp_kernel<true, false> : wfs_post_warp_kernel<false, false>);
    if (a.calsource != 0) a.readNoise = 0.f;
    int ctas = 0;
    cudaError_t e = kernel_smem_setup((const void*)kern, wsmem, kWarpThreads, &ctas);
    if (e != cudaSuccess) return e;
    if (ctas < 1) return cudaErrorInvalidConfiguration;
    const long long cap = (long long)numSMs * ctas;
    const long long warps = cap * (kWarpThreads / 32);
    // chunk size: as many items as fill the buffer, fewer when that would
    // leave resident warps without a chunk (small batches: latency)
    int K = std::max(1, std::min(kWarpMaxK, bufPx / mm));
    const long long perWarp = (nwork + warps - 1) / warps;
    if (perWarp < K) K = (int)std::max(1LL, perWarp);
    const long long nchunks = (nwork + K - 1) / K;
    const long long needCtas = (nchunks + kWarpThreads / 32 - 1) / (kWarpThreads / 32);
    const int grid = (int)std::max(1LL, std::min(cap, needCtas));
    if (done) {
      if (!a.imageOnly && a.unlit && a.nunlit > 0) {
        a.zeroUnlit = 1;
        *done |= kPostDidUnlit;
      } else if (!a.imageOnly) {
        *done |= kPostDidUnlit;  // nothing unlit to zero
      }
      if (a.bimgOut) *done |= kPostDidOut;
    } else {
      a.bimgOut = nullptr;
    }
    // programmatic launch: CTAs may become resident while the previous
    // kernel of the stream (the image formation) still runs and wait for it
    // in griddepcontrol.wait after loading their tables
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kWarpThreads);
    cfg.dynamicSmemBytes = (size_t)wsmem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const PoisTab* tabArg = pois ? tab : nullptr;
    return cudaLaunchKernelEx(&cfg, kern, a, tabArg, K, bufPx);
  }
  const int smem = (a.TS * mm + (a.centWeightDim == 2 ? mm : 0)) * (int)sizeof(float) +
                   (pois ? (int)sizeof(PoisTab) : 0);
  int ctas = 0;
  cudaError_t e = kernel_smem_setup((const void*)wfs_post_kernel, smem, kPostThreads, &ctas);
  if (e != cudaSuccess) return e;
  if (ctas < 1) return cudaErrorInvalidConfiguration;
  const long long ntiles = (nwork + a.TS - 1) / a.TS;
  const long long cap = (long long)numSMs * ctas;
  const int grid = (int)(ntiles < cap ? ntiles : cap);
  wfs_post_kernel<<<grid, kPostThreads, smem, stream>>>(a, tab);
  return cudaGetLastError();
}

}  // namespace shwfs
