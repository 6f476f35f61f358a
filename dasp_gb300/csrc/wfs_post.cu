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
// while the tensor-core kernel holds one 608-thread CTA per SM.
#include <algorithm>
#include <type_traits>

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

constexpr int kSlotThreads = 512;
constexpr int kSlotCtasPerSM = 2;  // one copy of the Poisson tables per CTA
constexpr int kSlotStages = 2;
constexpr int kSlotMaxTS = 96;

// The common configuration (window CoG or image only; no brightest-pixel
// selection, fit or optical binning) over tiles of TS consecutive
// subaperture slots of one frame: a tile's pixels are one contiguous range
// of bimg, so its copies into shared memory depend on nothing but the tile
// index and run kSlotStages - 1 tiles ahead (cp.async groups), whatever the
// lit pattern.  Unlit slots are copied but neither drawn nor written.
// RN (read noise on) and POIS (Poisson on) are compile-time so that each
// pixel's stream is consumed along a fixed path.  Pixels and streams are
// those of wfs_post_kernel (same images); the window CoG sums each window
// row first (one thread per subaperture row), then the rows.
template <bool RN, bool POIS>
__global__ void __launch_bounds__(kSlotThreads, kSlotCtasPerSM)
    wfs_post_slots_kernel(const WfsArgs a, const PoisTab* __restrict__ tab) {
  extern __shared__ __align__(16) float smem_post[];
  __shared__ int s_nbright[2];  // bright-pixel queue length, alternating between tiles
  __shared__ int s_bright[kPostBright];
  __shared__ float s_brightv[kPostBright];
  const int tid = threadIdx.x;
  const int m = a.m, mm = m * m, TS = a.TS;
  const bool cw2d = a.centWeightDim == 2;
  PoisTab* s_tab = reinterpret_cast<PoisTab*>(smem_post);
  float* s_cw = smem_post + (POIS ? sizeof(PoisTab) / sizeof(float) : 0);
  // per stage: TS*mm pixels, then TS each of totsig, frac, subflag
  float* ring = s_cw + ((cw2d ? mm : 0) + 3) / 4 * 4;
  const int stageFloats = (TS * mm + 3 * TS + 3) / 4 * 4;
  float* s_part = ring + kSlotStages * stageFloats;  // CoG row sums: TS*ncen pairs
  if constexpr (POIS) {
    const int4* src = reinterpret_cast<const int4*>(tab);
    int4* dst = reinterpret_cast<int4*>(s_tab);
    for (int k = tid; k < (int)(sizeof(PoisTab) / sizeof(int4)); k += blockDim.x) dst[k] = src[k];
  }
  if (cw2d)
    for (int k = tid; k < mm; k += blockDim.x) s_cw[k] = a.centWeight[k];
  // launched programmatically behind the image-formation kernel: everything
  // above reads constants only; bimg is read after that grid has completed
  // and its writes are visible (a no-op for an ordinary launch)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (a.statusOut && blockIdx.x == 0 && tid == 0) *(volatile int*)a.statusOut = *(const volatile int*)a.statusIn;

  const int tpf = (a.nsubaps + TS - 1) / TS;  // tiles per frame
  const long long ntiles = (long long)tpf * a.nframes;
  const bool noise = a.mode & kNoiseCounter;
  const float rn = a.readNoise;
  const unsigned long long fbase = frame_base(a);
  const bool vec = (mm & 3) == 0 && (a.bimgFrameStride & 3) == 0 && ((uintptr_t)a.bimg & 15) == 0;
  const bool cents = a.imageOnly == 0 && !a.skipCents;

  // copies of tile t (k-th of this CTA) into stage k % kSlotStages; one
  // cp.async group per tile and thread, empty past the last tile
  auto issue = [&](long long t, int k) {
    if (t < ntiles) {
      float* st = ring + (k % kSlotStages) * stageFloats;
      const int f = (int)(t / tpf), s0 = (int)(t - (long long)f * tpf) * TS;
      const int ns = min(TS, a.nsubaps - s0);
      const float* src = a.bimg + (long long)f * a.bimgFrameStride + (long long)s0 * mm;
      const int n = ns * mm;
      if (vec) {
        for (int c = tid; c < n / 4; c += blockDim.x)
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(st + 4 * c)),
                       "l"(src + 4 * c)
                       : "memory");
      } else {
        for (int c = tid; c < n; c += blockDim.x)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(st + c)),
                       "l"(src + c)
                       : "memory");
      }
      float* info = st + TS * mm;
      for (int c = tid; c < 3 * ns; c += blockDim.x) {
        const int which = c / ns, s = c - which * ns;
        const void* g = which == 0 ? (const void*)(a.totsig + s0 + s)
                                   : (which == 1 ? (const void*)(a.frac + s0 + s) : (const void*)(a.subflag + s0 + s));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(info + which * TS + s)),
                     "l"(g)
                     : "memory");
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  long long t = blockIdx.x;
  int k = 0;
  for (int d = 0; d < kSlotStages - 1; d++) issue(t + (long long)d * gridDim.x, d);
  if (tid == 0) s_nbright[0] = s_nbright[1] = 0;
  const int ncen = a.ncen, sx0 = (m - ncen) / 2;
  const float inv_mm = 1.0f / (float)mm, inv_nc = 1.0f / (float)ncen;
  for (; t < ntiles; t += gridDim.x, k++) {
    asm volatile("cp.async.wait_group %0;" ::"n"(kSlotStages - 2) : "memory");
    // tile t is in shared memory and every thread is done with tile t - 1,
    // whose stage is refilled next
    __syncthreads();
    issue(t + (long long)(kSlotStages - 1) * gridDim.x, k + kSlotStages - 1);
    if (tid == 0) s_nbright[(k + 1) & 1] = 0;  // the next tile's queue
    int* nbright = &s_nbright[k & 1];
    float* imgs = ring + (k % kSlotStages) * stageFloats;
    const float* s_tot = imgs + TS * mm;
    const float* s_frac = s_tot + TS;
    const int* s_flag = reinterpret_cast<const int*>(s_frac + TS);
    const int f = (int)(t / tpf), s0 = (int)(t - (long long)f * tpf) * TS;
    const int ns = min(TS, a.nsubaps - s0);
    float* dstF = a.bimg + (long long)f * a.bimgFrameStride + (long long)s0 * mm;
    // noise and threshold of pixel pix of slot s (pf: Poisson applies)
    // (bright: lambda >= 64, the rejection sampler; otherwise the tables,
    // whose path the first loop compiles without the rejection loop)
    auto draw = [&](float v, int s, int pix, bool pf, auto bright) {
      KeyedStream st(a.philoxKeys, fbase + f, s0 + s, pix, 0);
      float g = 0.f;
      if constexpr (RN) g = normal_counter(st);
      if constexpr (POIS) {
        if (pf) {
          if constexpr (decltype(bright)::value) {
            v = poisson_counter_tab(st, v, *s_tab);
          } else if (v > 0.f) {  // as poisson_counter_tab for 0 < lambda < 64
            const float u3 = st.uniform();
            const float u4 = st.uniform();
            v = poisson_tab(*s_tab, u3, u4, v);
          } else {
            v = 0.f;
          }
        }
      }
      if constexpr (RN)
        v += rn * g + a.readBg;
      else
        v += a.readBg;
      return threshold_px(v, a.floorv, a.threshType);
    };
    float* outF = a.bimgOut ? a.bimgOut + (long long)f * a.bimgFrameStride + (long long)s0 * mm : nullptr;
    auto store = [&](int w, float v) {
      if (a.pxlPower == 2.f)
        v = v * v;
      else if (a.pxlPower != 1.f && a.pxlPower != 0.f)
        v = powf(v, a.pxlPower);
      dstF[w] = v;
      if (outF) outF[w] = v;
      imgs[w] = v;
    };
    for (int w = tid; w < ns * mm; w += blockDim.x) {
      const int s = div_small(w, mm, inv_mm);
      if (s_flag[s] != 1) continue;
      float v = imgs[w];
      if (noise) {
        const bool pf = POIS && (s_tot[s] > 0.f || a.sky * s_frac[s] > 0.f || a.skyArr);
        if (POIS && pf && v >= kModalMaxLam) {
          // lambda >= 64 (the rejection sampler): queued and drawn after
          // the others by the whole CTA, so that one such pixel does not
          // hold the other lanes of its warp (same streams, same draws)
          const int slot = atomicAdd(nbright, 1);
          if (slot < kPostBright) {
            s_bright[slot] = w;
            s_brightv[slot] = v;
            continue;
          }
          // queue full: drawn here
          store(w, draw(v, s, w - s * mm, pf, std::true_type{}));
          continue;
        }
        v = draw(v, s, w - s * mm, pf, std::false_type{});
      }
      store(w, v);
    }
    if (a.zeroUnlit) {
      // unlit subapertures: centroids 0 (cmod/src/centmodule.c:1964-1981)
      float* c = a.cents + (long long)f * a.centsFrameStride + 2LL * s0;
      for (int s = tid; s < ns; s += blockDim.x)
        if (s_flag[s] != 1) {
          c[2 * s] = 0.f;
          c[2 * s + 1] = 0.f;
        }
    }
    if constexpr (POIS) {
      if (noise) {
        __syncthreads();
        const int nb = min(*nbright, kPostBright);
        for (int b = tid; b < nb; b += blockDim.x) {
          const int w = s_bright[b];
          const int s = div_small(w, mm, inv_mm);
          store(w, draw(s_brightv[b], s, w - s * mm, true, std::true_type{}));
        }
      }
    }
    if (!cents) continue;
    __syncthreads();
    // centred-window CoG: sums of each window row (one thread per
    // subaperture row), then of the rows (one thread per subaperture)
    for (int pr = tid; pr < ns * ncen; pr += blockDim.x) {
      const int s = div_small(pr, ncen, inv_nc), rr = pr - s * ncen;
      float ps = 0.f, px = 0.f;
      if (s_flag[s] == 1) {
        const int r = sx0 + rr;
        const float* row = imgs + s * mm + r * m + sx0;
        const float* wrow = cw2d ? s_cw + r * m + sx0
                                 : (a.centWeightDim == 4 ? a.centWeight + (long long)(s0 + s) * mm + r * m + sx0 : nullptr);
        for (int c = 0; c < ncen; c++) {
          float v = row[c];
          if (wrow) v *= wrow[c];
          ps += v;
          px += v * (float)(sx0 + c);
        }
      }
      s_part[2 * pr] = ps;
      s_part[2 * pr + 1] = px;
    }
    __syncthreads();
    for (int s = tid; s < ns; s += blockDim.x) {
      if (s_flag[s] != 1) continue;
      float sum = 0.f, sxv = 0.f, syv = 0.f;
      for (int rr = 0; rr < ncen; rr++) {
        const float ps = s_part[2 * (s * ncen + rr)];
        sum += ps;
        sxv += s_part[2 * (s * ncen + rr) + 1];
        syv += ps * (float)(sx0 + rr);
      }
      float cx = 0.f, cy = 0.f;
      if (sum > 0.f) {
        cx = sxv / sum - 0.5f * (float)(m - 1);
        cy = syv / sum - 0.5f * (float)(m - 1);
      }
      calibrate_and_store(a, s0 + s, f, cx, cy);
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
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
  const int perSlot = (kSlotStages * (mm + 3) + 2 * a.ncen) * (int)sizeof(float);
  if (simple && a.subflag && tabB + cwB + 2 * perSlot <= 160 * 1024) {
    // slot tiles: kSlotStages stages of TS slots, sized for kSlotCtasPerSM CTAs per SM
    const int budget = (228 * 1024) / kSlotCtasPerSM - 1024 - 4 * kPostBright * 2 - 64 - tabB - cwB;
    int ts = budget / perSlot - 1;
    ts = ts < 1 ? 1 : (ts > kSlotMaxTS ? kSlotMaxTS : ts);
    // small batches: tiles no larger than it takes to give every resident
    // CTA one (latency), nor smaller than one pixel per thread
    const long long slots = (long long)a.nsubaps * a.nframes;
    const long long fill = (slots + (long long)numSMs * kSlotCtasPerSM - 1) / ((long long)numSMs * kSlotCtasPerSM);
    const int minTs = (kSlotThreads + mm - 1) / mm;
    if (fill < ts) ts = (int)std::max<long long>(fill, std::min(minTs, ts));
    a.TS = ts;
    if (done) {
      if (!a.imageOnly) {
        a.zeroUnlit = 1;
        *done |= kPostDidUnlit;
      }
      if (a.bimgOut) *done |= kPostDidOut;
    } else {
      a.bimgOut = nullptr;
    }
    const int stageFloats = (ts * mm + 3 * ts + 3) / 4 * 4;
    const int smem = tabB + cwB + (kSlotStages * stageFloats + 2 * ts * a.ncen) * (int)sizeof(float);
    const bool rnOn = a.calsource == 0 && a.readNoise != 0.f;
    auto kern = pois ? (rnOn ? wfs_post_slots_kernel<true, true> : wfs_post_slots_kernel<false, true>)
                     : (rnOn ? wfs_post_slots_kernel<true, false> : wfs_post_slots_kernel<false, false>);
    if (a.calsource != 0) a.readNoise = 0.f;
    int ctas = 0;
    cudaError_t e = kernel_smem_setup((const void*)kern, smem, kSlotThreads, &ctas);
    if (e != cudaSuccess) return e;
    if (ctas < 1) return cudaErrorInvalidConfiguration;
    const long long ntiles = (long long)((a.nsubaps + ts - 1) / ts) * a.nframes;
    const long long cap = (long long)numSMs * ctas;
    const int grid = (int)(ntiles < cap ? ntiles : cap);
    // programmatic launch: CTAs may become resident while the previous
    // kernel of the stream (the image formation) still runs and wait for it
    // in griddepcontrol.wait after loading their tables
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kSlotThreads);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const PoisTab* tabArg = pois ? tab : nullptr;
    return cudaLaunchKernelEx(&cfg, kern, a, tabArg);
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
