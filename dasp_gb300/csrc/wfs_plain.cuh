// Fused FP32 Shack-Hartmann WFS kernel ("plain" form).
//
// One CTA works on tiles of TS lit subapertures (several frames may share a
// tile).  Everything between the phase read and the bimg/cents write stays in
// shared memory or registers:
//
//   1 field + row FFTs    pup*exp(i(phs-tilt)) for the p non-zero rows, one
//                          N-point register FFT per row      (centmodule.c:473-498)
//   2 column FFTs + |F|^2 only the c columns/rows that survive the central
//                          crop, written 180-degree rotated   (:430-471)
//   2b prebin              optional block sum                 (:1583-1626)
//   3 spot-PSF convolution r2c rows, column FFT * PSF spectrum * inverse
//                          column FFT fused in registers, c2r rows of the
//                          clip window only                   (:524-564)
//   4 bin + normalise + sky  gather form of binImage in the reference's
//                          summation order                    (:609-651,1829-1872)
//   5 optical binning      optional, sequential per subap     (:819-851)
//   6 Poisson + read noise + threshold (counter-based stream) (:1879-1881)
//   7 brightest-pixel selection                               (:1544-1581)
//   8 pixel power, bimg write                                  (:1893-1897)
//   9 CoG / fit / optical-binning centroids, calibration, refs (:1925-1961)
#pragma once
#include "shwfs_dev.cuh"

namespace shwfs {

constexpr int kThreads = 128;

__host__ __device__ inline int odd_stride(int n) { return n | 1; }

// per-subaperture shared-memory footprint (floats)
__host__ __device__ inline int bufA_floats(int p, int N, int P) {
  int a = p * odd_stride(N) * 2;
  if (P > 0) {
    int b = P * odd_stride(P / 2 + 1) * 2;
    if (b > a) a = b;
    if (P * P > a) a = P * P;
  }
  return a;
}
__host__ __device__ inline int bufB_floats(int padded, int C) {
  int a = padded * padded;
  return C * C > a ? C * C : a;
}
__host__ __device__ inline int persub_floats(int p, int N, int P, int padded, int C, int m) {
  // A, B, binned image, per-row amplitude partial sums (2p), 8 scalars;
  // rounded to 4 floats so every subaperture's A buffer is 16-byte aligned
  int n = bufA_floats(p, N, P) + bufB_floats(padded, C) + m * m + 2 * p + 8;
  return (n + 3) & ~3;
}
// per-CTA constants: [PSF spectrum (2-D PSF)] tilt, bin tables, [2-D weights]
__host__ __device__ inline int const_floats(int p, int C, int m, int P, int cw2d, int psf2d) {
  int n = p * p + 3 * C + 2 * m + (cw2d ? m * m : 0);
  if (psf2d) n += 2 * P * (P / 2 + 1);
  return (n + 3) & ~3;
}

// interp: cmod/src/centmodule.c:1506-1518
__device__ inline float cal_interp(float x, int n, const float* xp, const float* fp) {
  if (x <= xp[0]) return fp[0];
  if (x >= xp[n]) return fp[n];
  int i = 1;
  while (i < n && x > xp[i]) i++;
  return (x - xp[i - 1]) * (fp[i] - fp[i - 1]) / (xp[i] - xp[i - 1]) + fp[i - 1];
}

__device__ inline void calibrate_and_store(const WfsArgs& a, int i, int f, float cx, float cy) {
  if (a.calData) {
    int lo = a.calBounds[i * 2];
    int n = a.calBounds[i * 2 + 1] - lo;
    cx = cal_interp(cx, n, a.calData + (long long)i * a.calNSteps + lo, a.calSteps + lo);
    lo = a.calBounds[(a.nsubaps + i) * 2];
    n = a.calBounds[(a.nsubaps + i) * 2 + 1] - lo;
    cy = cal_interp(cy, n, a.calData + (long long)(a.nsubaps + i) * a.calNSteps + lo, a.calSteps + lo);
  } else if (a.calCoeff) {
    float rx = 0.f, ry = 0.f, xc = 1.f, yc = 1.f;
    const float* kx = a.calCoeff + (long long)i * 2 * a.calNCoeff;
    const float* ky = kx + a.calNCoeff;
    for (int k = 0; k < a.calNCoeff; k++) {
      rx += xc * kx[k];
      xc *= cx;
      ry += yc * ky[k];
      yc *= cy;
    }
    cx = rx;
    cy = ry;
  }
  if (a.refCents) {
    cx -= a.refCents[2 * i];
    cy -= a.refCents[2 * i + 1];
  }
  float* c = a.cents + (long long)f * a.centsFrameStride;
  c[2 * i] = cx;
  c[2 * i + 1] = cy;
}

// computeFit (cmod/src/centmodule.c:1069-1188), one thread, image in smem
__device__ inline void fit_centroid(const WfsArgs& a, float* img, float& ocx, float& ocy) {
  const int n = a.m, ncen = a.ncen;
  int fitsize = a.fitSize;
  const int nc = (n - ncen) / 2;
  int quad = 0;
  if (fitsize < 0) {
    quad = 1;
    fitsize = 3;
  }
  if (fitsize < 3) fitsize = 3;
  float sum = 0.f, mx = 0.f;
  int mxpos = 0;
  if (a.gaussianFit) {
    for (int i = 0; i < n * n; i++) {
      sum += img[i];
      if (img[i] > mx) {
        mxpos = i;
        mx = img[i];
      }
      img[i] = img[i] < a.gMin ? a.gRep : logf(img[i]);
    }
  } else if (a.cob == 0 || a.cob == 1 || a.cob == 5) {
    for (int i = 0; i < n * n; i++) {
      sum += img[i];
      if (img[i] > mx) {
        mxpos = i;
        mx = img[i];
      }
    }
  } else {
    mx = img[nc * n + nc];
    mxpos = nc * n + nc;
    for (int i = nc; i < nc + ncen; i++)
      for (int j = nc; j < nc + ncen; j++) {
        sum += img[i * n + j];
        if (img[i * n + j] < mx) {
          mxpos = i * n + j;
          mx = img[i * n + j];
        }
      }
  }
  float cx = 0.f, cy = 0.f;
  if (sum >= 0.f) {
    int startx = mxpos % n - fitsize / 2;
    int starty = mxpos / n - fitsize / 2;
    if (startx < nc) startx = nc;
    if (starty < nc) starty = nc;
    if (startx > nc + ncen - fitsize) startx = nc + ncen - fitsize;
    if (starty > nc + ncen - fitsize) starty = nc + ncen - fitsize;
    if (quad == 0) {
      float vec[6] = {0, 0, 0, 0, 0, 0};
      for (int y = 0; y < fitsize; y++)
        for (int x = 0; x < fitsize; x++) {
          float v = img[(y + starty) * n + x + startx];
          vec[0] += v * x * x;
          vec[1] += v * x * y;
          vec[2] += v * y * y;
          vec[3] += v * x;
          vec[4] += v * y;
          vec[5] += v;
        }
      float res[5];
      for (int r = 0; r < 5; r++) {
        float t = 0.f;
        for (int k = 0; k < 6; k++) t += a.fitMx[r * 6 + k] * vec[k];
        res[r] = t;
      }
      if (a.gaussianFit) {
        cx = -res[3] / (2 * res[0]);
        cy = -res[4] / (2 * res[2]);
      } else {
        cx = (float)((res[1] * res[4] / (2 * res[2]) - res[3]) / (2. * res[0] - res[1] * res[1] / (2. * res[2])));
        cy = (float)(-(res[4] + res[1] * cx) / (2. * res[2]));
      }
    } else {
      const float* b = img + starty * n + startx;
      float a2 = (b[2 * n + 1] - b[1]) / 2.f;
      float a3 = (b[2 * n + 1] - 2 * b[n + 1] + b[1]) / 2.f;
      float a4 = (b[n + 2] - b[n]) / 2.f;
      float a5 = (b[n + 2] - 2 * b[n + 1] + b[n]) / 2.f;
      float a6 = (b[2 * n + 2] - b[2] - b[2 * n] + b[0]) / 4.f;
      cy = (2 * a2 * a5 - a4 * a6) / (a6 * a6 - 4 * a3 * a5) + 1;
      cx = (2 * a3 * a4 - a2 * a6) / (a6 * a6 - 4 * a3 * a5) + 1;
    }
    if (cx < 0 || cy < 0 || cx >= fitsize || cy >= fitsize) {
      cx = (float)(mxpos % n - startx);
      cy = (float)(mxpos / n - starty);
    }
    cy -= (float)(ncen / 2. - 0.5);
    cx -= (float)(ncen / 2. - 0.5);
    cx += (float)(startx + ncen / 2. - n / 2.);
    cy += (float)(starty + ncen / 2. - n / 2.);
  }
  ocx = cx;
  ocy = cy;
}

// Stage 9 on a tile of ns subapertures whose images (a.m x a.m) are in shared
// memory (img_of(s)): centroids (optical binning, fit or CoG), calibration,
// reference subtraction (cmod/src/centmodule.c:1925-1961, 2069-2107).  Used on
// the correlation images too, with a.m the correlation size.
template <class ImgOf>
__device__ __forceinline__ void centroid_tile(const WfsArgs& a, int ns, const int* s_subap, const int* s_frame,
                                              const float* s_cw, ImgOf img_of) {
    const int tid = threadIdx.x;
    const int m = a.m, mm = m * m;
    // ---- 9: centroids, calibration, reference subtraction ----
    const bool seqMode = a.opticalBinning == 1 || a.fitSize != 0 || a.gaussianFit > 0 || a.cob != 0;
    if (seqMode) {
      for (int s = tid; s < ns; s += blockDim.x) {
        float* img = img_of(s);
        const int i = s_subap[s];
        float cx = 0.f, cy = 0.f;
        if (a.opticalBinning == 1) {
          const int ncen = a.ncen;
          float sx = 0.f, sy = 0.f;
          for (int k = 0; k < ncen; k++) {
            sx += img[k];
            cx += img[k] * k;
            sy += img[k + ncen];
            cy += img[k + ncen] * k;
          }
          if (sx > 0) cx = (float)(cx / sx - (ncen - 1) / 2.);
          if (sy > 0) cy = (float)(cy / sy - (ncen - 1) / 2.);
        } else if (a.fitSize != 0 || a.gaussianFit > 0) {
          fit_centroid(a, img, cx, cy);
        } else {
          const int n = m, ncen = a.ncen;
          float mx = 0.f;
          int mpos = 0;
          if (a.cob == 1) {
            for (int k = 0; k < n * n; k++)
              if (img[k] > mx) {
                mx = img[k];
                mpos = k;
              }
          } else {
            for (int k = 0; k < n * n; k++)
              if (img[k] < mx || mx == 0) {
                mx = img[k];
                mpos = k;
              }
          }
          int sx = (int)(mpos % n - ncen / 2. + 0.5), sy = (int)(mpos / n - ncen / 2. + 0.5);
          sx = max(0, min(sx, n - ncen));
          sy = max(0, min(sy, n - ncen));
          const float* wt = a.centWeightDim == 2 ? s_cw
                            : (a.centWeightDim == 4 ? a.centWeight + (long long)i * mm : nullptr);
          const float sgn = (wt == nullptr && a.cob != 1) ? -1.f : 1.f;
          float sum = 0.f;
          for (int r = sy; r < sy + ncen; r++)
            for (int c = sx; c < sx + ncen; c++) {
              float t = wt ? img[r * n + c] * wt[r * n + c] : img[r * n + c];
              sum += t;
              cx += sgn * t * c;
              cy += sgn * t * r;
            }
          if (sum > 0) {
            cx = cx / sum + sx;
            cy = cy / sum + sy;
            cx = (float)(cx - (n - 1) / 2.);
            cy = (float)(cy - (n - 1) / 2.);
          } else {
            cx = cy = 0.f;
          }
        }
        calibrate_and_store(a, i, s_frame[s], cx, cy);
      }
    } else {
      // centred-window CoG: one warp per subap, lanes over window pixels
      const int warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
      const int ncen = a.ncen;
      const int sx = (m - ncen) / 2;
      const int nwin = ncen * ncen;
      for (int s = warp; s < ns; s += nwarps) {
        const float* img = img_of(s);
        const int i = s_subap[s];
        const float* wt = a.centWeightDim == 2 ? s_cw
                          : (a.centWeightDim == 4 ? a.centWeight + (long long)i * mm : nullptr);
        float sum = 0.f, sxv = 0.f, syv = 0.f;
        for (int k = lane; k < nwin; k += 32) {
          const int r = sx + k / ncen, c = sx + k % ncen;
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

// Stages 7-9 on a tile of ns subapertures whose images are in shared memory
// (img_of(s)): brightest-pixel selection, pixel power, bimg write, centroids
// with calibration and reference subtraction.  nexp_of(s) is the number of
// exposed pixels of subaperture s (cmod/src/centmodule.c:1883-1961,
// 2033-2107).
template <class ImgOf, class NexpOf>
__device__ __forceinline__ void post_tile(const WfsArgs& a, int ns, const int* s_subap, const int* s_frame,
                                          const float* s_cw, ImgOf img_of, NexpOf nexp_of) {
    const int tid = threadIdx.x;
    const int m = a.m, mm = m * m;
    // ---- 7: brightest-pixel selection (one warp per subap) ----
    if (a.calsource == 0 && (a.useBrightest != 0 || a.useBrightestArr)) {
      const int warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
      for (int s = warp; s < ns; s += nwarps) {
        int ub = a.useBrightestArr ? a.useBrightestArr[s_subap[s]] : a.useBrightest;
        bool subtract = false;
        if (ub < 0) {
          ub = -ub;
          subtract = true;
        }
        if (!(ub > 0 && ub < nexp_of(s))) continue;
        float* img = img_of(s);
        const int pos = nexp_of(s) - ub;  // ascending sorted index of the threshold
        float thr = 0.f;
        bool found = false;
        for (int j = lane; j < nexp_of(s); j += 32) {
          const float xj = img[j];
          int lt = 0, le = 0;
          for (int k = 0; k < nexp_of(s); k++) {
            lt += img[k] < xj;
            le += img[k] <= xj;
          }
          if (lt <= pos && pos < le) {
            thr = xj;
            found = true;
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, found);
        if (bal == 0u) continue;  // only with NaN pixels: leave the image as is
        thr = __shfl_sync(0xffffffffu, thr, __ffs(bal) - 1);
        float sub = 0.f;
        if (subtract) {
          float best = -INFINITY;
          for (int j = lane; j < nexp_of(s); j += 32)
            if (img[j] < thr) best = fmaxf(best, img[j]);
          for (int o = 16; o; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
          sub = best == -INFINITY ? 0.f : best;
        }
        __syncwarp();
        for (int j = lane; j < nexp_of(s); j += 32) {
          const float v = img[j];
          img[j] = v < thr ? 0.f : (subtract ? v - sub : v);
        }
      }
      __syncthreads();
    }

    // ---- 8: pixel power, bimg write ----
    const float inv_mm = 1.0f / (float)mm;
    for (int w = tid; w < ns * mm; w += blockDim.x) {
      const int s = div_small(w, mm, inv_mm), pix = w - s * mm;
      float v = img_of(s)[pix];
      if (pix < nexp_of(s)) {
        if (a.pxlPower == 2.f)
          v = v * v;
        else if (a.pxlPower != 1.f && a.pxlPower != 0.f)
          v = powf(v, a.pxlPower);
        img_of(s)[pix] = v;
      }
      a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)s_subap[s] * mm + pix] = v;
    }
    if (a.imageOnly != 0 || a.skipCents) return;
    __syncthreads();
    centroid_tile(a, ns, s_subap, s_frame, s_cw, img_of);
    if (a.gaussianFit > 0 && a.opticalBinning != 1) {
      // computeFit takes the log of the image in place before fitting
      // (cmod/src/centmodule.c:1087-1096), and that image is the caller's
      // bimg: the reference's output holds the log image after a Gaussian fit
      __syncthreads();
      for (int w = tid; w < ns * mm; w += blockDim.x) {
        const int s = div_small(w, mm, inv_mm), pix = w - s * mm;
        a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)s_subap[s] * mm + pix] = img_of(s)[pix];
      }
    }
}

// The fused kernel's work for one handle, run by CTA `cta` of the `nctas`
// CTAs that share its tiles (the whole grid for a single handle, a slice of
// it in a multi-handle launch).
template <int N, int P>
__device__ __forceinline__ void plain_body(const WfsArgs& a, long long cta, long long nctas) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int tid = threadIdx.x;
  const int p = a.p, C = a.C, m = a.m, padded = a.padded;
  const int mm = m * m;
  const int NS = odd_stride(N);
  constexpr int HS = P > 0 ? P / 2 + 1 : 1;
  const int HSS = odd_stride(HS);
  const bool cw2d = a.centWeightDim == 2;
  const bool psf2d = P > 0 && a.psfDim == 2;

  // --- per-CTA constants ---
  float2* s_psf = reinterpret_cast<float2*>(smem);
  float* s_tilt = smem + (psf2d ? 2 * P * HS : 0);
  float* s_binT = s_tilt + p * p;
  float* s_binN = s_binT + C;
  int* s_binII = reinterpret_cast<int*>(s_binN + C);
  int* s_binLo = s_binII + C;
  int* s_binHi = s_binLo + m;
  float* s_cw = reinterpret_cast<float*>(s_binHi + m);
  float* s_sub0 = smem + const_floats(p, C, m, P, cw2d, psf2d);
  const int fA = bufA_floats(p, N, P), fB = bufB_floats(padded, C);
  const int persub = persub_floats(p, N, P, padded, C, m);

  for (int k = tid; k < p * p; k += blockDim.x) s_tilt[k] = a.tilt[k];
  for (int k = tid; k < C; k += blockDim.x) {
    s_binT[k] = a.binT[k];
    s_binN[k] = a.binN[k];
    s_binII[k] = a.binII[k];
  }
  for (int k = tid; k < m; k += blockDim.x) {
    s_binLo[k] = a.binLo[k];
    s_binHi[k] = a.binHi[k];
  }
  if (cw2d)
    for (int k = tid; k < mm; k += blockDim.x) s_cw[k] = a.centWeight[k];
  if (psf2d)
    for (int k = tid; k < P * HS; k += blockDim.x) s_psf[k] = a.psfSpec[k];

  __shared__ int s_subap[64];
  __shared__ int s_frame[64];

  const int TS = a.TS;
  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + TS - 1) / TS;
  const bool doForm = a.mode & kForm;
  const bool doNoise = a.mode & kNoiseCounter;
  const bool doPost = a.mode & kPost;
  const bool storePre = a.mode & kStorePreNoise;

  // power-spectrum crop/pad geometry (addPowerSpecCentral)
  const int rs = padded > N ? (padded - N) / 2 : 0;
  const int ro = padded > N ? 0 : (N - padded) / 2;
  const int cc = padded > N ? N : padded;
  const int nexp = a.opticalBinning == 1 ? 2 * a.ncen : mm;

  for (long long tile = cta; tile < ntiles; tile += nctas) {
    const long long w0 = tile * TS;
    const int ns = (int)min((long long)TS, nwork - w0);
    __syncthreads();  // previous tile fully consumed
    for (int s = tid; s < ns; s += blockDim.x) {
      long long w = w0 + s;
      s_frame[s] = (int)(w / a.nlit);
      s_subap[s] = a.lit[w % a.nlit];
    }
    __syncthreads();
#define SUB(s) (s_sub0 + (size_t)(s) * persub)
#define BUF_A(s) (SUB(s))
#define BUF_B(s) (SUB(s) + fA)
#define IMG(s) (SUB(s) + fA + fB)
#define AMPSUM(s) (SUB(s) + fA + fB + mm)
#define SCAL(s) (SUB(s) + fA + fB + mm + 2 * p)

    if (doForm) {
      // ---- 1: field + row FFTs ----
      for (int w = tid; w < ns * p; w += blockDim.x) {
        const int s = w / p, r = w - (w / p) * p;
        const int i = s_subap[s], f = s_frame[s];
        const int sy = i / a.nsubx, sx = i - sy * a.nsubx;
        const float* ph = a.phs + (long long)f * a.phsFrameStride + (long long)(sy * p + r) * a.W + sx * p;
        const float* pu = a.pup + ((long long)i * p + r) * p;
        float2 x[N];
        float ampsum = 0.f, pupsum = 0.f;
#pragma unroll
        for (int j = 0; j < N; j++) {
          if (j < p) {
            float t = ph[j] - s_tilt[r * p + j];
            float sn, cs;
            sincosf(t, &sn, &cs);
            float amp = pu[j];
            if (a.phaseAmp) {
              float am = ph[j + a.phsAmpOffset];
              pupsum += amp;
              amp = amp * am;
              ampsum += amp;
            }
            x[j] = make_float2(amp * cs, amp * sn);
          } else {
            x[j] = make_float2(0.f, 0.f);
          }
        }
        if (a.phaseAmp) {
          AMPSUM(s)[r] = ampsum;
          AMPSUM(s)[p + r] = pupsum;
        }
        fft<N, -1>(x);
        float2* rb = reinterpret_cast<float2*>(BUF_A(s)) + r * NS;
#pragma unroll
        for (int k = 0; k < N; k++) rb[k] = x[k];
      }
      if (padded > N) {
        for (int w = tid; w < ns * padded * padded; w += blockDim.x) {
          int s = w / (padded * padded);
          BUF_B(s)[w - s * padded * padded] = 0.f;
        }
      }
      __syncthreads();

      // ---- 2: column FFTs, |F|^2, rotated crop into hll (BUF_B) ----
      for (int w = tid; w < ns * cc; w += blockDim.x) {
        const int s = w / cc, kk = w - (w / cc) * cc;
        const int col = ro + kk;
        const float2* rb = reinterpret_cast<const float2*>(BUF_A(s));
        float2 x[N];
#pragma unroll
        for (int r = 0; r < N; r++) x[r] = r < p ? rb[r * NS + col] : make_float2(0.f, 0.f);
        fft<N, -1>(x);
        float* hll = BUF_B(s);
#pragma unroll
        for (int ii = 0; ii < N; ii++) {
          if (ii >= ro && ii < ro + cc) {
            const int i_ = ii - ro;
            hll[(cc - 1 - i_ + rs) * padded + (cc - 1 - kk + rs)] = x[ii].x * x[ii].x + x[ii].y * x[ii].y;
          }
        }
      }
      __syncthreads();

      if constexpr (P > 0) {
        // ---- 2b: prebin (hll padded x padded -> P x P) ----
        if (a.preBin > 1) {
          const int f = a.preBin, scaled = padded / f;
          const int b = scaled > P ? P : scaled;
          const int off = scaled > P ? (scaled - P) / 2 : 0;
          const int o2 = scaled < P ? (P - scaled) / 2 : 0;
          for (int w = tid; w < ns * P * P; w += blockDim.x) {
            const int s = w / (P * P), q = w - s * P * P;
            const int oi = q / P, oj = q - (q / P) * P;
            const int bi = oi - o2, bj = oj - o2;
            float v = 0.f;
            if (bi >= 0 && bi < b && bj >= 0 && bj < b) {
              const float* hll = BUF_B(s);
              for (int ii = 0; ii < f; ii++)
                for (int jj = 0; jj < f; jj++) v += hll[(bi * f + ii + off) * padded + bj * f + jj + off];
            }
            BUF_A(s)[q] = v;
          }
          __syncthreads();
          for (int w = tid; w < ns * P * P; w += blockDim.x) {
            const int s = w / (P * P), q = w - s * P * P;
            BUF_B(s)[q] = BUF_A(s)[q];
          }
          __syncthreads();
        }
        // ---- 3a: r2c rows of hll (P x P, stride P) -> spectrum rows in BUF_A;
        // two real rows per complex FFT: z = x + i y, X = (Z + conj Z(-k))/2,
        // Y = (Z - conj Z(-k))/(2i) ----
        constexpr int PH = (P + 1) / 2;
        for (int w = tid; w < ns * PH; w += blockDim.x) {
          const int s = w / PH, q = w - (w / PH) * PH;
          const int r0 = 2 * q, r1 = 2 * q + 1;
          const bool two = r1 < P;
          const float* h0 = BUF_B(s) + r0 * P;
          const float* h1 = h0 + P;
          float2 z[P];
#pragma unroll
          for (int n = 0; n < P; n++) z[n] = make_float2(h0[n], two ? h1[n] : 0.f);
          fft<P, -1>(z);
          float2* s0 = reinterpret_cast<float2*>(BUF_A(s)) + r0 * HSS;
          float2* s1 = s0 + HSS;
#pragma unroll
          for (int k = 0; k < HS; k++) {
            const float2 a = z[k], b = z[(P - k) % P];
            s0[k] = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
            if (two) s1[k] = make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x));
          }
        }
        __syncthreads();
        // ---- 3b: column FFT, * PSF spectrum, inverse column FFT ----
        for (int w = tid; w < ns * HS; w += blockDim.x) {
          const int s = w / HS, col = w - (w / HS) * HS;
          float2* sp = reinterpret_cast<float2*>(BUF_A(s));
          const float2* psf = psf2d ? s_psf : a.psfSpec + (long long)s_subap[s] * P * HS;
          float2 y[P];
#pragma unroll
          for (int r = 0; r < P; r++) y[r] = sp[r * HSS + col];
          fft<P, -1>(y);
#pragma unroll
          for (int r = 0; r < P; r++) y[r] = cmul(y[r], psf[r * HS + col]);
          fft<P, 1>(y);
#pragma unroll
          for (int r = 0; r < P; r++) sp[r * HSS + col] = y[r];
        }
        __syncthreads();
        // ---- 3c: c2r rows of the clip window -> C x C in BUF_B ----
        // two half-spectrum rows per complex inverse FFT (z = X + iY gives
        // x + iy); the imaginary parts of the DC and Nyquist bins are
        // ignored, as a c2r transform does
        const int off = (P - C) / 2;
        const int CH = (C + 1) / 2;
        for (int w = tid; w < ns * CH; w += blockDim.x) {
          const int s = w / CH, q = w - (w / CH) * CH;
          const int o0 = 2 * q, o1 = 2 * q + 1;
          const bool two = o1 < C;
          const float2* s0 = reinterpret_cast<const float2*>(BUF_A(s)) + (o0 + off) * HSS;
          const float2* s1 = s0 + HSS;
          float2 z[P];
#pragma unroll
          for (int k = 0; k < P; k++) {
            float2 X = k < HS ? s0[k] : cconj(s0[P - k]);
            float2 Y = two ? (k < HS ? s1[k] : cconj(s1[P - k])) : make_float2(0.f, 0.f);
            if (k == 0 || 2 * k == P) {
              X.y = 0.f;
              Y.y = 0.f;
            }
            z[k] = make_float2(X.x - Y.y, X.y + Y.x);
          }
          fft<P, 1>(z);
          float* out0 = BUF_B(s) + o0 * C;
          float* out1 = out0 + C;
#pragma unroll
          for (int n = 0; n < P; n++)
            if (n >= off && n < off + C) {
              out0[n - off] = z[n].x;
              if (two) out1[n - off] = z[n].y;
            }
        }
        __syncthreads();
      }

      // ---- 4: bin, normalise, sky -> IMG ----
      for (int w = tid; w < ns * mm; w += blockDim.x) {
        const int s = w / mm, pix = w - (w / mm) * mm;
        const int I = pix / m, J = pix - (pix / m) * m;
        const int i = s_subap[s];
        const float* src = BUF_B(s);  // C x C, stride C
        float v;
        if (C == m) {
          v = src[I * C + J];
        } else {
          v = 0.f;
          const int ilo = s_binLo[I], ihi = s_binHi[I], jlo = s_binLo[J], jhi = s_binHi[J];
          for (int ii = ilo; ii <= ihi; ii++) {
            const int iiv = s_binII[ii];
            const bool lastI = ii == C - 1;
            for (int jj = jlo; jj <= jhi; jj++) {
              const int jjv = s_binII[jj];
              const bool lastJ = jj == C - 1;
              if (iiv == I) {
                if (jjv == J)
                  v += s_binT[ii] * s_binT[jj] * src[ii * C + jj];
                else if (jjv + 1 == J && !lastJ)
                  v += s_binT[ii] * s_binN[jj] * src[ii * C + jj + 1];
              } else if (iiv + 1 == I && !lastI) {
                if (jjv == J)
                  v += s_binN[ii] * s_binT[jj] * src[(ii + 1) * C + jj];
                else if (jjv + 1 == J && !lastJ)
                  v += s_binN[ii] * s_binN[jj] * src[(ii + 1) * C + jj + 1];
              }
            }
          }
        }
        float totsig;
        if (a.phaseAmp) {
          float ts = 0.f, tp = 0.f;
          for (int r = 0; r < p; r++) {
            ts += AMPSUM(s)[r];
            tp += AMPSUM(s)[p + r];
          }
          totsig = tp != 0.f ? ts * (a.totsig[i] / tp) : 0.f;
        } else {
          totsig = a.totsig[i];
        }
        const float fr = a.frac[i];
        if (totsig > 0.f) v *= a.sigArr ? a.sigArr[i] / totsig : a.sig * fr / totsig;
        const float skyv = a.sky * fr;
        if (skyv > 0.f) v += skyv;
        if (a.skyArr) v += a.skyArr[(long long)i * mm + pix];
        IMG(s)[pix] = v;
        if (pix == 0) SCAL(s)[0] = (totsig > 0.f || skyv > 0.f || a.skyArr) ? 1.f : 0.f;
      }
      __syncthreads();

      // ---- 5: optical binning (sequential, one thread per subap) ----
      if (a.opticalBinning == 1) {
        for (int s = tid; s < ns; s += blockDim.x) {
          float* img = IMG(s);
          const int ncen = a.ncen;
          const int st = (m - ncen) / 2, e = m - st;
          float v0 = 0.f;
          for (int ii = st; ii < e; ii++) v0 += img[m * st + ii];
          if (st != 0)
            for (int k = 0; k < ncen; k++) img[k] = 0.f;
          for (int ii = st; ii < e; ii++)
            for (int j = (st == 0 ? 1 : st); j < e; j++) img[ii - st] += img[j * m + ii];
          for (int ii = st + 1; ii < e; ii++) {
            if (st != 0) img[ii - st + ncen] = 0.f;
            for (int j = (st == 0 ? 1 : st); j < e; j++) img[ii - st + ncen] += img[ii * m + j];
          }
          img[ncen] = v0;
          for (int k = 2 * ncen; k < mm; k++) img[k] = 0.f;
        }
        __syncthreads();
      }

      if (storePre) {
        for (int w = tid; w < ns * mm; w += blockDim.x) {
          const int s = w / mm, pix = w - (w / mm) * mm;
          a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)s_subap[s] * mm + pix] = IMG(s)[pix];
          if (pix == 0 && a.poisFlag) a.poisFlag[s_subap[s]] = SCAL(s)[0] != 0.f;
        }
        continue;
      }
    } else {
      // post-only launch: the (noised) image comes from bimg
      for (int w = tid; w < ns * mm; w += blockDim.x) {
        const int s = w / mm, pix = w - (w / mm) * mm;
        IMG(s)[pix] = a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)s_subap[s] * mm + pix];
      }
      __syncthreads();
    }

    // ---- 6: Poisson + read noise + threshold (counter-based streams) ----
    // one thread per quad of pixels (quad_normals, quad_poisson; lambda >= 64
    // from the pixel's own stream, ptrs_pixel), pixels from nexp on untouched
    if (doNoise) {
      const bool pois = a.addPoisson == 1 && a.calsource == 0;
      const float rn = a.calsource == 0 ? a.readNoise : 0.f;
      const int nqi = (nexp + 3) >> 2;
      for (int wq = tid; wq < ns * nqi; wq += blockDim.x) {
        const int s = wq / nqi, qd = wq - s * nqi;
        const int p0 = 4 * qd, np = min(4, nexp - p0);
        const uint32_t i = (uint32_t)s_subap[s];
        const uint32_t fr = (uint32_t)(frame_base(a) + s_frame[s]);
        float* px = IMG(s) + p0;
        float v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = k < np ? px[k] : 0.f;
        if (pois && SCAL(s)[0] != 0.f) {
          unsigned bm = 0;
#pragma unroll
          for (int k = 0; k < 4; k++)
            if (v[k] >= kModalMaxLam) bm |= 1u << k;
          quad_poisson(a.philoxKeys, fr, i, (uint32_t)qd, *a.poisTab, v, bm);
#pragma unroll
          for (int k = 0; k < 4; k++)
            if ((bm >> k) & 1u) v[k] = ptrs_pixel_cold(a.seed, fr, i, (uint32_t)(p0 + k), v[k]);
        }
        float g[4] = {0.f, 0.f, 0.f, 0.f};
        if (rn != 0.f) quad_normals(a.philoxKeys, fr, i, (uint32_t)qd, g);
#pragma unroll
        for (int k = 0; k < 4; k++)
          if (k < np) px[k] = threshold_px(v[k] + (rn * g[k] + a.readBg), a.floorv, a.threshType);
      }
      __syncthreads();
    }

    if (!doPost) continue;

    post_tile(a, ns, s_subap, s_frame, s_cw, [&](int s) { return IMG(s); }, [&](int) { return nexp; });
#undef SUB
#undef BUF_A
#undef BUF_B
#undef IMG
#undef AMPSUM
#undef SCAL
  }
}

template <int N, int P>
__global__ void __launch_bounds__(kThreads) wfs_plain_kernel(const __grid_constant__ WfsArgs a) {
  plain_body<N, P>(a, blockIdx.x, gridDim.x);
}

// Several handles of one (fftsize, psfsize) instantiation in one launch (the
// multi-sensor batches): handle h owns CTAs [ctaStart[h], ctaStart[h+1]) and
// each of them loops over that handle's tiles, as in a launch of its own.
constexpr int kPlainMulti = 8;
struct PlainMulti {
  WfsArgs a[kPlainMulti];
  int ctaStart[kPlainMulti + 1];
  int n;
};

template <int N, int P>
__global__ void __launch_bounds__(kThreads) wfs_plain_multi_kernel(const __grid_constant__ PlainMulti m) {
  int h = 0;
  while (h + 1 < m.n && (int)blockIdx.x >= m.ctaStart[h + 1]) h++;
  plain_body<N, P>(m.a[h], (long long)blockIdx.x - m.ctaStart[h], (long long)(m.ctaStart[h + 1] - m.ctaStart[h]));
}

// launcher of the unlit-subaperture kernel (wfs_unlit.cu)
cudaError_t launch_unlit(const WfsArgs& a, const int* unlit, int nunlit, cudaStream_t stream);
cudaError_t launch_test_corr(int n, const float* img, const float* K, float* out, cudaStream_t stream);
// correlation centroiding (wfs_corr.cu)
struct CorrArgs {
  int mode;       // correlationCentroiding, 1..5
  int cs;         // corrsize
  float thresh;   // corrThresh
  const float* K; // per subaperture cs*cs: mode 1 the convolution kernel hc2r(pattern), else the pattern
  float* corrimg; // [frame][nsubaps][cs*cs] output
  long long corrimgFrameStride;
  int TS;         // subapertures per CTA tile (set by the launcher)
};
// bicubic resample of nframes square nin x nin phase frames to nout x nout
// (interpolatePhase, wfs_interp.cu)
cudaError_t launch_interp_phase(const float* in, long long inStride, int nin, float* out, long long outStride, int nout,
                                int nframes, cudaStream_t stream);
// the p x p blocks of the lit subapertures of a W x W array, src -> dst
cudaError_t launch_copy_lit_blocks(const float* src, float* dst, const int* lit, int nlit, int nsubx, int p,
                                   cudaStream_t stream);
// one CTA waiting on an mbarrier nothing arrives on, up to max_cycles;
// out[0..2] = gave up, abort flag raised, cycles waited / 2^20 (selftest.cu)
cudaError_t launch_bounded_wait_selftest(long long max_cycles, int* out, cudaStream_t stream);
cudaError_t launch_corr(const WfsArgs& a, CorrArgs c, int numSMs, cudaStream_t stream);

// increment n device counters (graph replays of a batch)
cudaError_t launch_bump_counters(unsigned long long* const* ctrs, int n, cudaStream_t stream);
// counter-based noise draws for testing the samplers (kind 0 Poisson, 1 normal)
cudaError_t launch_sample_noise(const float* lam, long long n, unsigned long long seed, unsigned long long frame,
                                int kind, float* out, cudaStream_t stream);
// store v in one device counter, in stream order
cudaError_t launch_set_counter(unsigned long long* ctr, unsigned long long v, cudaStream_t stream);
// image-input (runSlope) kernel over the lit subapertures (wfs_image.cu)
cudaError_t launch_image(const WfsArgs& a, const float* img, int dims, int npxlx, const int* loc, int numSMs,
                         cudaStream_t stream);
// copy the listed subapertures' images src -> dst (dst: mapped host memory)
cudaError_t launch_publish(const float* src, float* dst, const int* list, int n, int mm, cudaStream_t stream);
// physical integration: acc = (first ? sub : acc + sub), then acc *= scale
// (the exposure's mean at its readout frame), over n values
cudaError_t launch_accumulate(float* acc, const float* sub, long long n, int first, float scale, cudaStream_t stream);

}  // namespace shwfs
