// Correlation centroiding (cmod/src/centmodule.c:1898-1925 and 2044-2066):
// from each lit subaperture's final image in bimg, the correlation image with
// the subaperture's pattern (corrsize x corrsize), its threshold, the
// correlation image written to corrimg, then the centroid stage on it.
//
//   mode 1  calcCorrelation (:1403-1486): r2hc(zero-padded image) times the
//           half-complex pattern, hc2r -- computed as the circular
//           convolution of the padded image with hc2r(pattern), which the
//           host builds once per pattern (the half-complex product is the
//           product of the complex spectra)
//   mode 2  diffCorrelation mode 1: mean squared difference over the overlap
//   mode 3  diffCorrelation mode 2: the reference's abs-difference branch,
//           with its own indexing
//   mode 4  diffCorrelation mode 3: squared difference / (flux of image *
//           flux of pattern) over the overlap
//   mode 5  bruteCorrelation (:1339-1398): overlap sums of the product
// then thresholdCorrelation (:1488-1505) over corrsize^2 pixels and
// computeCoG/computeFit with corrsize (centre on brightest for modes 1 and 5,
// faintest otherwise).
#include "wfs_plain.cuh"

namespace shwfs {

namespace {

constexpr int kCorrThreads = 256;
constexpr int kCorrMaxTS = 32;

// overlap of pattern and image for output offset i (diffCorrelation
// :1228-1240): start in the pattern, start in the image, extent
__device__ __forceinline__ void overlap(int i, int nimg, int cs, int ncen, int& sref, int& sin_, int& len) {
  const int off = i - ncen / 2;
  len = cs < nimg ? cs : nimg;
  sref = -off - (nimg - cs) / 2;
  if (sref < 0) sref = 0;
  sin_ = (nimg - cs) / 2 + off;
  if (sin_ < 0) sin_ = 0;
  if (sin_ + len > nimg) len = nimg - sin_;
  if (sref + len > cs) len = cs - sref;
}

__global__ void __launch_bounds__(kCorrThreads) wfs_corr_kernel(const WfsArgs a, const CorrArgs c) {
  extern __shared__ __align__(16) float smem_corr[];
  __shared__ int s_subap[kCorrMaxTS];
  __shared__ int s_frame[kCorrMaxTS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int m = a.m, mm = m * m, cs = c.cs, cc = cs * cs, ncen = a.ncen;
  const bool cw2d = a.centWeightDim == 2;
  float* s_cw = smem_corr;
  float* imgs = s_cw + (cw2d ? cc : 0);
  float* corr = imgs + c.TS * mm;
  float* Ks = corr + c.TS * cc;  // the tile's patterns (or hc2r(pattern) for mode 1)
  if (cw2d)
    for (int k = tid; k < cc; k += blockDim.x) s_cw[k] = a.centWeight[k];
  WfsArgs ac = a;  // the centroid stage sees corrsize x corrsize images
  ac.m = cs;
  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + c.TS - 1) / c.TS;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long w0 = tile * c.TS;
    const int ns = (int)min((long long)c.TS, nwork - w0);
    __syncthreads();
    for (int s = tid; s < ns; s += blockDim.x) {
      const long long w = w0 + s;
      s_frame[s] = (int)(w / a.nlit);
      s_subap[s] = a.lit[w % a.nlit];
    }
    __syncthreads();
    for (int w = tid; w < ns * mm; w += blockDim.x) {
      const int s = w / mm, pix = w - s * mm;
      imgs[w] = a.bimg[(long long)s_frame[s] * a.bimgFrameStride + (long long)s_subap[s] * mm + pix];
    }
    for (int w = tid; w < ns * cc; w += blockDim.x) {
      const int s = w / cc, o = w - s * cc;
      Ks[w] = c.K[(long long)s_subap[s] * cc + o];
    }
    __syncthreads();
    // ---- correlation images ----
    for (int w = tid; w < ns * cc; w += blockDim.x) {
      const int s = w / cc, o = w - s * cc, y = o / cs, x = o - y * cs;
      const float* img = imgs + s * mm;
      const float* K = Ks + s * cc;
      float v = 0.f;
      if (c.mode == 1) {
        // circular indices (y - p - off) mod cs and (x - q - off) mod cs: both
        // differences lie in [-cs, cs), so one conditional wrap each
        const int off = (cs - m) / 2;
        int kx0 = x - off;
        if (kx0 < 0) kx0 += cs;
        for (int p = 0; p < m; p++) {
          int ky = y - p - off;
          if (ky < 0) ky += cs;
          const float* Krow = K + ky * cs;
          const float* irow = img + p * m;
          int kx = kx0;
          for (int q = 0; q < m; q++) {
            v += irow[q] * Krow[kx];
            kx = kx == 0 ? cs - 1 : kx - 1;
          }
        }
      } else if (c.mode == 3) {
        // the abs-difference branch writes output (i + (nimg-ncen)/2,
        // j + (nimg-ncen)/2) of a corrsize-wide array
        const int i = y - (m - ncen) / 2, j = x - (m - ncen) / 2;
        if (i >= 0 && i < ncen && j >= 0 && j < ncen) {
          const int my = cs - abs(ncen / 2 - i), mx = cs - abs(ncen / 2 - j);
          float sacc = 0.f;
          for (int yy = 0; yy < my; yy++)
            for (int xx = 0; xx < mx; xx++) {
              float d;
              if (i < ncen / 2) {
                if (j < ncen / 2)
                  d = K[yy * cs + xx] - img[(ncen / 2 - i + yy) * m + ncen / 2 - j + xx];
                else
                  d = K[yy * cs + j - ncen / 2 + xx] - img[(ncen / 2 - i + yy) * m + xx];
              } else {
                if (j < ncen / 2)
                  d = K[(i - ncen / 2 + yy) * cs + xx] - img[yy * m + ncen / 2 - j + xx];
                else
                  d = K[(i - ncen / 2 + yy) * cs + j - ncen / 2 + xx] - img[yy * m + xx];
              }
              sacc += fabsf(d);
            }
          v = sacc * sacc / (float)(my * mx);
        }
      } else {
        const int i = y - (cs - ncen) / 2, j = x - (cs - ncen) / 2;
        if (i >= 0 && i < ncen && j >= 0 && j < ncen) {
          int srefy, siny, my, srefx, sinx, mx;
          overlap(i, m, cs, ncen, srefy, siny, my);
          overlap(j, m, cs, ncen, srefx, sinx, mx);
          float sacc = 0.f, tot = 0.f, tot2 = 0.f;
          for (int yy = 0; yy < my; yy++)
            for (int xx = 0; xx < mx; xx++) {
              const float b = img[(siny + yy) * m + sinx + xx];
              const float p = K[(srefy + yy) * cs + srefx + xx];
              if (c.mode == 5) {
                sacc += p * b;
              } else {
                const float d = p - b;
                sacc += d * d;
                tot += b;
                tot2 += p;
              }
            }
          if (c.mode == 2) {
            if (mx != 0 && my != 0) v = sacc / (float)(mx * my);
          } else if (c.mode == 4) {
            if (tot != 0.f && tot2 != 0.f) v = sacc / (tot * tot2);
          } else if (mx != 0 && my != 0) {
            v = sacc;
          }
        }
      }
      corr[w] = v;
    }
    __syncthreads();
    // ---- threshold (a fraction of the maximum when 0 < thresh <= 1), and
    // the thresholded image to corrimg: one warp per subaperture ----
    for (int s = warp; s < ns; s += nwarps) {
      float* im = corr + s * cc;
      float t = c.thresh;
      if (t <= 1.f && t > 0.f) {
        float mx = 0.f;
        for (int k = lane; k < cc; k += 32) mx = fmaxf(mx, im[k]);
#pragma unroll
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        t = mx * t;
      }
      __syncwarp();
      float* out = c.corrimg + (long long)s_frame[s] * c.corrimgFrameStride + (long long)s_subap[s] * cc;
      for (int k = lane; k < cc; k += 32) {
        const float v = im[k] < t ? 0.f : im[k] - t;
        im[k] = v;
        out[k] = v;
      }
    }
    __syncthreads();
    centroid_tile(ac, ns, s_subap, s_frame, s_cw, [&](int s) { return corr + s * cc; });
    if (ac.gaussianFit > 0 && ac.opticalBinning != 1) {
      // the Gaussian fit logs its input in place (cmod/src/centmodule.c:
      // 1087-1096); with correlation that input is the corrimg output
      __syncthreads();
      for (int s = warp; s < ns; s += nwarps) {
        float* out = c.corrimg + (long long)s_frame[s] * c.corrimgFrameStride + (long long)s_subap[s] * cc;
        for (int k = lane; k < cc; k += 32) out[k] = corr[s * cc + k];
      }
    }
  }
}

// testcorrelation: the correlation of one n x n image with a pattern whose
// inverse transform is K (mode 1 with corrsize = nimg = n: a circular
// convolution, summed in the correlation kernel's order)
__global__ void test_corr_kernel(int n, const float* __restrict__ img, const float* __restrict__ K,
                                 float* __restrict__ out) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n * n) return;
  const int y = o / n, x = o - y * n;
  float v = 0.f;
  for (int p = 0; p < n; p++) {
    int ky = y - p;
    if (ky < 0) ky += n;
    int kx = x;
    for (int q = 0; q < n; q++) {
      v += img[p * n + q] * K[ky * n + kx];
      kx = kx == 0 ? n - 1 : kx - 1;
    }
  }
  out[o] = v;
}

}  // namespace

cudaError_t launch_test_corr(int n, const float* img, const float* K, float* out, cudaStream_t stream) {
  const int nn = n * n;
  test_corr_kernel<<<(nn + 255) / 256, 256, 0, stream>>>(n, img, K, out);
  return cudaGetLastError();
}

cudaError_t launch_corr(const WfsArgs& a, CorrArgs c, int numSMs, cudaStream_t stream) {
  const long long nwork = (long long)a.nlit * a.nframes;
  if (nwork == 0) return cudaSuccess;
  const int mm = a.m * a.m, cc = c.cs * c.cs;
  // per subaperture: image, correlation image, pattern
  int ts = 12288 / (mm + 2 * cc);
  c.TS = ts < 1 ? 1 : (ts > kCorrMaxTS ? kCorrMaxTS : ts);
  const int smem = (c.TS * (mm + 2 * cc) + (a.centWeightDim == 2 ? cc : 0)) * (int)sizeof(float);
  cudaError_t e = kernel_smem_setup((const void*)wfs_corr_kernel, smem, kCorrThreads, nullptr);
  if (e != cudaSuccess) return e;
  const long long ntiles = (nwork + c.TS - 1) / c.TS;
  const long long cap = (long long)numSMs * 4;
  const int grid = (int)(ntiles < cap ? ntiles : cap);
  wfs_corr_kernel<<<grid, kCorrThreads, smem, stream>>>(a, c);
  return cudaGetLastError();
}

}  // namespace shwfs
