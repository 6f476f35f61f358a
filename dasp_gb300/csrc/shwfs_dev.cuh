// Device-side definitions shared by the WFS kernels: the per-launch argument
// block, the counter-based noise generator and the twiddle table.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_reg.cuh"

namespace shwfs {

// pipeline pieces a launch performs (bit mask)
enum : int {
  kForm = 1,        // field -> FFT -> |F|^2 -> [prebin] -> [PSF] -> bin -> normalise -> sky
  kNoiseCounter = 2,  // Poisson + read noise from the counter-based stream
  kPost = 4,        // threshold .. centroids, bimg/cents written
  kStorePreNoise = 8  // write the pre-noise image (and Poisson flag) to global memory
};

// Round keys of one seed, precomputed on the host: round r uses
// (k0 + r*0x9E3779B9, k1 + r*0xBB67AE85), the schedule of philox4x32_10.
// Kept in the kernel parameters, they are read as constant-bank operands.
struct PhiloxKeys {
  uint32_t k0[10], k1[10];
};

struct WfsArgs {
  // geometry
  int nsubx, nsubaps, p, N, C, m, ncen, P, padded, preBin;
  int psfDim;    // 0 none, 2 one PSF, 4 one PSF per subaperture
  int phaseAmp;  // 0 phase only, 1 phase + amplitude planes
  int W;         // phase row width (elements)
  long long phsFrameStride;
  long long phsAmpOffset;  // elements from phase plane to amplitude plane
  int nlit, nframes;
  int TS;  // subapertures per CTA tile
  const int* lit;
  const int* unlit;  // unlit subapertures (nunlit), for kernels that zero their centroids
  int nunlit;
  const int* subflag;  // per subaperture: 1 = lit
  const float* phs;
  const float* pup;
  const float* tilt;
  const float* frac;
  const float* totsig;
  float sig;
  const float* sigArr;
  float sky;
  const float* skyArr;
  const float2* psfSpec;  // [npsf][P][P/2+1]
  const float* binT;
  const float* binN;
  const int* binII;  // output row of each input row
  const int* binLo;  // first contributing input row per output row
  const int* binHi;  // last contributing input row per output row
  float readNoise, readBg, floorv;
  int threshType, addPoisson, calsource;
  int opticalBinning, imageOnly;
  int useBrightest;
  const int* useBrightestArr;
  float pxlPower;
  const float* centWeight;
  int centWeightDim;
  int cob;  // centre-on-brightest: 0 window, 1 brightest, other faintest
  int fitSize, gaussianFit;
  float gMin, gRep;
  const float* fitMx;  // 5 x 6
  const float* calData;
  const int* calBounds;
  const float* calSteps;
  int calNSteps;
  const float* calCoeff;
  int calNCoeff;
  const float* refCents;
  float* bimg;
  long long bimgFrameStride;
  float* cents;
  long long centsFrameStride;
  unsigned char* poisFlag;  // per subap: Poisson applies (reference-stream mode)
  unsigned long long seed;
  PhiloxKeys philoxKeys;  // round keys of seed
  unsigned long long frame0;
  // when set (CUDA-graph replays), the noise frame index is read from this
  // device counter instead of frame0
  const unsigned long long* frameCtr;
  // CDF tables of the tabulated Poisson sampler (device global memory)
  const struct PoisTab* poisTab;
  // 1: the post stages write bimg but no centroids (correlation
  // centroiding computes them afterwards from bimg)
  int skipCents;
  // 1: the noise/centroid kernel also zeroes the centroids of the unlit
  // subapertures (set by launch_post when it takes that work over)
  int zeroUnlit;
  // optional second destination of the final images (same layout as bimg),
  // e.g. the device alias of a pinned host array; written by the
  // noise/centroid kernel when launch_post reports it
  float* bimgOut;
  // optional: the noise/centroid kernel copies the pipeline status word
  // (statusIn, device) to statusOut (the device alias of a pinned host
  // word) once the image-formation kernel has completed
  const int* statusIn;
  int* statusOut;
  int mode;
};

// a.philoxKeys from a.seed (host side, after a.seed is set)
inline void set_philox_keys(WfsArgs& a) {
  for (int r = 0; r < 10; r++) {
    a.philoxKeys.k0[r] = (uint32_t)a.seed + (uint32_t)r * 0x9E3779B9u;
    a.philoxKeys.k1[r] = (uint32_t)(a.seed >> 32) + (uint32_t)r * 0xBB67AE85u;
  }
}

__device__ __forceinline__ unsigned long long frame_base(const WfsArgs& a) {
  return a.frameCtr ? *a.frameCtr : a.frame0;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with a
// Weyl-sequence key schedule.
// ---------------------------------------------------------------------------
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const unsigned long long p0 = (unsigned long long)0xD2511F53u * c.x;
    const unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c.z;
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ U4 philox4x32_10_rk(U4 c, const PhiloxKeys& K) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    // each 32x32 -> 64-bit product as one widening multiply (lo and hi words)
    const unsigned long long p0 = (unsigned long long)0xD2511F53u * c.x;
    const unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c.z;
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
    U4 n;
    n.x = hi1 ^ c.y ^ K.k0[r];
    n.y = lo1;
    n.z = hi0 ^ c.w ^ K.k1[r];
    n.w = lo0;
    c = n;
  }
  return c;
}

// the streams' uniform in (0, 1) from one 32-bit word: 24 random bits,
// centred in their bin
__device__ __forceinline__ float u32_to_uniform(uint32_t w) {
  return ((float)(w >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// Sequential uniform stream for one (frame, subap, pixel, purpose).
struct CounterStream {
  U4 ctr;
  uint32_t k0, k1;
  U4 buf;
  int avail;
  __device__ __forceinline__ CounterStream(unsigned long long seed, unsigned long long frame, int subap,
                                           int pixel, int purpose) {
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32);
    ctr.x = 0;
    ctr.y = (uint32_t)pixel | ((uint32_t)purpose << 24);
    ctr.z = (uint32_t)subap;
    ctr.w = (uint32_t)frame;
    avail = 0;
  }
  __device__ __forceinline__ uint32_t next_u32() {
    if (avail == 0) {
      buf = philox4x32_10(ctr, k0, k1);
      ctr.x++;
      avail = 4;
    }
    uint32_t v = avail == 4 ? buf.x : (avail == 3 ? buf.y : (avail == 2 ? buf.z : buf.w));
    avail--;
    return v;
  }
  // uniform in (0, 1): 24 random bits, centred in their bin
  __device__ __forceinline__ float uniform() { return u32_to_uniform(next_u32()); }
};

// The same stream as CounterStream(seed, ...), with the seed's round keys
// taken from a PhiloxKeys block (kernel parameters) instead of computed
// per block.
struct KeyedStream {
  const PhiloxKeys& keys;
  U4 ctr;
  U4 buf;
  int avail;
  __device__ __forceinline__ KeyedStream(const PhiloxKeys& k, unsigned long long frame, int subap, int pixel,
                                         int purpose)
      : keys(k) {
    ctr.x = 0;
    ctr.y = (uint32_t)pixel | ((uint32_t)purpose << 24);
    ctr.z = (uint32_t)subap;
    ctr.w = (uint32_t)frame;
    avail = 0;
  }
  __device__ __forceinline__ uint32_t next_u32() {
    if (avail == 0) {
      buf = philox4x32_10_rk(ctr, keys);
      ctr.x++;
      avail = 4;
    }
    uint32_t v = avail == 4 ? buf.x : (avail == 3 ? buf.y : (avail == 2 ? buf.z : buf.w));
    avail--;
    return v;
  }
  __device__ __forceinline__ float uniform() { return u32_to_uniform(next_u32()); }
};

// log Gamma(x) by the Stirling series with upward recursion below 7, as the
// reference's loggam (cmod/src/centmodule.c:683-721), in float.
__device__ __forceinline__ float loggam_f(float x) {
  const float a[10] = {8.333333333333333e-02f, -2.777777777777778e-03f, 7.936507936507937e-04f,
                       -5.952380952380952e-04f, 8.417508417508418e-04f, -1.917526917526918e-03f,
                       6.410256410256410e-03f, -2.955065359477124e-02f, 1.796443723688307e-01f,
                       -1.39243221690590e+00f};
  if (x == 1.0f || x == 2.0f) return 0.0f;
  int n = 0;
  float x0 = x;
  if (x <= 7.0f) {
    n = (int)(7.0f - x);
    x0 = x + n;
  }
  float x2 = 1.0f / (x0 * x0);
  float gl0 = a[9];
#pragma unroll
  for (int k = 8; k >= 0; k--) gl0 = gl0 * x2 + a[k];
  float gl = gl0 / x0 + 0.918938533204672742f + (x0 - 0.5f) * __logf(x0) - x0;
  for (int k = 1; k <= n; k++) {
    gl -= __logf(x0 - 1.0f);
    x0 -= 1.0f;
  }
  return gl;
}

// Poisson deviate by inversion of one uniform u along the support ordered
// from the mode outwards.  The visited values always form an interval around
// the mode m = floor(lam); each step extends it by the more probable of its
// two neighbours (a fixed order that depends on lam only, so the inversion is
// exact up to float rounding).  The expected number of steps is about
// 1.5 sqrt(lam) (4.4 at lam 9.7), against lam + 1 for the search from 0.
// P(m) = exp(m log1p((lam - m)/m) - (lam - m) + c(m)), c(m) = m ln m - m - ln m!
// from Stirling's series for m >= 4 (truncation below 4e-8) and its exact
// values for m = 1..3; m = 0 gives P(0) = exp(-lam).
constexpr float kModalMaxLam = 64.0f;
__device__ __forceinline__ float poisson_modal(float u, float lam) {
  const float fm = floorf(lam);
  float lp = -lam;
  if (fm > 0.0f) {
    const float d = lam - fm;  // exact
    const float r = __fdividef(1.0f, fm);
    float c;
    if (fm >= 4.0f) {
      const float r2 = r * r;
      c = -0.5f * __logf(6.28318530717958648f * fm) -
          r * (1.0f / 12.0f - r2 * (1.0f / 360.0f - r2 * (1.0f / 1260.0f)));
    } else {
      c = fm == 1.0f ? -1.0f : (fm == 2.0f ? -1.30685281944005469f : -1.49592260322372630f);
    }
    lp = fm * log1pf(d * r) - d + c;
  }
  const float pm = __expf(lp);
  float F = pm;
  if (u <= F) return fm;
  const float ilam = __fdividef(1.0f, lam);
  float kup = fm + 1.0f, kdn = fm - 1.0f;
  float pup = pm * __fdividef(lam, kup);
  float pdn = pm * fm * ilam;  // 0 when m = 0
  // bound far in the tail (at least 10 sqrt(lam) + 20 for lam < 64): keeps
  // the search finite when float rounding leaves F just below u
  const int kmax = 2 * (int)lam + 40;
  for (int it = 0; it < kmax; it++) {
    const bool up = pup >= pdn;
    F += up ? pup : pdn;
    if (u <= F) return up ? kup : kdn;
    if (up) {
      kup += 1.0f;
      pup *= __fdividef(lam, kup);
    } else {
      pdn *= kdn * ilam;
      kdn -= 1.0f;
    }
  }
  return fm;
}

// Tables for Poisson(lam) with lam < 64 as the sum of two independent parts,
// Poisson(L) + Poisson(d), L = floor(lam), d = lam - L in [0, 1):
//   Poisson(L): Walker's alias method (Walker 1977; table construction of
//     Vose 1991) over the support 0..n_L-1 of Poisson(L), L = 1..63, built
//     on the host in double (each support runs until the upper tail is
//     below 2^-30, the last entry taking the remaining mass): one 32-bit
//     word w gives the column i = floor(w n_L / 2^32) and, from the low 32
//     bits of w n_L, either i or its alias -- integer arithmetic, two table
//     reads, no search;
//   Poisson(d): inversion of a uniform, the first four CDF terms without
//     branches, a short loop beyond them (probability < 2%).
// The sum of independent Poisson variables is Poisson, so the draw is exact
// up to the 2^-32 resolution of the keep thresholds and the float rounding
// of the inversion.  ~22 KB, staged into shared memory by the kernels that
// use it.
constexpr int kPoisTabL = 64;      // L = 0..63
constexpr int kPoisCdfMax = 4480;  // >= sum of the support lengths
struct PoisTab {
  uint32_t prob[kPoisCdfMax];  // keep the column itself when the coin (32 bits) is below this
  uint8_t alias[kPoisCdfMax];
  uint32_t offlen[kPoisTabL];  // first entry << 8 | support length (<= 255)
};

// Poisson(L), integer 0 <= L < 64, by the alias method on one 32-bit word w:
// the column is floor(w n / 2^32), the coin the low 32 bits of w n (uniform
// at 2^-32 / n resolution and independent of the column); L = 0 is a
// one-column table that always gives 0
__device__ __forceinline__ int poisson_table_int(const PoisTab& T, int L, uint32_t w) {
  const uint32_t e = T.offlen[L], n = e & 0xffu, o = e >> 8;
  const uint32_t i = __umulhi(w, n), coin = w * n;
  return coin < T.prob[o + i] ? (int)i : (int)T.alias[o + i];
}

// Poisson(d), 0 <= d < 1, by inversion of the uniform u4: the smallest j
// with u4 <= F_j, F_j the CDF (d = 0 gives F_0 = 1, hence j = 0, without a
// branch); the first four terms without branches
__device__ __forceinline__ int poisson_frac(float d, float u4) {
  float t = __expf(-d), F = t;
  int k2 = u4 > F ? 1 : 0;
  t *= d;
  F += t;
  k2 += u4 > F ? 1 : 0;
  t *= d * 0.5f;
  F += t;
  k2 += u4 > F ? 1 : 0;
  t *= d * (1.0f / 3.0f);
  F += t;
  if (u4 > F) {
    int j = 3;
    while (u4 > F && j < 40) {
      j++;
      t *= __fdividef(d, (float)j);
      F += t;
    }
    k2 = j;
  }
  return k2;
}

__device__ __forceinline__ float poisson_tab(const PoisTab& T, uint32_t w3, float u4, float lam) {
  const int L = (int)lam;
  const float d = lam - (float)L;  // exact
  return (float)(poisson_table_int(T, L, w3) + poisson_frac(d, u4));
}

// Below lambda 64 the modal inversion above (one uniform); above, Hormann's
// PTRS transformed rejection as in the reference (cmod/src/centmodule.c:
// 722-758), whose quick-accept region grows with lambda.  Both draw from the
// pixel's counter stream, so one Philox block usually suffices.
template <class Stream>
__device__ __forceinline__ float poisson_counter(Stream& st, float lam) {
  if (!(lam > 0.0f)) return 0.0f;
  if (lam < kModalMaxLam) return poisson_modal(st.uniform(), lam);
  const float slam = sqrtf(lam), loglam = __logf(lam);
  const float b = 0.931f + 2.53f * slam;
  const float a = -0.059f + 0.02483f * b;
  const float lninvalpha = __logf(1.1239f + 1.1328f / (b - 3.4f));
  const float vr = 0.9277f - 3.6224f / (b - 2.0f);
  for (int it = 0; it < 1000; it++) {
    const float U = st.uniform() - 0.5f;
    const float V = st.uniform();
    const float us = 0.5f - fabsf(U);
    const float kf = floorf((2.0f * a / us + b) * U + lam + 0.43f);
    if (us >= 0.07f && V <= vr) return kf;
    if (kf < 0.0f || (us < 0.013f && V > us)) continue;
    if (__logf(V) + lninvalpha - __logf(a / (us * us) + b) <= -lam + kf * loglam - loggam_f(kf + 1.0f))
      return kf;
  }
  return floorf(lam + 0.5f);  // unreachable in practice: bounded loop
}

// device address of the tables on the current device, built on first use
// (pois_table.cu)
cudaError_t pois_table_device(const PoisTab** out);

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) and the occupancy query of
// a kernel, done once per (device, kernel, shared memory, threads) and then
// cached: host round trips that each frame would otherwise repeat
// (ctasPerSM may be NULL)
cudaError_t kernel_smem_setup(const void* kern, int smem, int threads, int* ctasPerSM);

// one standard normal deviate from two uniforms (Box-Muller, cosine branch)
__device__ __forceinline__ float normal_from_uniforms(float u1, float u2) {
  const float q = -2.0f * __logf(u1);  // > 0: u1 < 1
  const float r = q * rsqrtf(q);
  return r * __cosf(6.28318530717958648f * u2 - 3.14159265358979324f) * -1.0f;
}

// one standard normal deviate from the stream's next two uniforms
template <class Stream>
__device__ __forceinline__ float normal_counter(Stream& st) {
  const float u1 = st.uniform(), u2 = st.uniform();
  return normal_from_uniforms(u1, u2);
}

// Counter-based noise of one quad of pixels -- pixels 4q .. 4q+3 of
// subaperture i in frame f (the last quad of an image may be partial):
// blocks 0, 1, 2 of the stream (seed, f, i, quad q, purpose 0).  Block 0
// holds two Box-Muller pairs, the four pixels' read-noise normals (cosine
// then sine branch of each pair); block 1 the four alias words and block 2
// the four inversion uniforms of the tabulated Poisson draws (lambda < 64).
// A pixel whose mean needs the rejection sampler (lambda >= 64) draws it
// from its own stream (seed, f, i, pixel, purpose 4); summing tabulated
// Poisson(63) parts would be exact there too, but measured slower than PTRS
// from lambda 64 on.  Three blocks for four pixels: every 32-bit word is used
// once.
constexpr uint32_t kPurposeQuad = 0u, kPurposePtrs = 4u;

// block b of the stream of quad `quad` of subaperture `subap` in `frame`
__device__ __forceinline__ U4 quad_block(const PhiloxKeys& K, uint32_t frame, uint32_t subap, uint32_t quad,
                                         uint32_t b) {
  U4 c;
  c.x = b;
  c.y = quad | (kPurposeQuad << 24);
  c.z = subap;
  c.w = frame;
  return philox4x32_10_rk(c, K);
}

// two standard normal deviates from two words (Box-Muller: cosine and sine
// branch of one pair)
__device__ __forceinline__ void normal_pair(uint32_t w1, uint32_t w2, float& g0, float& g1) {
  const float u1 = u32_to_uniform(w1), u2 = u32_to_uniform(w2);
  const float q = -2.0f * __logf(u1);  // > 0: u1 < 1
  const float r = q * rsqrtf(q);
  float sn, cs;
  __sincosf(6.28318530717958648f * u2 - 3.14159265358979324f, &sn, &cs);
  g0 = -r * cs;
  g1 = -r * sn;
}

// the read-noise normals of the quad's four pixels (block 0)
__device__ __forceinline__ void quad_normals(const PhiloxKeys& K, uint32_t frame, uint32_t subap, uint32_t quad,
                                             float (&g)[4]) {
  const U4 r = quad_block(K, frame, subap, quad, 0u);
  normal_pair(r.x, r.y, g[0], g[1]);
  normal_pair(r.z, r.w, g[2], g[3]);
}

// the read-noise normal of pixel `pixel` alone (its quad's block 0)
__device__ __forceinline__ float pixel_normal(const PhiloxKeys& K, uint32_t frame, uint32_t subap, uint32_t pixel) {
  const U4 r = quad_block(K, frame, subap, pixel >> 2, 0u);
  const bool hi = (pixel & 2u) != 0;
  float g0, g1;
  normal_pair(hi ? r.z : r.x, hi ? r.w : r.y, g0, g1);
  return (pixel & 1u) ? g1 : g0;
}

// Shot noise of the quad's pixels in place (blocks 1 and 2): v[k] becomes a
// Poisson(v[k]) draw of the tabulated sampler; lambda <= 0 or NaN draws 0.
// Pixels whose bit is set in `skip` keep their value: every pixel with
// lambda >= 64 must be among them (drawn by ptrs_pixel).
__device__ __forceinline__ void quad_poisson(const PhiloxKeys& K, uint32_t frame, uint32_t subap, uint32_t quad,
                                             const PoisTab& T, float (&v)[4], unsigned skip) {
  const U4 w = quad_block(K, frame, subap, quad, 1u);
  const U4 u = quad_block(K, frame, subap, quad, 2u);
  const uint32_t ws[4] = {w.x, w.y, w.z, w.w}, us[4] = {u.x, u.y, u.z, u.w};
  // the four alias-table draws first, without branches (skipped pixels draw
  // Poisson(0)), so that their shared-memory reads overlap; then the
  // fractional parts
  float lam[4];
  int kt[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    lam[k] = ((skip >> k) & 1u) ? 0.0f : fmaxf(v[k], 0.0f);
    kt[k] = poisson_table_int(T, (int)lam[k], ws[k]);
  }
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (!((skip >> k) & 1u))
      v[k] = (float)(kt[k] + poisson_frac(lam[k] - (float)(int)lam[k], u32_to_uniform(us[k])));
}

// shot noise of a pixel with lambda >= 64 from its own stream (PTRS)
__device__ __forceinline__ float ptrs_pixel(const PhiloxKeys& K, uint32_t frame, uint32_t subap, uint32_t pixel,
                                            float lam) {
  KeyedStream st(K, frame, (int)subap, (int)pixel, (int)kPurposePtrs);
  return poisson_counter(st, lam);
}

// ptrs_pixel as an out-of-line call (the same stream, keys from the seed),
// for a rare path of a kernel whose registers are tight
static __device__ __noinline__ float ptrs_pixel_cold(unsigned long long seed, uint32_t frame, uint32_t subap,
                                              uint32_t pixel, float lam) {
  CounterStream st(seed, frame, (int)subap, (int)pixel, (int)kPurposePtrs);
  return poisson_counter(st, lam);
}

// floor(w / d) for 0 <= w < 2^22 and d >= 1 with the float reciprocal
// inv_d ~ 1/d, corrected to the exact quotient
__device__ __forceinline__ int div_small(int w, int d, float inv_d) {
  int q = (int)((float)w * inv_d);
  if (q * d > w) q--;
  else if ((q + 1) * d <= w) q++;
  return q;
}

// readCCD threshold (cmod/src/centmodule.c:785-817)
__device__ __forceinline__ float threshold_px(float v, float floorv, int threshType) {
  if (threshType == 0) return v < floorv ? 0.0f : v - floorv;
  if (threshType == 1) return v < floorv ? 0.0f : v;
  return v;
}

}  // namespace shwfs
