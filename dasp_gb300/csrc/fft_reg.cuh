// Register-resident mixed-radix complex FFTs for one thread.
//
// fft<N, S>(x) transforms the N complex values in x in place:
//   X[k] = sum_n x[n] * exp(S * 2*pi*i * n*k / N),  S = -1 forward, +1 inverse
// (unnormalised, the sign convention of FFTW_FORWARD / FFTW_BACKWARD that the
// reference's centmodule.c plans use).
//
// Decimation in time with radix R = first factor of N among {4, 2, 3, 5}:
// the R strided sub-sequences are transformed recursively, twiddled by
// W_N^(r*k1) and combined with an R-point butterfly.  Every loop has a
// compile-time trip count, so after inlining all indices are constants and x
// stays in registers; the permutations between levels are register renames.
// Twiddles come from a __constant__ table computed at compile time (own
// Taylor-series cos/sin in double, rounded to float), indexed by compile-time
// offsets, so they become constant-bank operands.  The templates are also
// host-callable so the transforms can be checked on a machine without a GPU.
#pragma once
#include <cuda_runtime.h>

namespace shwfs {

// sizes with a twiddle table; each table holds W_N^e = exp(-2*pi*i*e/N)
// for e in [0, N).
constexpr int kTwSizes[] = {8, 10, 12, 15, 16, 20, 24, 25, 30, 32, 40, 48, 50, 60, 64};
constexpr int kNumTwSizes = sizeof(kTwSizes) / sizeof(int);

__host__ __device__ constexpr int tw_offset(int N) {
  int off = 0;
  for (int i = 0; i < kNumTwSizes; i++) {
    if (kTwSizes[i] == N) return off;
    off += kTwSizes[i];
  }
  return -1;
}
__host__ __device__ constexpr int tw_total() {
  int off = 0;
  for (int i = 0; i < kNumTwSizes; i++) off += kTwSizes[i];
  return off;
}

// compile-time cos/sin of 2*pi*e/N by octant reduction and a Taylor series
// in double (|x| <= pi/4, 14 terms: error far below float resolution)
constexpr double kPi = 3.14159265358979323846;
__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 14; k++) {
    term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 14; k++) {
    term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}
// (cos, sin) of 2*pi*e/N, exact quadrant/octant symmetry on the rational e/N
struct CS {
  double c, s;
};
__host__ __device__ constexpr CS cos_sin_frac(int e, int N) {
  e %= N;
  // 8*e/N = octant + remainder
  int q = (4 * e) / N;       // quadrant 0..3
  int r = 4 * e - q * N;     // remainder, angle = (q + r/N) * pi/2
  double c0 = 0.0, s0 = 0.0;
  if (2 * r <= N) {
    double x = kPi / 2.0 * r / N;
    c0 = taylor_cos(x);
    s0 = taylor_sin(x);
  } else {
    double x = kPi / 2.0 * (N - r) / N;
    c0 = taylor_sin(x);
    s0 = taylor_cos(x);
  }
  switch (q) {
    case 0: return CS{c0, s0};
    case 1: return CS{-s0, c0};
    case 2: return CS{-c0, -s0};
    default: return CS{s0, -c0};
  }
}
struct TwTable {
  float2 v[tw_total()];
};
__host__ __device__ constexpr TwTable make_twiddles() {
  TwTable t{};
  int off = 0;
  for (int i = 0; i < kNumTwSizes; i++) {
    int N = kTwSizes[i];
    for (int e = 0; e < N; e++) {
      CS cs = cos_sin_frac(e, N);
      // W_N^e = exp(-2*pi*i*e/N)
      t.v[off + e] = float2{(float)cs.c, (float)(-cs.s)};
    }
    off += N;
  }
  return t;
}
// one copy per translation unit (no relocatable device code needed)
static __constant__ TwTable c_tw = make_twiddles();
static constexpr TwTable h_tw = make_twiddles();
#ifdef __CUDA_ARCH__
#define c_twiddle (c_tw.v)
#else
#define c_twiddle (h_tw.v)
#endif

__host__ __device__ constexpr bool fft_size_supported(int N) {
  if (N < 2 || tw_offset(N) < 0) return false;
  while (N % 4 == 0) N /= 4;
  while (N % 2 == 0) N /= 2;
  while (N % 3 == 0) N /= 3;
  while (N % 5 == 0) N /= 5;
  return N == 1;
}

__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// i * a
__host__ __device__ __forceinline__ float2 cmuli(float2 a) { return make_float2(-a.y, a.x); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

__host__ __device__ constexpr int first_radix(int N) {
  return (N % 4 == 0 && N != 8) ? 4 : (N % 2 == 0 ? 2 : (N % 3 == 0 ? 3 : 5));
}

// small DFT butterflies, in place
template <int R, int S>
__host__ __device__ __forceinline__ void butterfly(float2 (&a)[R]);

template <>
__host__ __device__ __forceinline__ void butterfly<2, -1>(float2 (&a)[2]) {
  float2 t = a[0];
  a[0] = cadd(t, a[1]);
  a[1] = csub(t, a[1]);
}
template <>
__host__ __device__ __forceinline__ void butterfly<2, 1>(float2 (&a)[2]) {
  float2 t = a[0];
  a[0] = cadd(t, a[1]);
  a[1] = csub(t, a[1]);
}

template <int S>
__host__ __device__ __forceinline__ void bfly4(float2 (&a)[4]) {
  float2 s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
  float2 s13 = cadd(a[1], a[3]), d13 = csub(a[1], a[3]);
  // w = exp(S*i*pi/2) = S*i
  float2 id13 = cmuli(d13);
  if (S < 0) id13 = make_float2(-id13.x, -id13.y);
  a[0] = cadd(s02, s13);
  a[2] = csub(s02, s13);
  a[1] = cadd(d02, id13);
  a[3] = csub(d02, id13);
}
template <>
__host__ __device__ __forceinline__ void butterfly<4, -1>(float2 (&a)[4]) { bfly4<-1>(a); }
template <>
__host__ __device__ __forceinline__ void butterfly<4, 1>(float2 (&a)[4]) { bfly4<1>(a); }

template <int S>
__host__ __device__ __forceinline__ void bfly3(float2 (&a)[3]) {
  constexpr float h = 0.866025403784438647f;  // sin(2*pi/3)
  float2 t1 = cadd(a[1], a[2]);
  float2 t2 = csub(a[1], a[2]);
  float2 b = make_float2(a[0].x - 0.5f * t1.x, a[0].y - 0.5f * t1.y);
  float2 d = cscale(cmuli(t2), S * h);
  a[0] = cadd(a[0], t1);
  a[1] = cadd(b, d);
  a[2] = csub(b, d);
}
template <>
__host__ __device__ __forceinline__ void butterfly<3, -1>(float2 (&a)[3]) { bfly3<-1>(a); }
template <>
__host__ __device__ __forceinline__ void butterfly<3, 1>(float2 (&a)[3]) { bfly3<1>(a); }

template <int S>
__host__ __device__ __forceinline__ void bfly5(float2 (&a)[5]) {
  constexpr float c1 = 0.309016994374947424f;   // cos(2*pi/5)
  constexpr float c2 = -0.809016994374947424f;  // cos(4*pi/5)
  constexpr float s1 = 0.951056516295153572f;   // sin(2*pi/5)
  constexpr float s2 = 0.587785252292473129f;   // sin(4*pi/5)
  float2 t1 = cadd(a[1], a[4]), t3 = csub(a[1], a[4]);
  float2 t2 = cadd(a[2], a[3]), t4 = csub(a[2], a[3]);
  float2 b1 = make_float2(a[0].x + c1 * t1.x + c2 * t2.x, a[0].y + c1 * t1.y + c2 * t2.y);
  float2 b2 = make_float2(a[0].x + c2 * t1.x + c1 * t2.x, a[0].y + c2 * t1.y + c1 * t2.y);
  float2 d1 = cscale(cmuli(make_float2(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y)), (float)S);
  float2 d2 = cscale(cmuli(make_float2(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y)), (float)S);
  a[0] = cadd(a[0], cadd(t1, t2));
  a[1] = cadd(b1, d1);
  a[4] = csub(b1, d1);
  a[2] = cadd(b2, d2);
  a[3] = csub(b2, d2);
}
template <>
__host__ __device__ __forceinline__ void butterfly<5, -1>(float2 (&a)[5]) { bfly5<-1>(a); }
template <>
__host__ __device__ __forceinline__ void butterfly<5, 1>(float2 (&a)[5]) { bfly5<1>(a); }

// exp(S*2*pi*i*e/N) from the table of the top-level transform of size NT
template <int NT, int S>
__host__ __device__ __forceinline__ float2 twiddle(int e) {
  float2 w = c_twiddle[tw_offset(NT) + e];
  return S < 0 ? w : cconj(w);
}

// Transform the N values of x in place; NT is the top-level size (selects the
// twiddle table, whose stride for this level is NT/N).
template <int N, int S, int NT = N>
__host__ __device__ __forceinline__ void fft(float2 (&x)[N]) {
  if constexpr (N == 2 || N == 3 || N == 4 || N == 5) {
    butterfly<N, S>(x);
  } else {
    constexpr int R = first_radix(N);
    constexpr int M = N / R;
    float2 sub[R][M];
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
      for (int q = 0; q < M; q++) sub[r][q] = x[R * q + r];
#pragma unroll
    for (int r = 0; r < R; r++) fft<M, S, NT>(sub[r]);
#pragma unroll
    for (int k1 = 0; k1 < M; k1++) {
      float2 t[R];
      t[0] = sub[0][k1];
#pragma unroll
      for (int r = 1; r < R; r++) {
        if (k1 == 0)
          t[r] = sub[r][0];
        else
          t[r] = cmul(sub[r][k1], twiddle<NT, S>(r * k1 * (NT / N)));
      }
      butterfly<R, S>(t);
#pragma unroll
      for (int k2 = 0; k2 < R; k2++) x[k1 + M * k2] = t[k2];
    }
  }
}

}  // namespace shwfs
