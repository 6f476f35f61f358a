// GEMM-DFT ("precision") form of the WFS step on the tcgen05 tensor cores.
//
// For a tile of 128 subapertures (one per TMEM lane / MMA row):
//
//   GEMM1  F[s, (o,re|im)] = E[s, k] . W2[(o,re|im), k]          bf16 -> f32 (TMEM)
//          E = pup*exp(i(phs - tilt)) as [Re E | Im E] over the p x p pixels
//          (k < 2p^2), W2 = real embedding of the 2-D DFT restricted to the
//          c x c outputs that survive the central crop (addPowerSpecCentral,
//          cmod/src/centmodule.c:430-471), 64 complex outputs per chunk
//   |F|^2  per thread (its own subaperture), split into bf16 hi/lo
//   GEMM2  B[s, q] += I[s, o] . Kc[q, o]                          bf16 -> f32 (TMEM)
//          Kc = the whole linear chain 180-degree placement -> [prebin] ->
//          spot-PSF circular convolution -> clip -> binImage, as one matrix
//          (cmod/src/centmodule.c:504, 1816-1827)
//
// then normalisation, sky, noise, threshold and the shared post stages
// (post_tile) exactly as the FP32 kernel.  Precision: one bf16 pass, or three
// split-product passes (a.b ~ ah.bh + ah.bl + al.bh) with f32 accumulation.
//
// Constants (W2, Kc, hi and lo) are laid out on the host in the tensor-core
// shared-memory order (K-major 8x8 core matrices, no swizzle) and streamed
// into shared memory with bulk asynchronous copies; MMAs are issued by one
// thread and tracked with mbarriers.  Every wait is bounded: a wait that runs
// out records an error for the host instead of hanging.
#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>

#include <cmath>
#include <vector>

#include "gemm_form.h"
#include "tc_sm103.cuh"
#include "wfs_plain.cuh"

namespace shwfs {

namespace {

constexpr int kGemmThreads = 512;
constexpr int kTileSubaps = 128;
constexpr uint32_t kTmemCols = 512;
constexpr int kWaitIter = 1 << 22;
constexpr uint32_t kLBO = 128;  // bytes between core matrices along K

__device__ __forceinline__ uint16_t bf16_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf16_val(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }

struct GemmSmem {
  uint32_t a1, w0, w1, a2, kc, img;  // byte offsets in dynamic smem
  uint32_t total;
};

__host__ __device__ inline GemmSmem gemm_smem_layout(const GemmGeom& g, int m) {
  GemmSmem L;
  const uint32_t a1 = (uint32_t)kTileSubaps * g.K1 * 2 * 2;            // E hi + lo
  const uint32_t img = (uint32_t)kTileSubaps * m * m * 4;              // post-stage images
  const uint32_t r0 = a1 > img ? a1 : img;
  const uint32_t wst = (uint32_t)128 * g.KC * 2 * 2;                   // one W2 stage, hi + lo
  const uint32_t a2 = (uint32_t)kTileSubaps * 64 * 2 * 2;              // |F|^2 chunk hi + lo
  const uint32_t kc = (uint32_t)g.N2 * 64 * 2 * 2;                     // Kc chunk hi + lo
  L.a1 = 0;
  L.img = 0;
  L.w0 = (r0 + 1023) & ~1023u;
  L.w1 = L.w0 + wst;
  L.a2 = L.w1 + wst;
  L.kc = L.a2 + a2;
  L.total = L.kc + kc;
  return L;
}

struct Bars {
  uint64_t w[2], wfree[2], d1[2], k, d2;
};

template <int PASSES>
__global__ void __launch_bounds__(kGemmThreads, 1)
    wfs_gemm_kernel(const WfsArgs a, const GemmGeom g, int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ Bars bars;
  __shared__ uint32_t s_tmem;
  __shared__ int s_subap[kTileSubaps];
  __shared__ int s_frame[kTileSubaps];
  __shared__ float s_tilt[256];
  __shared__ float s_cw[256];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p = a.p, pp = p * p, m = a.m, mm = m * m;
  const GemmSmem L = gemm_smem_layout(g, m);
  uint8_t* A1hi = smem + L.a1;
  uint8_t* A1lo = A1hi + (size_t)kTileSubaps * g.K1 * 2;
  uint8_t* Wst[2] = {smem + L.w0, smem + L.w1};
  uint8_t* A2hi = smem + L.a2;
  uint8_t* A2lo = A2hi + kTileSubaps * 64 * 2;
  uint8_t* KChi = smem + L.kc;
  float* imgs = reinterpret_cast<float*>(smem + L.img);
  const uint32_t sboE = (uint32_t)(g.K1 / 8) * 128;
  const uint32_t sboW = (uint32_t)(g.KC / 8) * 128;
  const uint32_t sbo64 = 8 * 128;
  const uint32_t wHalf = (uint32_t)128 * g.KC * 2;   // bytes of the hi half of a W2 stage
  const uint32_t kHalf = (uint32_t)g.N2 * 64 * 2;    // bytes of the hi half of a Kc chunk

  for (int k = tid; k < pp; k += blockDim.x) s_tilt[k] = a.tilt[k];
  if (a.centWeightDim == 2)
    for (int k = tid; k < mm; k += blockDim.x) s_cw[k] = a.centWeight[k];
  if (warp == 0) {
    tc::tmem_alloc<kTmemCols>(&s_tmem);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&bars.w[i], 1);
      tc::mbar_init(&bars.wfree[i], 1);
      tc::mbar_init(&bars.d1[i], 1);
    }
    tc::mbar_init(&bars.k, 1);
    tc::mbar_init(&bars.d2, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t tD1[2] = {tmem, tmem + 128};
  const uint32_t tD2 = tmem + 256;
  constexpr uint32_t idesc1 = tc::idesc_bf16_f32(128, 128);
  const uint32_t idesc2 = tc::idesc_bf16_f32(128, g.N2);
  const int nks1 = g.K1 / 16;          // k-steps of GEMM1
  const int ksPerChunk = g.KC / 16;
  bool ok = true;

  // global counters (continue across tiles) for barrier parities
  uint32_t gW = 0;   // W2 chunk loads issued (thread 0)
  uint32_t gC = 0;   // output chunks processed (all threads)

  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + kTileSubaps - 1) / kTileSubaps;

  // ---- thread 0: constant streaming and MMA issue ----
  // The W2 K-chunks of a tile form one sequence j = oc*nkc + kc (global index
  // gW + j across tiles) through a two-stage ring: chunk j+1 is fetched while
  // chunk j's MMAs run.  Chunk 0 of the next tile is fetched during the last
  // chunk of this one (the constants do not depend on the tile).
  const int nseq = g.noc * g.nkc;
  auto w2_load = [&](uint32_t gidx, int j) {
    const uint32_t s = gidx & 1;
    if (gidx >= 2 && !tc::mbar_wait(&bars.wfree[s], ((gidx >> 1) - 1) & 1, kWaitIter)) ok = false;
    tc::mbar_expect_tx(&bars.w[s], 2 * wHalf);
    tc::bulk_g2s(Wst[s], g.w2 + (size_t)j * 2 * wHalf, 2 * wHalf, &bars.w[s]);
  };
  auto kc_load = [&](int oc) {
    tc::mbar_expect_tx(&bars.k, 2 * kHalf);
    tc::bulk_g2s(KChi, g.kc2 + (size_t)oc * 2 * kHalf, 2 * kHalf, &bars.k);
  };
  auto issue_gemm1 = [&](int oc, uint32_t dcol, uint32_t gbase, bool more_tiles) {
    for (int kc = 0; kc < g.nkc; kc++) {
      const int j = oc * g.nkc + kc;
      const uint32_t gidx = gbase + j;
      const uint32_t s = gidx & 1;
      if (!tc::mbar_wait(&bars.w[s], (gidx >> 1) & 1, kWaitIter)) ok = false;
      tc::fence_after_sync();
      const int k0 = kc * ksPerChunk;
      const int k1 = min(nks1, k0 + ksPerChunk);
      const uint32_t whi = tc::smem_addr(Wst[s]), wlo = whi + wHalf;
      const uint32_t ehi = tc::smem_addr(A1hi), elo = tc::smem_addr(A1lo);
      for (int ks = k0; ks < k1; ks++) {
        const uint32_t eoff = (uint32_t)ks * 2 * kLBO, woff = (uint32_t)(ks - k0) * 2 * kLBO;
        const uint32_t acc0 = (kc > 0 || ks > k0) ? 1u : 0u;
        tc::mma_bf16(dcol, tc::smem_desc(ehi + eoff, kLBO, sboE), tc::smem_desc(whi + woff, kLBO, sboW), idesc1, acc0);
        if (PASSES == 3) {
          tc::mma_bf16(dcol, tc::smem_desc(ehi + eoff, kLBO, sboE), tc::smem_desc(wlo + woff, kLBO, sboW), idesc1, 1u);
          tc::mma_bf16(dcol, tc::smem_desc(elo + eoff, kLBO, sboE), tc::smem_desc(whi + woff, kLBO, sboW), idesc1, 1u);
        }
      }
      tc::mma_commit(&bars.wfree[s]);
      if (j + 1 < nseq)
        w2_load(gidx + 1, j + 1);
      else if (more_tiles)
        w2_load(gidx + 1, 0);
    }
  };

  if (tid == 0 && blockIdx.x < ntiles) {
    w2_load(0, 0);
    kc_load(0);
  }
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long w0 = tile * kTileSubaps;
    const int ns = (int)min((long long)kTileSubaps, nwork - w0);
    const bool more = tile + gridDim.x < ntiles;
    for (int s = tid; s < kTileSubaps; s += blockDim.x) {
      if (s < ns) {
        const long long w = w0 + s;
        s_frame[s] = (int)(w / a.nlit);
        s_subap[s] = a.lit[w % a.nlit];
      }
    }
    __syncthreads();

    // ---- E = pup*exp(i(phs - tilt)), split into bf16 hi/lo (row = subap);
    // work items (subap, pixel), subap fastest ----
    for (int w = tid; w < kTileSubaps * pp; w += blockDim.x) {
      const int s = w & (kTileSubaps - 1), pix = w >> 7;
      float er = 0.f, ei = 0.f;
      if (s < ns) {
        const int i = s_subap[s];
        const int sy = i / a.nsubx, sx = i - sy * a.nsubx;
        const int r = pix / p, j = pix - r * p;
        const float t = a.phs[(long long)s_frame[s] * a.phsFrameStride + (long long)(sy * p + r) * a.W + sx * p + j] -
                        s_tilt[pix];
        float sn, cs;
        sincosf(t, &sn, &cs);
        const float pu = a.pup[(long long)i * pp + pix];
        er = pu * cs;
        ei = pu * sn;
      }
      const uint16_t hr = bf16_bits(er), hi_ = bf16_bits(ei);
      const uint32_t offr = tc::kmajor_offset(s, pix, kLBO, sboE), offi = tc::kmajor_offset(s, pp + pix, kLBO, sboE);
      *reinterpret_cast<uint16_t*>(A1hi + offr) = hr;
      *reinterpret_cast<uint16_t*>(A1lo + offr) = bf16_bits(er - bf16_val(hr));
      *reinterpret_cast<uint16_t*>(A1hi + offi) = hi_;
      *reinterpret_cast<uint16_t*>(A1lo + offi) = bf16_bits(ei - bf16_val(hi_));
    }
    for (int w = tid; w < kTileSubaps * (g.K1 - 2 * pp); w += blockDim.x) {
      const int s = w & (kTileSubaps - 1), k = 2 * pp + (w >> 7);
      const uint32_t off = tc::kmajor_offset(s, k, kLBO, sboE);
      *reinterpret_cast<uint16_t*>(A1hi + off) = 0;
      *reinterpret_cast<uint16_t*>(A1lo + off) = 0;
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    if (tid == 0) {
      issue_gemm1(0, tD1[gC & 1], gW, more);
      tc::mma_commit(&bars.d1[gC & 1]);
    }
    for (int oc = 0; oc < g.noc; oc++, gC++) {
      const uint32_t buf = gC & 1;
      // chunk oc+1 runs on the tensor cores while chunk oc is read out; its
      // D1 buffer was last read before the previous iteration's barrier
      if (tid == 0 && oc + 1 < g.noc) {
        issue_gemm1(oc + 1, tD1[(gC + 1) & 1], gW, more);
        tc::mma_commit(&bars.d1[(gC + 1) & 1]);
      }
      if (!tc::mbar_wait(&bars.d1[buf], (gC >> 1) & 1, kWaitIter)) ok = false;
      // A2 and the Kc stage are free once the previous chunk's GEMM2 completed
      if (oc > 0) {
        if (!tc::mbar_wait(&bars.d2, (gC - 1) & 1, kWaitIter)) ok = false;
        if (tid == 0) kc_load(oc);
      }
      tc::fence_after_sync();
      // ---- |F|^2 of 64 outputs: warp w reads lanes 32*(w%4), columns
      // 32*(w/4) .. +31 (16 complex outputs) ----
      {
        const int row = 32 * (warp & 3) + lane;
        const int qtr = warp >> 2;
        uint32_t ph_[8], pl_[8];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          float v[8];
          tc::tmem_ld8(tD1[buf] + ((uint32_t)(32 * (warp & 3)) << 16) + qtr * 32 + q * 8, v);
          tc::tmem_ld_wait();
#pragma unroll
          for (int e = 0; e < 4; e += 2) {
            const float I0 = v[2 * e] * v[2 * e] + v[2 * e + 1] * v[2 * e + 1];
            const float I1 = v[2 * e + 2] * v[2 * e + 2] + v[2 * e + 3] * v[2 * e + 3];
            const uint16_t h0 = bf16_bits(I0), h1 = bf16_bits(I1);
            const uint16_t l0 = bf16_bits(I0 - bf16_val(h0)), l1 = bf16_bits(I1 - bf16_val(h1));
            ph_[q * 2 + e / 2] = (uint32_t)h0 | ((uint32_t)h1 << 16);
            pl_[q * 2 + e / 2] = (uint32_t)l0 | ((uint32_t)l1 << 16);
          }
        }
#pragma unroll
        for (int c8 = 0; c8 < 2; c8++) {
          const uint32_t off = tc::kmajor_offset(row, qtr * 16 + c8 * 8, kLBO, sbo64);
          *reinterpret_cast<uint4*>(A2hi + off) = make_uint4(ph_[4 * c8], ph_[4 * c8 + 1], ph_[4 * c8 + 2], ph_[4 * c8 + 3]);
          *reinterpret_cast<uint4*>(A2lo + off) = make_uint4(pl_[4 * c8], pl_[4 * c8 + 1], pl_[4 * c8 + 2], pl_[4 * c8 + 3]);
        }
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (tid == 0) {
        if (!tc::mbar_wait(&bars.k, gC & 1, kWaitIter)) ok = false;
        tc::fence_after_sync();
        const uint32_t ahi = tc::smem_addr(A2hi), alo = tc::smem_addr(A2lo);
        const uint32_t khi = tc::smem_addr(KChi), klo = khi + kHalf;
        for (int ks = 0; ks < 4; ks++) {
          const uint32_t off = (uint32_t)ks * 2 * kLBO;
          const uint32_t acc0 = (oc > 0 || ks > 0) ? 1u : 0u;
          tc::mma_bf16(tD2, tc::smem_desc(ahi + off, kLBO, sbo64), tc::smem_desc(khi + off, kLBO, sbo64), idesc2, acc0);
          if (PASSES == 3) {
            tc::mma_bf16(tD2, tc::smem_desc(ahi + off, kLBO, sbo64), tc::smem_desc(klo + off, kLBO, sbo64), idesc2, 1u);
            tc::mma_bf16(tD2, tc::smem_desc(alo + off, kLBO, sbo64), tc::smem_desc(khi + off, kLBO, sbo64), idesc2, 1u);
          }
        }
        tc::mma_commit(&bars.d2);
      }
    }
    gW += nseq;
    // ---- binned image: normalise, sky, noise, threshold -> shared memory;
    // warp w reads lanes 32*(w%4), pixel columns 32*(w/4) + 128*j .. +31 ----
    if (!tc::mbar_wait(&bars.d2, (gC - 1) & 1, kWaitIter)) ok = false;
    if (tid == 0 && more) kc_load(0);  // Kc stage free: prefetch for the next tile
    tc::fence_after_sync();
    {
      const int s = 32 * (warp & 3) + lane;
      const int qtr = warp >> 2;
      const bool live = s < ns;
      const int i = live ? s_subap[s] : 0;
      const float totsig = a.totsig[i];
      const float fr = a.frac[i];
      const float scale = totsig > 0.f ? (a.sigArr ? a.sigArr[i] / totsig : a.sig * fr / totsig) : 1.f;
      const float skyv = a.sky * fr;
      const bool pflag = totsig > 0.f || skyv > 0.f || a.skyArr;
      const bool pois = a.addPoisson == 1 && a.calsource == 0 && pflag;
      const float rn = a.calsource == 0 ? a.readNoise : 0.f;
      const unsigned long long frm = frame_base(a) + (live ? s_frame[s] : 0);
      for (int cb = qtr * 32; cb < mm; cb += 128) {
      const int c1 = min(mm, cb + 32);
      for (int q0 = cb; q0 < c1; q0 += 8) {
        float v[8];
        tc::tmem_ld8(tD2 + ((uint32_t)(32 * (warp & 3)) << 16) + q0, v);
        tc::tmem_ld_wait();
        if (!live) continue;
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int pix = q0 + e;
          if (pix >= c1) break;
          float x = v[e];
          if (totsig > 0.f) x *= scale;
          if (skyv > 0.f) x += skyv;
          if (a.skyArr) x += a.skyArr[(long long)i * mm + pix];
          CounterStream st(a.seed, frm, i, pix, 0);
          const float gnoise = rn != 0.f ? normal_counter(st) : 0.f;
          if (pois) x = poisson_counter(st, x);
          x += rn != 0.f ? rn * gnoise + a.readBg : a.readBg;
          imgs[s * mm + pix] = threshold_px(x, a.floorv, a.threshType);
        }
      }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    post_tile(a, ns, s_subap, s_frame, s_cw, [&](int s) { return imgs + s * mm; }, [&](int) { return mm; });
    __syncthreads();  // the next tile's E build overwrites the image region
  }
  if (!ok) atomicOr(err, 2);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc<kTmemCols>(tmem);
}

// ---------------------------------------------------------------- host side

uint16_t host_bf16(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);  // inf/nan
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float host_bf16_val(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}
void put_split(uint8_t* hi, uint8_t* lo, uint32_t off, double v) {
  const float f = (float)v;
  const uint16_t h = host_bf16(f);
  const uint16_t l = host_bf16(f - host_bf16_val(h));
  memcpy(hi + off, &h, 2);
  memcpy(lo + off, &l, 2);
}
uint32_t host_kmajor(int row, int k, uint32_t sbo) {
  return (uint32_t)(row >> 3) * sbo + (uint32_t)(k >> 3) * kLBO + (uint32_t)(row & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

}  // namespace

bool gemm_geometry(const GemmSpec& sp, GemmGeom* g) {
  const int K1 = ((2 * sp.p * sp.p + 15) / 16) * 16;
  const int mm = sp.m * sp.m;
  const int N2 = ((mm + 15) / 16) * 16;
  if (K1 > 208 || N2 > 256 || mm > 256 || sp.p * sp.p > 256) return false;
  g->K1 = K1;
  g->N2 = N2;
  g->noc = (sp.c * sp.c + 63) / 64;
  int KC = 64;
  for (; KC >= 16; KC -= 16) {
    GemmGeom t = *g;
    t.KC = KC;
    // dynamic limit 227 KB minus the kernel's ~3.2 KB of static shared memory
    if (gemm_smem_layout(t, sp.m).total <= 227 * 1024 - 4096) break;
  }
  if (KC < 16) return false;
  g->KC = KC;
  g->nkc = (K1 + KC - 1) / KC;
  return true;
}

int gemm_smem_bytes(const GemmGeom& g, int m) { return (int)gemm_smem_layout(g, m).total; }

void gemm_build_w2(const GemmSpec& sp, const GemmGeom& g, std::vector<uint8_t>& out) {
  const int p = sp.p, pp = p * p, c = sp.c, N = sp.N;
  const size_t half = (size_t)128 * g.KC * 2;
  out.assign((size_t)g.noc * g.nkc * 2 * half, 0);
  const uint32_t sbo = (uint32_t)(g.KC / 8) * 128;
  for (int oc = 0; oc < g.noc; oc++)
    for (int ol = 0; ol < 64; ol++) {
      const int o = oc * 64 + ol;
      if (o >= c * c) continue;
      const int ku = sp.ro + o / c, kv = sp.ro + o % c;
      for (int k = 0; k < 2 * pp; k++) {
        const int pix = k < pp ? k : k - pp;
        const int i = pix / p, j = pix % p;
        const long long e = ((long long)ku * i + (long long)kv * j) % N;
        const double th = -2.0 * M_PI * (double)e / N;
        const double cr = cos(th), si = sin(th);
        // row 2ol: Re F = sum Re W Re E - Im W Im E ; row 2ol+1: Im F = Im W Re E + Re W Im E
        const double vre = k < pp ? cr : -si;
        const double vim = k < pp ? si : cr;
        const int kc = k / g.KC, kk = k % g.KC;
        uint8_t* hi = out.data() + ((size_t)oc * g.nkc + kc) * 2 * half;
        uint8_t* lo = hi + half;
        put_split(hi, lo, host_kmajor(2 * ol, kk, sbo), vre);
        put_split(hi, lo, host_kmajor(2 * ol + 1, kk, sbo), vim);
      }
    }
}

// The chain from one power-spectrum output o = (u, v) of the c x c crop to
// the binned image, applied to a unit impulse (all stages are linear):
// 180-degree placement into the paddedsize image (addPowerSpecCentral), block
// pre-binning with the reference's unbinned clip offset (prebinImage), the
// unnormalised circular convolution with the quadrant-swapped PSF that
// r2c * fftPsf -> c2r computes (P^2 * sum_ab h[a,b] f[(y-a)%P][(x-b)%P]),
// the central clip to C, and binImage with its weights.
void gemm_kc_matrix(const GemmSpec& sp, std::vector<double>& kc) {
  const int c = sp.c, cc = c * c, m = sp.m, mm = m * m, C = sp.C, P = sp.P, pad = sp.padded;
  kc.assign((size_t)mm * cc, 0.0);
  std::vector<double> hll((size_t)pad * pad), work((size_t)P * P), img((size_t)C * C), out((size_t)mm);
  for (int o = 0; o < cc; o++) {
    const int u = o / c, v = o % c;
    std::fill(hll.begin(), hll.end(), 0.0);
    hll[(size_t)(c - 1 - u + sp.rs) * pad + (c - 1 - v + sp.rs)] = 1.0;
    if (sp.psfDim) {
      const double* src = hll.data();
      std::vector<double> pre;
      if (sp.preBin > 1) {
        const int f = sp.preBin, scaled = pad / f;
        const int b = scaled > P ? P : scaled;
        const int off = scaled > P ? (scaled - P) / 2 : 0;
        const int o2 = scaled < P ? (P - scaled) / 2 : 0;
        pre.assign((size_t)P * P, 0.0);
        for (int i = 0; i < b; i++)
          for (int j = 0; j < b; j++) {
            double t = 0;
            for (int ii = 0; ii < f; ii++)
              for (int jj = 0; jj < f; jj++) t += hll[(size_t)(i * f + ii + off) * pad + j * f + jj + off];
            pre[(size_t)(i + o2) * P + j + o2] = t;
          }
        src = pre.data();
      }
      std::fill(work.begin(), work.end(), 0.0);
      for (int a = 0; a < P; a++)
        for (int b = 0; b < P; b++) {
          const double h = src[(size_t)a * P + b];
          if (h == 0.0) continue;
          for (int y = 0; y < P; y++)
            for (int x = 0; x < P; x++) {
              // quadrant-swapped PSF: f[y][x] = psf[(y + P/2) % P][(x + P/2) % P]
              const int fy = ((y - a) % P + P) % P, fx = ((x - b) % P + P) % P;
              work[(size_t)y * P + x] += h * sp.psf[(size_t)((fy + P / 2) % P) * P + (fx + P / 2) % P];
            }
        }
      const int off = (P - C) / 2;
      for (int y = 0; y < C; y++)
        for (int x = 0; x < C; x++) img[(size_t)y * C + x] = (double)P * P * work[(size_t)(y + off) * P + x + off];
    } else {
      for (int y = 0; y < C; y++)
        for (int x = 0; x < C; x++) img[(size_t)y * C + x] = hll[(size_t)y * pad + x];
    }
    // binImage (cmod/src/centmodule.c:609-651)
    if (C == m) {
      for (int q = 0; q < mm; q++) out[q] = img[q];
    } else {
      std::fill(out.begin(), out.end(), 0.0);
      const std::vector<float>&t = sp.binT, &n = sp.binN;
      const std::vector<int>& idx = sp.binIdx;
      int ii = 0;
      for (int i = 0; i < C; i++) {
        int jj = 0;
        const bool li = i == C - 1;
        for (int j = 0; j < C; j++) {
          const bool lj = j == C - 1;
          out[(size_t)ii * m + jj] += (double)t[i] * t[j] * img[(size_t)i * C + j];
          if (!lj && jj + 1 < m) out[(size_t)ii * m + jj + 1] += (double)t[i] * n[j] * img[(size_t)i * C + j + 1];
          if (!li && ii + 1 < m) {
            out[(size_t)(ii + 1) * m + jj] += (double)n[i] * t[j] * img[(size_t)(i + 1) * C + j];
            if (!lj && jj + 1 < m)
              out[(size_t)(ii + 1) * m + jj + 1] += (double)n[i] * n[j] * img[(size_t)(i + 1) * C + j + 1];
          }
          if (!lj) jj += idx[j];
        }
        if (!li) ii += idx[i];
      }
    }
    for (int q = 0; q < mm; q++) kc[(size_t)q * cc + o] = out[q];
  }
}

void gemm_build_kc(const GemmSpec& sp, const GemmGeom& g, const std::vector<double>& kc, std::vector<uint8_t>& out) {
  // kc: [m*m][c*c] dense, row-major
  const int mm = sp.m * sp.m, cc = sp.c * sp.c;
  const size_t half = (size_t)g.N2 * 64 * 2;
  out.assign((size_t)g.noc * 2 * half, 0);
  for (int oc = 0; oc < g.noc; oc++) {
    uint8_t* hi = out.data() + (size_t)oc * 2 * half;
    uint8_t* lo = hi + half;
    for (int q = 0; q < mm; q++)
      for (int ol = 0; ol < 64; ol++) {
        const int o = oc * 64 + ol;
        if (o >= cc) continue;
        put_split(hi, lo, host_kmajor(q, ol, 8 * 128), kc[(size_t)q * cc + o]);
      }
  }
}

cudaError_t launch_gemm(const WfsArgs& a, const GemmGeom& g, int passes, int numSMs, int* err, cudaStream_t stream) {
  const int smem = gemm_smem_bytes(g, a.m);
  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + kTileSubaps - 1) / kTileSubaps;
  const int grid = (int)(ntiles < numSMs ? (ntiles > 0 ? ntiles : 1) : numSMs);
  cudaError_t e;
  if (passes == 3) {
    e = cudaFuncSetAttribute(wfs_gemm_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    wfs_gemm_kernel<3><<<grid, kGemmThreads, smem, stream>>>(a, g, err);
  } else {
    e = cudaFuncSetAttribute(wfs_gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    wfs_gemm_kernel<1><<<grid, kGemmThreads, smem, stream>>>(a, g, err);
  }
  return cudaGetLastError();
}

}  // namespace shwfs
