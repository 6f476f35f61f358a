// GEMM-DFT ("precision") form of the WFS image formation on the tcgen05
// tensor cores.
//
// For a tile of 128 subapertures (one per TMEM lane / MMA row):
//
//   GEMM1  F[s, (o,re|im)] = E[s, k] . W2[(o,re|im), k]                 -> f32 (TMEM)
//          E = pup*exp(i(phs - tilt)) as [Re E | Im E] over the p x p pixels,
//          W2 = real embedding of the 2-D DFT restricted to the c x c outputs
//          that survive the central crop (addPowerSpecCentral,
//          cmod/src/centmodule.c:430-471), CW complex outputs per chunk
//          (64, or wider when that needs fewer chunks)
//   |F|^2  per thread (its own subaperture row)
//   GEMM2  B[s, q] += I[s, o] . Kc[q, o]                                   -> f32 (TMEM)
//          Kc = the whole linear chain 180-degree placement -> [prebin] ->
//          spot-PSF circular convolution -> clip -> binImage, as one matrix
//          (cmod/src/centmodule.c:504, 1816-1827)
//
// then normalisation and sky (cmod/src/centmodule.c:1829-1872); the binned
// pre-noise image goes to bimg, and wfs_post_kernel (wfs_post.cu) adds the
// noise and computes the centroids.
//
// Operand formats: bf16 (one pass, or three split-product passes
// a.b ~ ah.bh + ah.bl + al.bh), fp16 (one pass; |F|^2 scaled per
// subaperture by 1/(sum pup)^2 so that it stays far from the fp16 range
// limit) and tf32 (one pass, kind::tf32).  Accumulation is always f32.
//
// Warp roles (608 threads):
//   warps 0-7   epilogue: thread t owns MMA row r = t & 127 (its
//               subaperture, TMEM lane) and column half t >> 7; reads D1 and
//               writes |F|^2 into the GEMM2 operand, reads D2 and stores the
//               image
//   warps 8-15  field build: E of the next tile (row r, every other pixel
//               group), one tile ahead of GEMM1 when two field buffers fit,
//               so that its global loads overlap the epilogue and the MMAs
//   warp 16     GEMM1 issuer: the GEMM1 MMAs over the W2 ring, into two or
//               three D1 accumulator buffers
//   warp 17     GEMM2 producer: streams Kc chunks (NK-stage ring) and
//               issues the GEMM2 MMAs
//   warp 18     W2 loader: refills the NW-stage W2 ring with bulk
//               asynchronous copies as soon as the MMAs reading a stage
//               complete
// All hand-offs are mbarriers (no block-wide barrier inside the tile loop);
// every wait is bounded and a wait that runs out records an error for the
// host instead of hanging.
//
// Constants (W2, Kc) are laid out on the host in the tensor-core
// shared-memory order (K-major 8-row x 16-byte core matrices, no swizzle).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <string.h>

#include <cmath>
#include <type_traits>
#include <vector>

#include "gemm_form.h"
#include "tc_sm103.cuh"
#include "wfs_plain.cuh"

namespace shwfs {

namespace {

constexpr int kConsumers = 512;
constexpr int kEpiWarps = 8;    // warps 0-7: D1/D2 epilogue
constexpr int kFieldWarps = 8;  // warps 8-15: field build
constexpr int kGemmThreads = kConsumers + 96;  // + GEMM1 issuer, GEMM2 producer, W2 loader
constexpr int kTileSubaps = 128;
constexpr uint32_t kTmemCols = 512;
constexpr long long kWaitCycles = 4000000000LL;  // about 2 s at the maximum SM clock
constexpr uint32_t kLBO = 128;  // bytes between core matrices along K

// TMEM columns: D1 buffers 0 and 1 at 0 and 128, D2 at 256 (N2 <= 256
// columns), a third D1 buffer at 384 when N2 <= 128

// ---- element encodings (device) ----
template <int FMT>
__device__ __forceinline__ uint32_t enc(float x) {
  if constexpr (FMT == kFmtBF16) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
  } else if constexpr (FMT == kFmtFP16) {
    return __half_as_ushort(__float2half_rn(x));
  } else {  // tf32: round to nearest even on the top 19 bits, kept as f32 bits
    const uint32_t u = __float_as_uint(x);
    return (u + 0xfffu + ((u >> 13) & 1u)) & 0xffffe000u;
  }
}
template <int FMT>
__device__ __forceinline__ float dec(uint32_t b) {
  if constexpr (FMT == kFmtBF16) {
    return __bfloat162float(__ushort_as_bfloat16((unsigned short)b));
  } else if constexpr (FMT == kFmtFP16) {
    return __half2float(__ushort_as_half((unsigned short)b));
  } else {
    return __uint_as_float(b);
  }
}

// 8 consecutive K elements of one row (16 bytes for 16-bit formats, 32 for
// tf32) at byte offset `off` of a K-major tile: hi (and lo) parts
template <int FMT, bool SPLIT>
__device__ __forceinline__ void store8(uint8_t* hi, uint8_t* lo, uint32_t off, const float (&x)[8]) {
  if constexpr (FMT == kFmtTF32) {
    uint32_t h[8];
#pragma unroll
    for (int e = 0; e < 8; e++) h[e] = enc<FMT>(x[e]);
    // elements 0-3 and 4-7 are in consecutive core matrices along K
    *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(hi + off + kLBO) = make_uint4(h[4], h[5], h[6], h[7]);
  } else {
    uint32_t h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const uint32_t h0 = enc<FMT>(x[2 * e]), h1 = enc<FMT>(x[2 * e + 1]);
      h[e] = h0 | (h1 << 16);
      if constexpr (SPLIT) {
        const uint32_t l0 = enc<FMT>(x[2 * e] - dec<FMT>(h0)), l1 = enc<FMT>(x[2 * e + 1] - dec<FMT>(h1));
        l[e] = l0 | (l1 << 16);
      }
    }
    *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    if constexpr (SPLIT) *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

// byte offset of K element k of row `row` in a K-major no-swizzle tile whose
// row groups are sbo bytes apart (esz = bytes per element)
__host__ __device__ __forceinline__ uint32_t kmaj(int row, int k, int esz, uint32_t sbo) {
  const uint32_t kb = (uint32_t)(k * esz);
  return (uint32_t)(row >> 3) * sbo + (kb >> 4) * kLBO + (uint32_t)(row & 7) * 16u + (kb & 15u);
}

// phase -> [0, 2pi) reduction in float (Cody-Waite, 2pi = C1 + C2 with C1 =
// 201/32 exact in 8 bits), then the fast sine/cosine on |t| <= pi
__device__ __forceinline__ void sincos_reduced(float t, float* s, float* c) {
  const float k = rintf(t * 0.15915494309189535f);
  float r = fmaf(-k, 6.28125f, t);
  r = fmaf(-k, 1.9353071795864769e-3f, r);
  __sincosf(r, s, c);
}

struct Bars {
  uint64_t wfull[kGemmMaxNW], wfree[kGemmMaxNW];
  uint64_t kfull[kGemmMaxNK], kfree[kGemmMaxNK];
  uint64_t efull[2], efree[2];  // per field buffer
  uint64_t d1full[3], d1free[3];  // per D1 buffer (two or three)
  uint64_t a2full[2], a2free[2];  // per GEMM2 operand buffer
  uint64_t d2full, d2free;
  uint64_t ehelp;  // the epilogue warps' share of the first tile's field
};

template <int FMT, int PASSES>
__global__ void __launch_bounds__(kGemmThreads, 1)
    wfs_gemm_kernel(const WfsArgs a, const GemmGeom g, const float* __restrict__ iscale, int* err) {
  constexpr bool SPLIT = PASSES == 3;
  constexpr int ESZ = FMT == kFmtTF32 ? 4 : 2;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ Bars bars;
  __shared__ uint32_t s_tmem;
  __shared__ float s_tilt[256];
  __shared__ int s_poff[256];  // pixel -> (row, column) offset in the phase frame
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p = a.p, pp = p * p, ppr = (pp + 7) & ~7, mm = a.m * a.m;
  const GemmSmem L = gemm_smem_layout(g);
  uint8_t* A1hi = smem + L.a1;
  uint8_t* A1lo = A1hi + L.a1Half;
  uint8_t* A2hi = smem + L.a2;
  uint8_t* A2lo = A2hi + L.a2Half;
  const uint32_t sboE = (uint32_t)(g.K1 * ESZ / 16) * 128;
  const uint32_t sboW = (uint32_t)(g.KCB / 16) * 128;
  const uint32_t sbo2 = (uint32_t)(g.CW * ESZ / 16) * 128;
  const uint32_t d2c = gemm_d2_col(g);
  const int nseq = g.noc * g.nkc;
  const int K1B = g.K1 * ESZ;

  for (int k = tid; k < pp; k += blockDim.x) {
    s_tilt[k] = a.tilt[k];
    const int ii = k / p;
    s_poff[k] = ii * a.W + (k - ii * p);
  }
  if (tid == 0) s_abort = 0;
  if (warp == 0) {
    tc::tmem_alloc<kTmemCols>(&s_tmem);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < g.NW; i++) {
      tc::mbar_init(&bars.wfull[i], 1);
      tc::mbar_init(&bars.wfree[i], 1);
    }
    for (int i = 0; i < g.NK; i++) {
      tc::mbar_init(&bars.kfull[i], 1);
      tc::mbar_init(&bars.kfree[i], 1);
    }
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&bars.efull[i], kFieldWarps);
      tc::mbar_init(&bars.efree[i], 1);
    }
    for (int i = 0; i < 3; i++) {
      tc::mbar_init(&bars.d1full[i], 1);
      tc::mbar_init(&bars.d1free[i], kEpiWarps);
    }
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&bars.a2full[i], kEpiWarps);
      tc::mbar_init(&bars.a2free[i], 1);
    }
    tc::mbar_init(&bars.d2full, 1);
    tc::mbar_init(&bars.d2free, kEpiWarps);
    tc::mbar_init(&bars.ehelp, kEpiWarps);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // the noise/centroid kernel queued behind this one (programmatic launch)
  // may start its CTAs on SMs this grid leaves free; it reads nothing of
  // ours before griddepcontrol.wait, which waits for this whole grid
  if (tid == 0) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const uint32_t tmem = s_tmem;
  bool ok = true;
  auto wait = [&](uint64_t* bar, uint32_t parity) {
    if (!tc::mbar_wait_abortable(bar, parity, &s_abort, kWaitCycles)) ok = false;
  };

  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + kTileSubaps - 1) / kTileSubaps;
  const int myTiles = blockIdx.x < ntiles ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  // the epilogue warps build half of the first tile's field, which their
  // first D1 chunk waits for anyway (the field warps go on to the next tile)
  const bool help = myTiles > 0;

  if (warp == kConsumers / 32) {
    // ================= GEMM1 producer (MMA issue only) =================
    // The whole warp runs the loop (so that counters and descriptors stay
    // warp-uniform); lane 0 issues the MMAs and commits.  W2 chunk gJ sits
    // in ring stage cs with phase bit cph (the loader warp fills the ring);
    // output chunk gC goes to D1 buffer d1b in round d1r.
    if (myTiles > 0) {
      const bool leader = lane == 0;
      const uint32_t idesc1 = tc::idesc_f32acc(FMT, 128, 2 * g.CW);
      const uint32_t wbase = tc::smem_addr(smem + L.w);
      // descriptors: the 14-bit start-address field (bits 0-13, in 16-byte
      // units) advances by 16 per k-step of 256 bytes; all addresses < 256 KB
      // field buffer of tile lt: (lt & 1) when double buffered
      const uint64_t dEh0 = tc::smem_desc(tc::smem_addr(A1hi), kLBO, sboE);
      const uint64_t dEl0 = tc::smem_desc(tc::smem_addr(A1lo), kLBO, sboE);
      const uint64_t dEstep = (uint64_t)((L.a1Half * (SPLIT ? 2u : 1u)) >> 4);
      const uint64_t dW0 = tc::smem_desc(wbase, kLBO, sboW);
      const uint64_t dWstage = (uint64_t)(L.wStage >> 4), dWlo = (uint64_t)(L.wHalf >> 4);
      int cs = 0;
      uint32_t cph = 0;
      int d1b = 0;
      uint32_t d1r = 0;
      for (int lt = 0; lt < myTiles; lt++) {
        // field buffer eb; its uses alternate when double buffered
        const int eb = g.dbE ? (lt & 1) : 0;
        wait(&bars.efull[eb], (uint32_t)((g.dbE ? (lt >> 1) : lt) & 1));
        if (lt == 0 && help) wait(&bars.ehelp, 0);
        tc::fence_after_sync();
        const uint64_t dEh = dEh0 + (eb ? dEstep : 0);
        const uint64_t dEl = dEl0 + (eb ? dEstep : 0);
        for (int oc = 0; oc < g.noc; oc++) {
          if (d1r > 0) wait(&bars.d1free[d1b], (d1r - 1) & 1);
          tc::fence_after_sync();
          const uint32_t dcol = tmem + gemm_d1_col(g, d1b);
          int ks = 0;
          for (int kc = 0; kc < g.nkc; kc++) {
            wait(&bars.wfull[cs], cph);
            const uint64_t dWh = dW0 + (uint64_t)cs * dWstage;
            const int ks1 = min(K1B, (kc + 1) * g.KCB) >> 5;
            if (leader) {
              for (uint64_t wo = 0; ks < ks1; ks++, wo += 16) {
                const uint64_t eo = (uint64_t)ks * 16;
                tc::mma<FMT>(dcol, dEh + eo, dWh + wo, idesc1, ks > 0 ? 1u : 0u);
                if constexpr (SPLIT) {
                  tc::mma<FMT>(dcol, dEh + eo, dWh + dWlo + wo, idesc1, 1u);
                  tc::mma<FMT>(dcol, dEl + eo, dWh + wo, idesc1, 1u);
                }
              }
              tc::mma_commit(&bars.wfree[cs]);
            }
            ks = ks1;
            if (++cs == g.NW) {
              cs = 0;
              cph ^= 1u;
            }
          }
          if (leader) tc::mma_commit(&bars.d1full[d1b]);
          if (++d1b == g.nd1) {
            d1b = 0;
            d1r++;
          }
        }
        if (leader) tc::mma_commit(&bars.efree[eb]);
      }
    }
    __syncwarp();
  } else if (warp == kConsumers / 32 + 2) {
    // ================= W2 loader =================
    // refills each ring stage as soon as the MMAs that read it complete, so
    // that the MMA issuer never waits on a copy it has to start itself
    if (myTiles > 0) {
      const int totalJ = myTiles * nseq;
      int s = 0, lseq = 0;
      uint32_t round = 0;
      for (int J = 0; J < totalJ; J++) {
        if (round > 0) wait(&bars.wfree[s], (round - 1) & 1);
        if (lane == 0) {
          tc::mbar_expect_tx(&bars.wfull[s], L.wStage);
          tc::bulk_g2s(smem + L.w + (size_t)s * L.wStage, g.w2 + (size_t)lseq * L.wStage, L.wStage, &bars.wfull[s]);
        }
        if (++lseq == nseq) lseq = 0;
        if (++s == g.NW) {
          s = 0;
          round++;
        }
      }
    }
    __syncwarp();
  } else if (warp == kConsumers / 32 + 1) {
    // ================= GEMM2 producer (whole warp, lane 0 issues) =================
    if (myTiles > 0) {
      const bool leader = lane == 0;
      const int totalK = myTiles * g.noc;
      const uint32_t idesc2 = tc::idesc_f32acc(FMT, 128, g.N2);
      const uint32_t kbase = tc::smem_addr(smem + L.k);
      int nextK = 0, kseq = 0;
      auto kload = [&](int s) {  // chunk kseq -> stage s
        if (leader) {
          tc::mbar_expect_tx(&bars.kfull[s], L.kStage);
          tc::bulk_g2s(smem + L.k + (size_t)s * L.kStage, g.kc2 + (size_t)kseq * L.kStage, L.kStage,
                       &bars.kfull[s]);
        }
        nextK++;
        if (++kseq == g.noc) kseq = 0;
      };
      for (int s0 = 0; s0 < g.NK && nextK < totalK; s0++) kload(s0);
      // GEMM2 operand buffer of chunk gK: (gK & 1) when double buffered
      const uint64_t dAh0 = tc::smem_desc(tc::smem_addr(A2hi), kLBO, sbo2);
      const uint64_t dAl0 = tc::smem_desc(tc::smem_addr(A2lo), kLBO, sbo2);
      const uint64_t dAstep = (uint64_t)((L.a2Half * (SPLIT ? 2u : 1u)) >> 4);
      uint32_t gK = 0;
      const uint64_t dK0 = tc::smem_desc(kbase, kLBO, sbo2);
      const uint64_t dKstage = (uint64_t)(L.kStage >> 4), dKlo = (uint64_t)(L.kHalf >> 4);
      const uint32_t dcol = tmem + d2c;
      const int ks2 = g.CW * ESZ / 32;  // k-steps of one chunk
      int ksg = 0;
      uint32_t kph = 0;
      for (int lt = 0; lt < myTiles; lt++) {
        for (int oc = 0; oc < g.noc; oc++) {
          if (oc == 0 && lt >= 1) wait(&bars.d2free, (lt - 1) & 1);
          const uint32_t ab = g.dbA2 ? (gK & 1) : 0;
          wait(&bars.a2full[ab], g.dbA2 ? ((gK >> 1) & 1) : (gK & 1));
          const uint64_t dAh = dAh0 + (ab ? dAstep : 0), dAl = dAl0 + (ab ? dAstep : 0);
          wait(&bars.kfull[ksg], kph);
          tc::fence_after_sync();
          const uint64_t dKh = dK0 + (uint64_t)ksg * dKstage;
          if (leader) {
            for (int ks = 0; ks < ks2; ks++) {
              const uint64_t o = (uint64_t)ks * 16;
              const uint32_t acc0 = (oc > 0 || ks > 0) ? 1u : 0u;
              tc::mma<FMT>(dcol, dAh + o, dKh + o, idesc2, acc0);
              if constexpr (SPLIT) {
                tc::mma<FMT>(dcol, dAh + o, dKh + dKlo + o, idesc2, 1u);
                tc::mma<FMT>(dcol, dAl + o, dKh + o, idesc2, 1u);
              }
            }
            tc::mma_commit(&bars.a2free[ab]);
            tc::mma_commit(&bars.kfree[ksg]);
            if (oc == g.noc - 1) tc::mma_commit(&bars.d2full);
          }
          if (nextK < totalK) {
            wait(&bars.kfree[ksg], kph);
            kload(ksg);
          }
          gK++;
          if (++ksg == g.NK) {
            ksg = 0;
            kph ^= 1u;
          }
        }
      }
    }
    __syncwarp();
  } else {
    // ================= consumers =================
    // warps 0-7: epilogue (TMEM lane quarter warp & 3, column half h);
    // warps 8-15: field build (row r, pixel-group parity h)
    const int r = tid & 127, h = (tid >> 7) & 1;
    const bool fieldRole = warp >= kEpiWarps;
    const bool vecPup = (pp & 3) == 0 && ((uintptr_t)a.pup & 15) == 0;
    const bool vecPhs = (p & 1) == 0 && (a.W & 1) == 0 && (a.phsFrameStride & 1) == 0 && ((uintptr_t)a.phs & 7) == 0;
    const bool vecOut = (mm & 3) == 0 && (a.bimgFrameStride & 3) == 0 && ((uintptr_t)a.bimg & 15) == 0;
    const uint32_t lanebase = (uint32_t)(32 * (warp & 3)) << 16;

    struct Row {
      bool live;
      int sub, frm, li;
    };
    // this thread's row (subaperture-frame) of tile lt
    auto row_of = [&](int lt) {
      Row o{false, 0, 0, 0};
      const long long w = (blockIdx.x + (long long)lt * gridDim.x) * kTileSubaps + r;
      if (lt < myTiles && w < nwork) {
        o.live = true;
        o.frm = (int)(w / a.nlit);
        o.li = (int)(w - (long long)o.frm * a.nlit);
        o.sub = a.lit[o.li];
      }
      return o;
    };

    // ---- field build: E = pup*exp(i(phs - tilt)) of this row in pixel
    // groups g8 of 8 pixels, Re at K = pix, Im at K = ppr + pix
    auto load_group = [&](const Row& R, const float* ph, const float* pu, int g8, float (&phv)[8],
                          float (&puv)[8]) {
      const int pix0 = g8 * 8;
      if (R.live && g.pupT) {
        // grouped copy: lanes (consecutive lit subapertures) read
        // consecutive 32-byte entries; zero past the last pixel
        const float* pt = g.pupT + ((long long)g8 * a.nlit + R.li) * 8;
        const float4 u0 = *reinterpret_cast<const float4*>(pt);
        const float4 u1 = *reinterpret_cast<const float4*>(pt + 4);
        puv[0] = u0.x; puv[1] = u0.y; puv[2] = u0.z; puv[3] = u0.w;
        puv[4] = u1.x; puv[5] = u1.y; puv[6] = u1.z; puv[7] = u1.w;
      } else if (R.live && vecPup && pix0 + 8 <= pp) {
        const float4 u0 = *reinterpret_cast<const float4*>(pu + pix0);
        const float4 u1 = *reinterpret_cast<const float4*>(pu + pix0 + 4);
        puv[0] = u0.x; puv[1] = u0.y; puv[2] = u0.z; puv[3] = u0.w;
        puv[4] = u1.x; puv[5] = u1.y; puv[6] = u1.z; puv[7] = u1.w;
      } else {
#pragma unroll
        for (int e = 0; e < 8; e++) puv[e] = (R.live && pix0 + e < pp) ? pu[pix0 + e] : 0.f;
      }
      if (R.live && vecPhs) {
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          const int pix = pix0 + e;
          if (pix < pp) {
            // the column is even: the pair stays in the row
            const float2 v2 = *reinterpret_cast<const float2*>(ph + s_poff[pix]);
            phv[e] = v2.x;
            phv[e + 1] = v2.y;
          } else {
            phv[e] = phv[e + 1] = 0.f;
          }
        }
      } else {
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int pix = pix0 + e;
          phv[e] = (R.live && pix < pp) ? ph[s_poff[pix]] : 0.f;
        }
      }
    };
    auto emit_group = [&](uint8_t* Ehi, uint8_t* Elo, const Row& R, int g8, const float (&phv)[8],
                          const float (&puv)[8]) {
      const int pix0 = g8 * 8;
      float er[8], ei[8];
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const int pix = pix0 + e;
        er[e] = 0.f;
        ei[e] = 0.f;
        if (R.live && pix < pp) {
          const float t = phv[e] - s_tilt[pix];
          float sn, cs;
          if constexpr (SPLIT) {
            sincosf(t, &sn, &cs);
          } else {
            sincos_reduced(t, &sn, &cs);
          }
          er[e] = puv[e] * cs;
          ei[e] = puv[e] * sn;
        }
      }
      store8<FMT, SPLIT>(Ehi, Elo, kmaj(r, pix0, ESZ, sboE), er);
      store8<FMT, SPLIT>(Ehi, Elo, kmaj(r, ppr + pix0, ESZ, sboE), ei);
    };
    const int ng8 = ppr / 8;
    // the field of row R into (Ehi, Elo): this thread's pixel groups of
    // parity h in [g0, g1) (two groups' loads in flight)
    auto build_field = [&](const Row& R, uint8_t* Ehi, uint8_t* Elo, int g0, int g1) {
      const int sy = R.sub / a.nsubx, sx = R.sub - sy * a.nsubx;
      const float* ph = a.phs + (long long)R.frm * a.phsFrameStride + (long long)sy * p * a.W + sx * p;
      const float* pu = a.pup + (long long)R.sub * pp;
      for (int g8 = g0 + h; g8 < g1; g8 += 4) {
        float phA[8], puA[8], phB[8], puB[8];
        const bool two = g8 + 2 < g1;
        load_group(R, ph, pu, g8, phA, puA);
        if (two) load_group(R, ph, pu, g8 + 2, phB, puB);
        emit_group(Ehi, Elo, R, g8, phA, puA);
        if (two) emit_group(Ehi, Elo, R, g8 + 2, phB, puB);
      }
    };
    // with help the first tile's groups split at gMid (even): the field
    // warps take [0, gMid), the epilogue warps [gMid, ng8)
    const int gMid = (ng8 / 2) & ~1;

    {
      // ---- field build (warps 8-15): row r, pixel groups of parity h.
      // With help the epilogue warps run the first pass of this loop too
      // (one copy of the field code for both roles), then leave it.
      Row next = row_of(0);
      const int fieldTiles = fieldRole ? myTiles : (help ? 1 : 0);
      for (int lt = 0; lt < fieldTiles; lt++) {
        const Row R = next;
        if (fieldRole) next = row_of(lt + 1);  // its index loads overlap this tile
        const int eb = g.dbE ? (lt & 1) : 0;
        uint8_t* Ehi = A1hi + (size_t)eb * L.a1Half * (SPLIT ? 2 : 1);
        uint8_t* Elo = Ehi + L.a1Half;
        const int reuse = g.dbE ? 2 : 1;  // tiles between two uses of a buffer
        if (lt >= reuse) wait(&bars.efree[eb], (uint32_t)(((lt - reuse) / reuse) & 1));
        if (lt < reuse && fieldRole) {
          // zero K padding beyond 2*ppr once per buffer (none when 2*ppr is
          // a multiple of 16)
          for (int k = 2 * ppr + h; k < g.K1; k += 2) {
            const uint32_t off = kmaj(r, k, ESZ, sboE);
            if constexpr (ESZ == 4) {
              *reinterpret_cast<uint32_t*>(Ehi + off) = 0u;
            } else {
              *reinterpret_cast<uint16_t*>(Ehi + off) = 0;
              if constexpr (SPLIT) *reinterpret_cast<uint16_t*>(Elo + off) = 0;
            }
          }
        }
        const bool split = lt == 0 && help;
        build_field(R, Ehi, Elo, split && !fieldRole ? gMid : 0, split && fieldRole ? gMid : ng8);
        tc::fence_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(fieldRole ? &bars.efull[eb] : &bars.ehelp);
      }
    }
    if (!fieldRole) {
      // ---- epilogue ----
      int d1b = 0;
      uint32_t d1r = 0, gA = 0;
      // binned image of tile lt (row P) from D2: normalise, sky -> bimg
      // per-row image scale and sky level, computed a tile before their D2
      // read-out so the scattered loads are off the read-out's critical path
      struct RowNorm {
        float scale, skyv;
      };
      auto row_norm = [&](const Row& P) {
        const int i = P.sub;
        const float totsig = a.totsig[i], fr = a.frac[i];
        float scale = totsig > 0.f ? (a.sigArr ? a.sigArr[i] / totsig : a.sig * fr / totsig) : 1.f;
        if (iscale) scale = scale / iscale[i];  // undo the fp16 range scaling
        return RowNorm{scale, a.sky * fr};
      };
      auto read_D2 = [&](int lt, const Row& P, const RowNorm& nv) {
        const int i = P.sub;
        wait(&bars.d2full, lt & 1);
        tc::fence_after_sync();
        const float scale = nv.scale;  // exactly 1 when there is nothing to scale
        const float skyv = nv.skyv;
        float* out = a.bimg + (long long)P.frm * a.bimgFrameStride + (long long)i * mm;
        const float* skyA = a.skyArr ? a.skyArr + (long long)i * mm : nullptr;
        for (int cb = h * 32; cb < mm; cb += 64) {
          uint32_t v[32];
          tc::tmem_ld32(tmem + d2c + lanebase + cb, v);
          tc::tmem_ld_wait();
          if (!P.live) continue;
          const int n = min(32, mm - cb);
          float x[32];
#pragma unroll
          for (int e = 0; e < 32; e++) {
            x[e] = __uint_as_float(v[e]);
            x[e] *= scale;
            if (skyv > 0.f) x[e] += skyv;
            if (skyA && e < n) x[e] += skyA[cb + e];
          }
          if (vecOut) {  // n is a multiple of 4 here
#pragma unroll
            for (int e = 0; e < 32; e += 4)
              if (e < n) *reinterpret_cast<float4*>(out + cb + e) = make_float4(x[e], x[e + 1], x[e + 2], x[e + 3]);
          } else {
#pragma unroll
            for (int e = 0; e < 32; e++)
              if (e < n) out[cb + e] = x[e];
          }
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&bars.d2free);
      };

      // one output chunk of the current tile: |F|^2 of the CW/2 complex
      // outputs in columns h CW .. h CW + CW - 1 of this row -> the GEMM2
      // operand (K h CW/2 .. h CW/2 + CW/2 - 1)
      auto chunk = [&](float isc) {
        wait(&bars.d1full[d1b], d1r & 1);
        tc::fence_after_sync();
        const uint32_t col = tmem + gemm_d1_col(g, d1b) + lanebase + h * g.CW;
        // A2 buffer of this chunk
        const uint32_t ab = g.dbA2 ? (gA & 1) : 0;
        uint8_t* Ahi = A2hi + (size_t)ab * L.a2Half * (SPLIT ? 2 : 1);
        uint8_t* Alo = Ahi + L.a2Half;
        auto a2_wait = [&]() {
          // A2 is free once the previous chunk's GEMM2 has completed
          if (g.dbA2) {
            if (gA >= 2) wait(&bars.a2free[ab], ((gA >> 1) - 1) & 1);
          } else if (gA >= 1) {
            wait(&bars.a2free[0], (gA - 1) & 1);
          }
        };
        if (g.CW == 64) {
          float I[32];
          {
            // both halves in flight before one wait
            uint32_t v0[32], v1[32];
            tc::tmem_ld32(col, v0);
            tc::tmem_ld32(col + 32, v1);
            tc::tmem_ld_wait();
#pragma unroll
            for (int e = 0; e < 16; e++) {
              I[e] = (__uint_as_float(v0[2 * e]) * __uint_as_float(v0[2 * e]) +
                      __uint_as_float(v0[2 * e + 1]) * __uint_as_float(v0[2 * e + 1])) * isc;
              I[16 + e] = (__uint_as_float(v1[2 * e]) * __uint_as_float(v1[2 * e]) +
                           __uint_as_float(v1[2 * e + 1]) * __uint_as_float(v1[2 * e + 1])) * isc;
            }
          }
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&bars.d1free[d1b]);
          a2_wait();
#pragma unroll
          for (int k8 = 0; k8 < 4; k8++) {
            float x8[8];
#pragma unroll
            for (int e = 0; e < 8; e++) x8[e] = I[k8 * 8 + e];
            store8<FMT, SPLIT>(Ahi, Alo, kmaj(r, h * 32 + k8 * 8, ESZ, sbo2), x8);
          }
        } else {
          // wider chunks: 64 columns (32 complex outputs) at a time with
          // one wait, then 16 at a time, each stored as soon as it is computed
          a2_wait();
          int u = 0;
          for (; u + 64 <= g.CW; u += 64) {
            uint32_t v0[32], v1[32];
            tc::tmem_ld32(col + u, v0);
            tc::tmem_ld32(col + u + 32, v1);
            tc::tmem_ld_wait();
#pragma unroll
            for (int k8 = 0; k8 < 4; k8++) {
              const uint32_t* vv = k8 < 2 ? v0 : v1;
              const int o = (k8 & 1) * 16;
              float x8[8];
#pragma unroll
              for (int e = 0; e < 8; e++)
                x8[e] = (__uint_as_float(vv[o + 2 * e]) * __uint_as_float(vv[o + 2 * e]) +
                         __uint_as_float(vv[o + 2 * e + 1]) * __uint_as_float(vv[o + 2 * e + 1])) * isc;
              store8<FMT, SPLIT>(Ahi, Alo, kmaj(r, h * (g.CW / 2) + u / 2 + k8 * 8, ESZ, sbo2), x8);
            }
          }
          for (; u < g.CW; u += 16) {
            float v16[16];
            tc::tmem_ld16_sync(col + u, v16);
            float x8[8];
#pragma unroll
            for (int e = 0; e < 8; e++) x8[e] = (v16[2 * e] * v16[2 * e] + v16[2 * e + 1] * v16[2 * e + 1]) * isc;
            store8<FMT, SPLIT>(Ahi, Alo, kmaj(r, h * (g.CW / 2) + u / 2, ESZ, sbo2), x8);
          }
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&bars.d1free[d1b]);
        }
        if (++d1b == g.nd1) {
          d1b = 0;
          d1r++;
        }
        tc::fence_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&bars.a2full[ab]);
        gA++;
      };

      Row prev{false, 0, 0, 0};
      Row cur = row_of(0);
      RowNorm prevN{1.f, 0.f};
      RowNorm curN = row_norm(cur);
      float isc = (iscale && cur.live) ? iscale[cur.sub] : 1.f;
      for (int lt = 0; lt < myTiles; lt++) {
        const Row next = row_of(lt + 1);
        const float iscn = (iscale && next.live) ? iscale[next.sub] : 1.f;
        const RowNorm nextN = row_norm(next);  // used two read-outs from now
        for (int oc = 0; oc < g.noc; oc++) {
          if (oc == 0 && lt >= 1) read_D2(lt - 1, prev, prevN);
          chunk(isc);
        }
        prev = cur;
        prevN = curN;
        cur = next;
        curN = nextN;
        isc = iscn;
      }
      if (myTiles > 0) read_D2(myTiles - 1, prev, prevN);
    }
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
// IEEE binary16, round to nearest even (finite inputs of magnitude < 65520)
uint16_t host_f16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7fffffffu;
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // overflow -> inf
  if (ax < 0x38800000u) {                                    // below 2^-14: subnormal, unit 2^-24
    float v;
    memcpy(&v, &ax, 4);
    return (uint16_t)(sign | (uint32_t)std::nearbyint(v * 16777216.0f));
  }
  uint32_t h = ((((ax >> 23) - 127 + 15) & 0x1fu) << 10) | ((ax & 0x7fffffu) >> 13);
  const uint32_t rem = ax & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return (uint16_t)(sign | h);
}
uint32_t host_tf32(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return (u + 0xfffu + ((u >> 13) & 1u)) & 0xffffe000u;
}
// one constant in the operand format; with split, hi and lo parts
void put_val(int fmt, bool split, uint8_t* hi, uint8_t* lo, uint32_t off, double v) {
  const float f = (float)v;
  if (fmt == kFmtTF32) {
    const uint32_t b = host_tf32(f);
    memcpy(hi + off, &b, 4);
  } else if (fmt == kFmtFP16) {
    const uint16_t b = host_f16(f);
    memcpy(hi + off, &b, 2);
  } else {
    const uint16_t h = host_bf16(f);
    memcpy(hi + off, &h, 2);
    if (split) {
      const uint16_t l = host_bf16(f - host_bf16_val(h));
      memcpy(lo + off, &l, 2);
    }
  }
}

template <int FMT, int PASSES>
cudaError_t launch_one(const WfsArgs& a, const GemmGeom& g, const float* iscale, int numSMs, int* err,
                       cudaStream_t stream) {
  const int smem = (int)gemm_smem_layout(g).total;
  const long long nwork = (long long)a.nlit * a.nframes;
  const long long ntiles = (nwork + kTileSubaps - 1) / kTileSubaps;
  const int grid = (int)(ntiles < numSMs ? (ntiles > 0 ? ntiles : 1) : numSMs);
  cudaError_t e = kernel_smem_setup((const void*)wfs_gemm_kernel<FMT, PASSES>, smem, kGemmThreads, nullptr);
  if (e != cudaSuccess) return e;
  wfs_gemm_kernel<FMT, PASSES><<<grid, kGemmThreads, smem, stream>>>(a, g, iscale, err);
  return cudaGetLastError();
}

}  // namespace

namespace {

// GEMM1 output-chunk widths for a c x c crop: for each chunk count below
// that of 64-wide chunks, the narrowest multiple of 16 covering the crop in
// that many chunks, when GEMM1 N = 2 CW <= 256 and two D1 buffers and D2 fit
// the 512 TMEM columns; fewest chunks first, 64 last
std::vector<int> chunk_widths(int cc, int N2) {
  std::vector<int> widths;
  for (int k = (cc + 127) / 128; k < (cc + 63) / 64; k++) {
    const int cw = 16 * ((cc + 16 * k - 1) / (16 * k));
    if (cw <= 64 || 2 * cw > 256 || 4 * cw + N2 > 512) continue;
    bool dup = false;
    for (int w : widths) dup = dup || w == cw;
    if (!dup) widths.push_back(cw);
  }
  widths.push_back(64);
  return widths;
}

// the stagings of chunk width cw that fit shared memory, in preference
// order: four k-steps per W2 chunk, then two field buffers (one-pass 16-bit
// formats), two |F|^2 buffers, two Kc stages, as long as the W2 ring keeps
// enough stages (as deep as shared memory allows)
std::vector<GemmGeom> stagings_of_width(GemmGeom g, int cw, int cc, int passes) {
  std::vector<GemmGeom> out;
  const int esz = g.fmt == kFmtTF32 ? 4 : 2;
  // dynamic limit: 227 KB minus the kernel's static shared memory (< 4 KB)
  const uint32_t limit = 227 * 1024 - 4096;
  g.CW = cw;
  g.noc = (cc + cw - 1) / cw;
  g.nd1 = (cw == 64 && g.N2 <= 128) ? 3 : 2;
  for (int kcb = passes == 1 ? 128 : 64; kcb >= 64; kcb -= 64)
    for (int db = (passes == 1 && esz == 2) ? 1 : 0; db >= 0; db--)
      for (int da = 1; da >= 0; da--)
        for (int nk = 2; nk >= 1; nk--) {
          GemmGeom t = g;
          t.KCB = kcb;
          t.nkc = (t.K1 * esz + kcb - 1) / kcb;
          t.dbE = db;
          t.dbA2 = da;
          t.NK = nk;
          t.NW = 0;
          const GemmSmem base = gemm_smem_layout(t);
          if (base.total > limit) continue;
          int nw = (int)((limit - base.total) / base.wStage);
          if (nw > kGemmMaxNW) nw = kGemmMaxNW;
          if (nw < (nk == 2 ? 3 : 2)) continue;
          t.NW = nw;
          out.push_back(t);
        }
  return out;
}

}  // namespace

bool gemm_geometry(const GemmSpec& sp, int fmt, int passes, GemmGeom* g) {
  if (fmt != kFmtBF16 && fmt != kFmtFP16 && fmt != kFmtTF32) return false;
  if (passes != 1 && !(passes == 3 && fmt == kFmtBF16)) return false;
  const int pp = sp.p * sp.p, ppr = (pp + 7) & ~7;
  const int K1 = ((2 * ppr + 15) / 16) * 16;
  const int mm = sp.m * sp.m;
  const int N2 = ((mm + 15) / 16) * 16;
  if (N2 > 256 || pp > 256) return false;
  GemmGeom t = *g;
  t.fmt = fmt;
  t.passes = passes;
  t.K1 = K1;
  t.N2 = N2;
  // the first staging that fits, with the fewest GEMM1 output chunks (each
  // chunk costs the epilogue a TMEM read, a fence and barrier round trips)
  const int cc = sp.c * sp.c;
  for (int cw : chunk_widths(cc, N2)) {
    const std::vector<GemmGeom> st = stagings_of_width(t, cw, cc, passes);
    if (!st.empty()) {
      *g = st[0];
      return true;
    }
  }
  return false;
}

std::vector<GemmGeom> gemm_geometry_candidates(const GemmSpec& sp, int fmt, int passes) {
  std::vector<GemmGeom> out;
  GemmGeom g0{};
  if (!gemm_geometry(sp, fmt, passes, &g0)) return out;
  out.push_back(g0);  // the default first
  const int cc = sp.c * sp.c;
  for (int cw : chunk_widths(cc, g0.N2))
    for (const GemmGeom& t : stagings_of_width(g0, cw, cc, passes)) {
      if (t.CW == g0.CW && t.KCB == g0.KCB && t.dbE == g0.dbE && t.dbA2 == g0.dbA2 && t.NK == g0.NK &&
          t.NW == g0.NW)
        continue;
      out.push_back(t);
    }
  return out;
}

int gemm_smem_bytes(const GemmGeom& g) { return (int)gemm_smem_layout(g).total; }

void gemm_build_w2(const GemmSpec& sp, const GemmGeom& g, std::vector<uint8_t>& out) {
  const int p = sp.p, pp = p * p, ppr = (pp + 7) & ~7, c = sp.c, N = sp.N;
  const int esz = g.fmt == kFmtTF32 ? 4 : 2;
  const bool split = g.passes == 3;
  const GemmSmem L = gemm_smem_layout(g);
  out.assign((size_t)g.noc * g.nkc * L.wStage, 0);
  const uint32_t sbo = (uint32_t)(g.KCB / 16) * 128;
  const int kce = g.KCB / esz;  // elements per chunk row
  for (int oc = 0; oc < g.noc; oc++)
    for (int ol = 0; ol < g.CW; ol++) {
      const int o = oc * g.CW + ol;
      if (o >= c * c) continue;
      const int ku = sp.ro + o / c, kv = sp.ro + o % c;
      for (int k = 0; k < 2 * ppr; k++) {
        const bool re = k < ppr;
        const int pix = re ? k : k - ppr;
        if (pix >= pp) continue;
        const int i = pix / p, j = pix % p;
        const long long e = ((long long)ku * i + (long long)kv * j) % N;
        const double th = -2.0 * M_PI * (double)e / N;
        const double cr = cos(th), si = sin(th);
        // row 2ol: Re F = sum Re W Re E - Im W Im E ; row 2ol+1: Im F = Im W Re E + Re W Im E
        const double vre = re ? cr : -si;
        const double vim = re ? si : cr;
        const int kc = k / kce, kk = k % kce;
        uint8_t* hi = out.data() + ((size_t)oc * g.nkc + kc) * L.wStage;
        uint8_t* lo = hi + L.wHalf;
        put_val(g.fmt, split, hi, lo, kmaj(2 * ol, kk, esz, sbo), vre);
        put_val(g.fmt, split, hi, lo, kmaj(2 * ol + 1, kk, esz, sbo), vim);
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
  const int esz = g.fmt == kFmtTF32 ? 4 : 2;
  const bool split = g.passes == 3;
  const GemmSmem L = gemm_smem_layout(g);
  const uint32_t sbo = (uint32_t)(g.CW * esz / 16) * 128;
  out.assign((size_t)g.noc * L.kStage, 0);
  for (int oc = 0; oc < g.noc; oc++) {
    uint8_t* hi = out.data() + (size_t)oc * L.kStage;
    uint8_t* lo = hi + L.kHalf;
    for (int q = 0; q < mm; q++)
      for (int ol = 0; ol < g.CW; ol++) {
        const int o = oc * g.CW + ol;
        if (o >= cc) continue;
        put_val(g.fmt, split, hi, lo, kmaj(q, ol, esz, sbo), kc[(size_t)q * cc + o]);
      }
  }
}

cudaError_t launch_gemm(const WfsArgs& a, const GemmGeom& g, const float* iscale, int numSMs, int* err,
                        cudaStream_t stream) {
  if (g.NW < 2 || g.NW > kGemmMaxNW || g.NK < 1 || g.NK > kGemmMaxNK) return cudaErrorInvalidValue;
  if (g.fmt == kFmtBF16) {
    return g.passes == 3 ? launch_one<kFmtBF16, 3>(a, g, nullptr, numSMs, err, stream)
                         : launch_one<kFmtBF16, 1>(a, g, nullptr, numSMs, err, stream);
  }
  if (g.fmt == kFmtFP16) return launch_one<kFmtFP16, 1>(a, g, iscale, numSMs, err, stream);
  if (g.fmt == kFmtTF32) return launch_one<kFmtTF32, 1>(a, g, nullptr, numSMs, err, stream);
  return cudaErrorInvalidValue;
}

}  // namespace shwfs
