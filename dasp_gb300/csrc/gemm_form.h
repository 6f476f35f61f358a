// Host/device interface of the GEMM-DFT form (wfs_gemm.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "shwfs_dev.cuh"

namespace shwfs {

// operand formats of the tensor-core passes
enum : int { kFmtBF16 = 0, kFmtFP16 = 1, kFmtTF32 = 2 };
constexpr int kGemmMaxNW = 8;  // W2 ring stages
constexpr int kGemmMaxNK = 2;  // Kc ring stages

// geometry of one handle, as the GEMM form needs it
struct GemmSpec {
  int p, N, c, ro, rs, padded, P, C, m, preBin, psfDim;
  std::vector<float> psf;                // 2-D PSF (P x P) when psfDim == 2
  std::vector<float> binT, binN;         // prepareBinImage weights (C)
  std::vector<int> binIdx;               // prepareBinImage indx (C)
};

// launch geometry and device constants
struct GemmGeom {
  int fmt;     // kFmt*
  int passes;  // 1, or 3 split-product passes (bf16 only)
  int K1;      // GEMM1 K in elements: [Re E | Im E], each p^2 rounded up to 8, total rounded up to 16
  int KCB;     // GEMM1 K bytes per row of one streamed W2 chunk (multiple of 32)
  int nkc;     // W2 chunks per output chunk
  int CW;      // complex outputs per GEMM1 output chunk (GEMM1 N = 2 CW columns; 64, or a wider
               // multiple of 16 that needs fewer chunks for the c x c crop)
  int noc;     // output chunks of CW complex outputs
  int N2;      // GEMM2 N: nimg^2 rounded up to 16
  int NW, NK;  // ring stages for W2 and Kc chunks
  int dbE;     // 1: two field (GEMM1 A operand) buffers, the next tile's built during this one
  int dbA2;    // 1: two |F|^2 (GEMM2 A operand) buffers, alternating between output chunks
  int nd1;     // D1 (GEMM1 accumulator) buffers in TMEM: 3 when N2 <= 128 and CW == 64, else 2
  const uint8_t* w2;   // [noc][nkc] x {hi[, lo]} x [128 x KCB bytes], tensor-core smem order
  const uint8_t* kc2;  // [noc] x {hi[, lo]} x [N2 x 64 elements], tensor-core smem order
  const float* pupT;   // pupil by pixel group: [ppr/8][nlit][8], lit order
};

// TMEM columns of D1 buffer b and of D2: three 128-column D1 buffers around
// D2 at 256 when nd1 == 3 (CW 64, N2 <= 128), else D1 at 0 and 2 CW and D2
// after them (4 CW + N2 <= 512)
__host__ __device__ inline uint32_t gemm_d1_col(const GemmGeom& g, int b) {
  return (g.nd1 == 3 && b == 2) ? 384u : (uint32_t)(b * 2 * g.CW);
}
__host__ __device__ inline uint32_t gemm_d2_col(const GemmGeom& g) { return g.nd1 == 3 ? 256u : (uint32_t)(4 * g.CW); }

// dynamic shared-memory layout (byte offsets)
struct GemmSmem {
  uint32_t a1, a2, w, k, total;
  uint32_t a1Half, a2Half, wHalf, wStage, kHalf, kStage;
};

__host__ __device__ inline GemmSmem gemm_smem_layout(const GemmGeom& g) {
  GemmSmem L;
  const uint32_t esz = g.fmt == kFmtTF32 ? 4u : 2u, hl = g.passes == 3 ? 2u : 1u;
  L.a1Half = 128u * (uint32_t)g.K1 * esz;
  L.a2Half = 128u * (uint32_t)g.CW * esz;
  L.wHalf = 2u * (uint32_t)g.CW * (uint32_t)g.KCB;
  L.wStage = L.wHalf * hl;
  L.kHalf = (uint32_t)g.N2 * (uint32_t)g.CW * esz;
  L.kStage = L.kHalf * hl;
  L.a1 = 0;
  L.a2 = (L.a1 + L.a1Half * hl * (g.dbE ? 2u : 1u) + 1023u) & ~1023u;
  L.w = (L.a2 + L.a2Half * hl * (g.dbA2 ? 2u : 1u) + 1023u) & ~1023u;
  L.k = (L.w + (uint32_t)g.NW * L.wStage + 1023u) & ~1023u;
  L.total = L.k + (uint32_t)g.NK * L.kStage;
  return L;
}

// fills the geometry for one operand format; false if it does not fit the kernel
bool gemm_geometry(const GemmSpec& sp, int fmt, int passes, GemmGeom* g);
// every staging that fits the kernel for this spec and format (W2 chunk
// width, field / GEMM2-operand double buffering, Kc stages; the W2 ring as
// deep as shared memory allows), gemm_geometry's choice first; empty if none
std::vector<GemmGeom> gemm_geometry_candidates(const GemmSpec& sp, int fmt, int passes);
int gemm_smem_bytes(const GemmGeom& g);
void gemm_build_w2(const GemmSpec& sp, const GemmGeom& g, std::vector<uint8_t>& out);
// dense [m^2][c^2] map from the cropped power spectrum to the binned image
void gemm_kc_matrix(const GemmSpec& sp, std::vector<double>& kc);
void gemm_build_kc(const GemmSpec& sp, const GemmGeom& g, const std::vector<double>& kc, std::vector<uint8_t>& out);
// image formation of the lit subaperture-frames into bimg (pre-noise);
// iscale: per-subaperture |F|^2 scale of the fp16 format (else null)
cudaError_t launch_gemm(const WfsArgs& a, const GemmGeom& g, const float* iscale, int numSMs, int* err,
                        cudaStream_t stream);
// noise, threshold and the post stages on the pre-noise images in bimg
// (wfs_post.cu)
// done (optional) receives kPostDidUnlit when the launched kernel also
// zeroed the centroids of the unlit subapertures, and kPostDidOut when it
// also wrote the final images to a.bimgOut
constexpr unsigned kPostDidUnlit = 1u, kPostDidOut = 2u;
cudaError_t launch_post(const WfsArgs& a, int numSMs, cudaStream_t stream, unsigned* done = nullptr);

}  // namespace shwfs
