// Host/device interface of the GEMM-DFT form (wfs_gemm.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "shwfs_dev.cuh"

namespace shwfs {

// geometry of one handle, as the GEMM form needs it
struct GemmSpec {
  int p, N, c, ro, rs, padded, P, C, m, preBin, psfDim;
  std::vector<float> psf;                // 2-D PSF (P x P) when psfDim == 2
  std::vector<float> binT, binN;         // prepareBinImage weights (C)
  std::vector<int> binIdx;               // prepareBinImage indx (C)
};

// launch geometry and device constants
struct GemmGeom {
  int K1;    // 2 p^2 rounded up to 16 (GEMM1 K)
  int KC;    // GEMM1 K columns per streamed chunk (multiple of 16)
  int nkc;   // GEMM1 K chunks
  int noc;   // output chunks of 64 complex outputs (GEMM1 N = 128 columns each)
  int N2;    // GEMM2 N: nimg^2 rounded up to 16
  const uint8_t* w2;   // [noc][nkc] x {hi, lo} x [128 x KC] bf16, tensor-core smem order
  const uint8_t* kc2;  // [noc] x {hi, lo} x [N2 x 64] bf16, tensor-core smem order
};

// fills K1/KC/nkc/noc/N2; false if the geometry does not fit the kernel
bool gemm_geometry(const GemmSpec& sp, GemmGeom* g);
int gemm_smem_bytes(const GemmGeom& g, int m);
void gemm_build_w2(const GemmSpec& sp, const GemmGeom& g, std::vector<uint8_t>& out);
// dense [m^2][c^2] map from the cropped power spectrum to the binned image
void gemm_kc_matrix(const GemmSpec& sp, std::vector<double>& kc);
void gemm_build_kc(const GemmSpec& sp, const GemmGeom& g, const std::vector<double>& kc, std::vector<uint8_t>& out);
cudaError_t launch_gemm(const WfsArgs& a, const GemmGeom& g, int passes, int numSMs, int* err, cudaStream_t stream);

}  // namespace shwfs
