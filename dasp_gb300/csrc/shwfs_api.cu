// Host side of the C ABI declared in include/shwfs.h.
//
// A handle holds what the reference's centstruct holds (cmod/src/
// centmodule.c:139-249): scalar parameters, the integration state, the
// borrowed phase/cents/bimg arrays, and device-resident copies of every
// constant (pupil, flags, area fractions, normalisation totals, PSF spectra,
// binning tables, weights, calibration data, reference centroids).  A run
// queues: [H2D phase] -> fused kernel (+ unlit kernel) -> [D2H outputs].
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/shwfs.h"
#include "engine_internal.h"
#include "gemm_form.h"
#include "refnoise.h"
#include "wfs_launch.cuh"

using namespace shwfs;

namespace {

thread_local std::string g_err;

shwfs_status fail(shwfs_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return st;
}

#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fail(SHWFS_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    reset();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  cudaError_t upload(const T* src, size_t count) {
    cudaError_t e = alloc(count);
    if (e != cudaSuccess || count == 0) return e;
    return cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyDefault);
  }
};

int64_t numel(const shwfs_array& a) {
  if (!a.data) return 0;
  int64_t n = 1;
  for (int i = 0; i < a.ndim; i++) n *= a.shape[i];
  return n;
}

bool is_none(const shwfs_array& a) { return a.data == nullptr; }

// copy an array (host or device) to host memory
template <typename T>
std::vector<T> to_host(const shwfs_array& a) {
  std::vector<T> v((size_t)numel(a));
  if (!v.empty()) cudaMemcpy(v.data(), a.data, v.size() * sizeof(T), cudaMemcpyDefault);
  return v;
}

}  // namespace

// a fused-kernel launch of one handle held back for a multi-handle launch
struct DeferredPlain {
  struct shwfs_handle* h;
  shwfs::WfsArgs a;
  long long ntiles;
};

struct shwfs_handle {
  // parameters (names as in centstruct)
  int nthreads = 1, nsubaps = 0, nsubx = 0, ncen = 0, fftsize = 0, clipsize = 0, nimg = 0, phasesize = 0;
  float readNoise = 0, readBg = 0, noiseFloor = 0;
  int addPoisson = 0;
  float sig = 0;
  bool sigIsArr = false;
  float sky = 0;
  bool skyIsArr = false;
  int calsource = 0;
  float pxlPower = 1;
  int nintegrations = 1, nlatency = 0, curInteg = 0;
  uint64_t seed = 0;
  int opticalBinning = 0, correlationCentroiding = 0, threshType = 0, imageOnly = 0;
  int useBrightest = 0;
  bool ubIsArr = false;
  int preBinOrig = 1, preBin = 1, parabolicFit = 0, gaussianFit = 0;
  float gMin = 0, gRep = 0, corrThresh = 0;
  int psfDim = 0, psfsize = 0, padded = 0, phaseAmp = 0, W = 0;
  int centWeightDim = 0;
  int cwSize = 0;  // image size the centroid weights are for
  int noiseMode = SHWFS_NOISE_COUNTER;
  uint64_t framesRead = 0;
  bool haveCalData = false, haveCalCoeff = false, haveRef = false;
  int calNSteps = 0, calNCoeff = 0;
  int fitMxParam = 0;

  std::vector<int> subflag, lit, unlit;
  std::vector<float> pup, frac, psfSums;  // host copies for totsig
  std::vector<int> subapStart;

  // borrowed I/O
  shwfs_array phs{}, cents{}, bimg{};
  shwfs_array inputImage{};           // borrowed detector image (runSlope)
  int imageDims = 0, imageRows = 0, imageCols = 0;
  std::vector<int> subapLoc;
  float* bimgMapped = nullptr;        // device alias of a pinned host bimg
  float* centsMapped = nullptr;       // ... of a pinned host cents
  const float* phsMapped = nullptr;   // ... of a pinned host phase
  const float* imageMapped = nullptr; // ... of a pinned host detector image (runSlope)
  int hostIO = SHWFS_HOSTIO_OUTPUTS | SHWFS_HOSTIO_PHASE;  // zero-copy switches
  bool centsDirect = false, bimgDirect = false;  // this readout's kernels wrote the host outputs
  bool inDirect = false;                         // ... read the host input
  std::vector<float> bimgStage;       // fallback: full copy, then host scatter
  bool scatterPending = false;
  std::vector<void*> registered;  // host ranges pinned by the engine
  // host arrays bound before: (data, bytes) -> device alias or null.  Their
  // pinning lasts until the handle is freed, so rebinding one of them (a
  // few buffers in turn, every frame) needs no driver query.
  struct BoundHost {
    const void* data;
    size_t bytes;
    float* alias;
  };
  std::vector<BoundHost> boundHost;

  // device state
  int device = 0;
  cudaStream_t stream = nullptr;
  DevBuf<float> d_pup, d_tilt, d_frac, d_totsig, d_sigArr, d_skyArr, d_cw, d_ref, d_calData, d_calSteps,
      d_calCoeff, d_fitMx, d_binT, d_binN, d_psf;
  DevBuf<int> d_lit, d_unlit, d_binII, d_binLo, d_binHi, d_ubArr, d_calBounds, d_subflag, d_subapStart, d_status;
  DevBuf<float2> d_psfSpec;
  DevBuf<float> d_phs, d_cents, d_bimg, d_image;  // mirrors of host I/O
  DevBuf<int> d_subapLoc;
  DevBuf<unsigned char> d_poisFlag;
  DevBuf<RefRng> d_rng;
  DevBuf<float> d_inj;  // caller-drawn noise of shwfs_run_prenoise (shot, then read)
  // physical integration (SHWFS_INTEG_PHYSICAL): this sub-exposure's
  // pre-noise images and the exposure's running sum (nsubaps*nimg^2 each)
  int integMode = SHWFS_INTEG_COMPAT;
  int accumCount = 0;
  DevBuf<float> d_sub, d_accum;
  const PlainEntry* entry = nullptr;
  int TS = 1, smem = 0, ctasPerSM = 1, numSMs = 1;
  int tileOverride = 0;  // SHWFS_TILESUBAPS; 0 = default
  // GEMM-DFT form
  int form = SHWFS_FORM_FP32;
  bool gemmBuilt = false;
  GemmGeom gemm{};
  int gemmStaging = 0;     // SHWFS_GEMMSTAGING: index into gemm_geometry_candidates
  int gemmCandidates = 0;  // their number for the built geometry
  DevBuf<uint8_t> d_w2, d_kc2;
  DevBuf<float> d_iscale;  // fp16 form: 1 / (sum of the subaperture's pupil)^2
  DevBuf<float> d_pupT;    // tensor-core forms: pupil by pixel group [ppr/8][nlit][8]
  cudaEvent_t splitEvent = nullptr;  // recorded between image formation and post stages
  // while a multi-sensor batch captures: where the fused FP32 kernel's
  // launch goes instead of the stream (the batch launches the kernels of
  // several handles of one instantiation as one multi-handle kernel)
  std::vector<struct DeferredPlain>* plainSink = nullptr;
  const PoisTab* poisTab = nullptr;  // Poisson CDF tables on this device
  // correlation centroiding: pattern (host copy), its size, the per-mode
  // device kernel, and the corrimg output (borrowed; device mirror)
  std::vector<float> corrPatHost;
  int corrPatternSize = 0;
  int corrKMode = -1;  // mode the device kernel was built for
  DevBuf<float> d_corrK;
  shwfs_array corrimg{};
  // phase interpolation (interpolatePhase): the phase array is inputPhaseSize
  // square instead of W x W; d_interp holds the resampled frames
  bool interp = false;
  int inputPhaseSize = 0;
  DevBuf<float> d_interp;
  shwfs_array interpOut{};  // OUTPUTPHASEARR: interpolated phase of the lit subapertures
  std::vector<float> interpStage;
  DevBuf<float> d_corrimg;
  std::vector<float> corrimgStage;
  std::vector<float> psfHost, binTHost, binNHost;
  std::vector<int> binIdxHost;
  // CUDA-graph batches: bumped whenever a launch captured from this handle
  // could change (update, rebinding, replanning)
  uint64_t version = 0;
  const unsigned long long* graphCtr = nullptr;  // set while a batch captures
  DevBuf<unsigned long long> d_frameCtr;

  int* h_status = nullptr;      // pinned host copy of d_status, read after a sync
  int* h_statusDev = nullptr;   // its device alias (written by the noise/centroid kernel)

  ~shwfs_handle() {
    for (void* p : registered) cudaHostUnregister(p);
    if (h_status) cudaFreeHost(h_status);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

shwfs_status check_f32(const shwfs_array& a, const char* name) {
  if (a.dtype != SHWFS_F32) return fail(SHWFS_ERR_INVALID, "%s must be float32 and contiguous", name);
  return SHWFS_OK;
}

float* pin_host(shwfs_handle* h, const void* data, size_t bytes);

// bind a borrowed array; host pages are pinned in place (once) so the
// per-frame copies are asynchronous DMA
shwfs_status bind_io(shwfs_handle* h, shwfs_array& slot, const shwfs_array& a, DevBuf<float>& mirror, size_t count,
                     bool copy_initial) {
  slot = a;
  if (a.on_device) {
    mirror.reset();
    return SHWFS_OK;
  }
  if (mirror.n != count) {
    cudaError_t e = mirror.alloc(count);
    if (e != cudaSuccess) return fail(SHWFS_ERR_NOMEM, "device mirror allocation failed: %s", cudaGetErrorString(e));
  }
  const size_t bytes = count * sizeof(float);
  float* alias = nullptr;
  bool known = false;
  for (const auto& b : h->boundHost)
    if (b.data == a.data && b.bytes == bytes) {
      alias = b.alias;
      known = true;
      break;
    }
  if (!known) alias = pin_host(h, a.data, bytes);
  if (&slot == &h->bimg) h->bimgMapped = alias;
  if (&slot == &h->cents) h->centsMapped = alias;
  if (&slot == &h->phs) h->phsMapped = alias;
  if (&slot == &h->inputImage) h->imageMapped = alias;
  // outputs start from the caller's contents: entries the engine does not
  // write (unlit subapertures, non-readout frames) come back unchanged
  if (copy_initial) CK(cudaMemcpy(mirror.p, a.data, count * sizeof(float), cudaMemcpyHostToDevice));
  return SHWFS_OK;
}

// pin a borrowed host range in place (once) so that per-frame copies are
// asynchronous DMA, and return its device alias for zero-copy I/O, or null
float* pin_host(shwfs_handle* h, const void* data, size_t bytes) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, data) == cudaSuccess && attr.type == cudaMemoryTypeUnregistered) {
    if (cudaHostRegister((void*)data, bytes, cudaHostRegisterDefault) == cudaSuccess)
      h->registered.push_back((void*)data);
  }
  cudaGetLastError();  // a refused registration only costs copy speed
  // device alias, only when the whole range is pinned and maps contiguously
  // (a registration refused because a neighbour already pinned some of its
  // pages leaves it partial)
  float* alias = nullptr;
  cudaPointerAttributes last;
  const char* lastByte = (const char*)data + bytes - 1;
  if (cudaPointerGetAttributes(&attr, data) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
      attr.devicePointer && cudaPointerGetAttributes(&last, lastByte) == cudaSuccess &&
      last.type == cudaMemoryTypeHost && last.devicePointer &&
      (const char*)last.devicePointer - (const char*)attr.devicePointer == (ptrdiff_t)(bytes - 1))
    alias = (float*)attr.devicePointer;
  cudaGetLastError();
  if (h->boundHost.size() < 64) h->boundHost.push_back({data, bytes, alias});
  return alias;
}

// updateTotSigArr (cmod/src/centmodule.c:2403-2427): float accumulation in
// the reference's order
shwfs_status update_totsig(shwfs_handle* h) {
  const int pp = h->phasesize * h->phasesize;
  std::vector<float> tot(h->nsubaps);
  for (int i = 0; i < h->nsubaps; i++) {
    float t = 0.f;
    for (int j = 0; j < pp; j++) t += h->pup[(size_t)i * pp + j];
    t *= (float)(h->fftsize * h->fftsize);
    if (h->psfDim) {
      float s = h->psfSums[h->psfDim == 2 ? 0 : i];
      t *= s * h->psfsize * h->psfsize;
    }
    tot[i] = t;
  }
  CK(h->d_totsig.upload(tot.data(), tot.size()));
  return SHWFS_OK;
}

// prepareBinImage (cmod/src/centmodule.c:565-608) plus the gather ranges of
// the fused kernel's binning stage
shwfs_status prepare_bin(shwfs_handle* h) {
  const int C = h->clipsize, m = h->nimg;
  std::vector<float> t(C), n(C);
  std::vector<int> idx(C), ii(C), lo(m, C), hi(m, -1);
  int cnt = 0;
  for (int i = 0; i < C; i++) {
    cnt += m;
    if (cnt >= C) {
      int excess = cnt - C;
      t[i] = (m - excess) / (float)m;
      n[i] = excess / (float)m;
      idx[i] = 1;
      cnt = excess;
    } else {
      t[i] = 1.f;
      n[i] = 0.f;
      idx[i] = 0;
    }
  }
  int acc = 0;
  for (int i = 0; i < C; i++) {
    ii[i] = acc;
    if (i < C - 1) acc += idx[i];
  }
  for (int i = 0; i < C; i++) {
    // row i feeds output ii[i] (this share) and, through the next-pixel
    // share of row i-1, output ii[i-1]+1
    if (ii[i] < m) {
      lo[ii[i]] = std::min(lo[ii[i]], i);
      hi[ii[i]] = std::max(hi[ii[i]], i);
    }
    if (i < C - 1 && n[i] != 0.f && ii[i] + 1 < m) {
      lo[ii[i] + 1] = std::min(lo[ii[i] + 1], i);
      hi[ii[i] + 1] = std::max(hi[ii[i] + 1], i);
    }
  }
  for (int I = 0; I < m; I++)
    if (hi[I] < lo[I]) {
      lo[I] = 0;
      hi[I] = -1;
    }
  h->binTHost = t;
  h->binNHost = n;
  h->binIdxHost = idx;
  CK(h->d_binT.upload(t.data(), C));
  CK(h->d_binN.upload(n.data(), C));
  CK(h->d_binII.upload(ii.data(), C));
  CK(h->d_binLo.upload(lo.data(), m));
  CK(h->d_binHi.upload(hi.data(), m));
  return SHWFS_OK;
}

// setSpotPsf + prepareSpotPsf (cmod/src/centmodule.c:2255-2375)
shwfs_status set_spot_psf(shwfs_handle* h, const shwfs_array& psf) {
  int dim = 0, P = h->clipsize, preBin = 1, padded = h->clipsize;
  if (!is_none(psf)) {
    if (psf.ndim == 2) {
      dim = 2;
      P = (int)psf.shape[0];
      if (psf.shape[1] != P) return fail(SHWFS_ERR_INVALID, "spotpsf must be square");
    } else if (psf.ndim == 4) {
      dim = 4;
      P = (int)psf.shape[2];
      if (psf.shape[0] * psf.shape[1] != h->nsubaps || psf.shape[3] != P)
        return fail(SHWFS_ERR_INVALID, "spotpsf 4d must be (nsubx,nsubx,P,P)");
    } else {
      return fail(SHWFS_ERR_INVALID, "spotpsf not 2d or 4d");
    }
    preBin = h->preBinOrig;
    padded = preBin <= 1 ? P : h->fftsize;
    if (preBin > 0 && padded % preBin != 0)
      return fail(SHWFS_ERR_INVALID, "paddedsize(%d) modulo preBinningFactor(%d) should be zero", padded, preBin);
    if (preBin > 1 && P > padded)
      return fail(SHWFS_ERR_INVALID, "spotpsf dimensions should be equal to or less than paddedsize (%d)", padded);
    if (P < h->clipsize) return fail(SHWFS_ERR_INVALID, "spotpsf dimensions should be at least clipsize");
    shwfs_status st = check_f32(psf, "spotpsf");
    if (st) return st;
  }
  if (preBin < 1) preBin = 1;
  const PlainEntry* entry = nullptr;
  auto& reg = plain_registry();
  auto it = reg.find({h->fftsize, dim ? P : 0});
  if (it == reg.end())
    return fail(SHWFS_ERR_UNSUPPORTED, "no compiled kernel for fftsize %d with psfsize %d", h->fftsize, dim ? P : 0);
  entry = &it->second;
  if (dim) {
    std::vector<float> hp = to_host<float>(psf);
    h->psfHost.assign(hp.begin(), hp.begin() + (dim == 2 ? (size_t)P * P : 0));
    const int npsf = dim == 2 ? 1 : h->nsubaps;
    h->psfSums.assign(npsf, 0.f);
    for (int k = 0; k < npsf; k++) {
      float s = 0.f;
      for (int j = 0; j < P * P; j++) s += hp[(size_t)k * P * P + j];
      h->psfSums[k] = s;
    }
    CK(h->d_psf.upload(hp.data(), hp.size()));
    CK(h->d_psfSpec.alloc((size_t)npsf * P * (P / 2 + 1)));
    CK(entry->psf_spectra(h->d_psf.p, npsf, h->d_psfSpec.p, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->d_psf.reset();
  } else {
    h->d_psfSpec.reset();
    h->psfSums.clear();
  }
  h->psfDim = dim;
  h->psfsize = P;
  h->preBin = preBin;
  h->padded = padded;
  h->entry = entry;
  return SHWFS_OK;
}

// launch geometry: tile size, shared memory, persistent grid
shwfs_status plan(shwfs_handle* h) {
  const int P = h->psfDim ? h->psfsize : 0;
  const int per = persub_floats(h->phasesize, h->fftsize, P, h->padded, h->clipsize, h->nimg);
  const int cst = const_floats(h->phasesize, h->clipsize, h->nimg, P, h->centWeightDim == 2, h->psfDim == 2);
  int TS = std::max(1, std::min(64, (kThreads + h->phasesize - 1) / h->phasesize));
  if (h->tileOverride > 0) TS = std::min(64, h->tileOverride);
  while (TS > 1 && (size_t)(cst + TS * per) * 4 > 100 * 1024) TS--;
  const int smem = (cst + TS * per) * 4;
  if (smem > 227 * 1024) return fail(SHWFS_ERR_UNSUPPORTED, "subaperture too large for shared memory (%d bytes)", smem);
  int ctas = 0;
  CK(h->entry->occupancy(&ctas, smem));
  if (ctas < 1) return fail(SHWFS_ERR_UNSUPPORTED, "kernel cannot be resident with %d bytes of shared memory", smem);
  h->TS = TS;
  h->smem = smem;
  h->ctasPerSM = ctas;
  return SHWFS_OK;
}

// corrsize: the pattern's size while correlating with a pattern, else nimg
// (cmod/src/centmodule.c:2717-2721, 3006)
int corr_size(const shwfs_handle* h) {
  return (h->correlationCentroiding && !h->corrPatHost.empty()) ? h->corrPatternSize : h->nimg;
}

// correlation images are computed (patterns set, centroids wanted)
bool corr_active(const shwfs_handle* h) {
  return h->correlationCentroiding != 0 && !h->corrPatHost.empty() && h->imageOnly == 0 && h->opticalBinning != 1;
}

// hc2r x hc2r (FFTW's unnormalised half-complex inverse along each axis) of
// an n x n half-complex array, in double
void hc2r_2d(const float* h, int n, std::vector<double>& out) {
  std::vector<double> cs(n * n), sn(n * n), t((size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int k = 0; k < n; k++) {
      const double a = 2.0 * M_PI * (double)((long long)j * k % n) / n;
      cs[j * n + k] = cos(a);
      sn[j * n + k] = sin(a);
    }
  auto line = [&](const double* in, double* o, int stride) {  // one 1-D inverse
    for (int j = 0; j < n; j++) {
      double y = in[0];
      for (int k = 1; k < (n + 1) / 2; k++) y += 2.0 * (in[k * stride] * cs[j * n + k] - in[(n - k) * stride] * sn[j * n + k]);
      if (n % 2 == 0) y += ((j & 1) ? -1.0 : 1.0) * in[(n / 2) * stride];
      o[j * stride] = y;
    }
  };
  std::vector<double> src((size_t)n * n);
  for (int i = 0; i < n * n; i++) src[i] = h[i];
  for (int r = 0; r < n; r++) line(&src[(size_t)r * n], &t[(size_t)r * n], 1);  // along rows
  out.assign((size_t)n * n, 0.0);
  for (int c = 0; c < n; c++) line(&t[c], &out[c], n);  // along columns
}

shwfs_status load_corr_pattern(shwfs_handle* h, const shwfs_array& cp) {
  h->corrKMode = -1;
  if (is_none(cp)) {
    h->corrPatHost.clear();
    h->d_corrK.reset();
    return SHWFS_OK;
  }
  if (check_f32(cp, "corrPattern") || cp.ndim != 4 || cp.shape[0] * cp.shape[1] != h->nsubaps ||
      cp.shape[2] != cp.shape[3] || cp.shape[2] < h->nimg)
    return fail(SHWFS_ERR_INVALID, "corrPattern wrong shape or type - should be (nsubx,nsubx,>=nimg,>=nimg), float32");
  if (cp.shape[2] > 64) return fail(SHWFS_ERR_UNSUPPORTED, "correlation patterns larger than 64 pixels");
  h->corrPatternSize = (int)cp.shape[2];
  h->corrPatHost = to_host<float>(cp);
  return SHWFS_OK;
}

shwfs_status set_corr_pattern(shwfs_handle* h, const shwfs_array& cp) {
  if (shwfs_status s = load_corr_pattern(h, cp)) return s;
  return plan(h);
}

// the device kernel for the current mode: hc2r of each pattern (mode 1) or
// the patterns themselves
shwfs_status prepare_corr(shwfs_handle* h) {
  if (!corr_active(h) || h->corrKMode == h->correlationCentroiding) return SHWFS_OK;
  const int n = h->corrPatternSize, cc = n * n;
  std::vector<float> K(h->corrPatHost.size());
  if (h->correlationCentroiding == 1) {
    std::vector<double> o;
    for (int i = 0; i < h->nsubaps; i++) {
      hc2r_2d(h->corrPatHost.data() + (size_t)i * cc, n, o);
      for (int k = 0; k < cc; k++) K[(size_t)i * cc + k] = (float)o[k];
    }
  } else {
    K = h->corrPatHost;
  }
  CK(h->d_corrK.upload(K.data(), K.size()));
  if (h->d_corrimg.n < (size_t)h->nsubaps * cc) CK(h->d_corrimg.alloc((size_t)h->nsubaps * cc));
  h->corrKMode = h->correlationCentroiding;
  return SHWFS_OK;
}

shwfs_status set_cent_weight(shwfs_handle* h, const shwfs_array& cw) {
  h->centWeightDim = 0;
  h->d_cw.reset();
  if (is_none(cw)) return SHWFS_OK;
  const int corr = corr_size(h);
  if (cw.ndim != 2 && cw.ndim != 4) return fail(SHWFS_ERR_INVALID, "centWeight not 2d or 4d");
  if (check_f32(cw, "centWeight")) return SHWFS_ERR_INVALID;
  if (cw.shape[cw.ndim - 2] != corr || cw.shape[cw.ndim - 1] != corr)
    return fail(SHWFS_ERR_INVALID, "centweight array not correct dimensions (need to be nsubx,nsubx,corrsize,corrsize)");
  if (cw.ndim == 4 && cw.shape[0] * cw.shape[1] != h->nsubaps)
    return fail(SHWFS_ERR_INVALID, "centWeight 4d must be (nsubx,nsubx,corrsize,corrsize)");
  std::vector<float> v = to_host<float>(cw);
  CK(h->d_cw.upload(v.data(), v.size()));
  h->centWeightDim = cw.ndim;
  h->cwSize = corr;
  return SHWFS_OK;
}

shwfs_status set_sig(shwfs_handle* h, double sig, const shwfs_array* arr) {
  if (arr && !is_none(*arr)) {
    if (check_f32(*arr, "sig array")) return SHWFS_ERR_INVALID;
    if (arr->ndim != 1 || arr->shape[0] != h->nsubaps)
      return fail(SHWFS_ERR_INVALID, "sig arr dimensions must be 1D (nsubx^2)");
    std::vector<float> v = to_host<float>(*arr);
    CK(h->d_sigArr.upload(v.data(), v.size()));
    h->sigIsArr = true;
  } else {
    h->sig = (float)sig;
    // a scalar update keeps a previously set array, as py_update does
  }
  return SHWFS_OK;
}

shwfs_status set_sky(shwfs_handle* h, double sky, const shwfs_array* arr) {
  if (arr && !is_none(*arr)) {
    if (check_f32(*arr, "skybrightness")) return SHWFS_ERR_INVALID;
    if (arr->ndim != 3 || arr->shape[0] != h->nsubaps || arr->shape[1] != h->nimg || arr->shape[2] != h->nimg)
      return fail(SHWFS_ERR_INVALID, "skybrightness should be 3D array shape nsubaps,nimg,nimg");
    std::vector<float> v = to_host<float>(*arr);
    CK(h->d_skyArr.upload(v.data(), v.size()));
    h->sky = 0.f;
    h->skyIsArr = true;
  } else {
    h->sky = (float)sky;
    h->skyIsArr = false;
    h->d_skyArr.reset();
  }
  return SHWFS_OK;
}

shwfs_status set_use_brightest(shwfs_handle* h, int ub, const shwfs_array* arr) {
  if (arr && !is_none(*arr)) {
    if (arr->dtype != SHWFS_I32) return fail(SHWFS_ERR_INVALID, "useBrightest must be int or int contiguous array");
    if (arr->ndim != 1 || arr->shape[0] != h->nsubaps)
      return fail(SHWFS_ERR_INVALID, "useBrightest array should be 1D of shape nsubaps (nsubx^2)");
    std::vector<int> v = to_host<int>(*arr);
    CK(h->d_ubArr.upload(v.data(), v.size()));
    h->useBrightest = 0;
    h->ubIsArr = true;
  } else {
    h->useBrightest = ub;
    h->ubIsArr = false;
    h->d_ubArr.reset();
  }
  return SHWFS_OK;
}

// setupThreads (cmod/src/centmodule.c:2457-2571): partition + RNG seeding
shwfs_status setup_threads(shwfs_handle* h, int nthreads) {
  if (nthreads < 1) return fail(SHWFS_ERR_INVALID, "nthreads must be >= 1");
  h->nthreads = nthreads;
  h->subapStart.assign(nthreads + 1, 0);
  int cnt = 0, left = h->nsubaps;
  for (int i = 0; i < nthreads; i++) {
    h->subapStart[i] = cnt;
    cnt += left / (nthreads - i);
    left -= left / (nthreads - i);
  }
  h->subapStart[nthreads] = h->nsubaps;
  std::vector<RefRng> rng(nthreads);
  const uint64_t base = h->seed == 0 ? (uint64_t)time(nullptr) : h->seed;
  for (int i = 0; i < nthreads; i++) seed_ref_rng(&rng[i], base + i);
  CK(h->d_rng.upload(rng.data(), rng.size()));
  CK(h->d_subapStart.upload(h->subapStart.data(), h->subapStart.size()));
  return SHWFS_OK;
}

// 6x6 normal-matrix inverse for the parabolic/Gaussian fit (makeFitMx,
// cmod/src/centmodule.c:997-1056), Gauss-Jordan with partial pivoting
shwfs_status make_fit_mx(shwfs_handle* h, int ncen) {
  double a[6][12];
  memset(a, 0, sizeof(a));
  for (int y = 0; y < ncen; y++)
    for (int x = 0; x < ncen; x++) {
      double v[6] = {(double)x * x, (double)x * y, (double)y * y, (double)x, (double)y, 1.0};
      for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++) a[r][c] += v[r] * v[c];
    }
  for (int r = 0; r < 6; r++) a[r][6 + r] = 1.0;
  for (int c = 0; c < 6; c++) {
    int piv = c;
    for (int r = c + 1; r < 6; r++)
      if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
    if (a[piv][c] == 0.0) return fail(SHWFS_ERR_INVALID, "singular fit matrix for fit size %d", ncen);
    if (piv != c)
      for (int k = 0; k < 12; k++) std::swap(a[c][k], a[piv][k]);
    double d = a[c][c];
    for (int k = 0; k < 12; k++) a[c][k] /= d;
    for (int r = 0; r < 6; r++)
      if (r != c) {
        double f = a[r][c];
        for (int k = 0; k < 12; k++) a[r][k] -= f * a[c][k];
      }
  }
  float mx[30];
  for (int r = 0; r < 5; r++)
    for (int c = 0; c < 6; c++) mx[r * 6 + c] = (float)a[r][6 + c];
  CK(h->d_fitMx.upload(mx, 30));
  h->fitMxParam = ncen;
  return SHWFS_OK;
}

WfsArgs make_args(shwfs_handle* h, const float* phs, float* cents, float* bimg, int nframes, long long phsStride,
                  int mode) {
  WfsArgs a;
  memset(&a, 0, sizeof(a));
  a.nsubx = h->nsubx;
  a.nsubaps = h->nsubaps;
  a.p = h->phasesize;
  a.N = h->fftsize;
  a.C = h->clipsize;
  a.m = h->nimg;
  a.ncen = h->ncen;
  a.P = h->psfsize;
  a.padded = h->padded;
  a.preBin = h->preBin;
  a.psfDim = h->psfDim;
  a.phaseAmp = h->phaseAmp;
  a.W = h->W;
  a.phsFrameStride = phsStride;
  a.phsAmpOffset = (long long)h->W * h->W;
  a.nlit = (int)h->lit.size();
  a.nframes = nframes;
  a.TS = h->TS;
  a.lit = h->d_lit.p;
  a.unlit = h->d_unlit.p;
  a.nunlit = (int)h->unlit.size();
  a.subflag = h->d_subflag.p;
  a.phs = phs;
  a.pup = h->d_pup.p;
  a.tilt = h->d_tilt.p;
  a.frac = h->d_frac.p;
  a.totsig = h->d_totsig.p;
  a.sig = h->sig;
  a.sigArr = h->sigIsArr ? h->d_sigArr.p : nullptr;
  a.sky = h->sky;
  a.skyArr = h->skyIsArr ? h->d_skyArr.p : nullptr;
  a.psfSpec = h->d_psfSpec.p;
  a.binT = h->d_binT.p;
  a.binN = h->d_binN.p;
  a.binII = h->d_binII.p;
  a.binLo = h->d_binLo.p;
  a.binHi = h->d_binHi.p;
  a.readNoise = h->readNoise;
  a.readBg = h->readBg;
  a.floorv = h->noiseFloor;
  a.threshType = h->threshType;
  a.addPoisson = h->addPoisson;
  a.calsource = h->calsource;
  a.opticalBinning = h->opticalBinning;
  a.imageOnly = h->imageOnly;
  a.useBrightest = h->useBrightest;
  a.useBrightestArr = h->ubIsArr ? h->d_ubArr.p : nullptr;
  a.pxlPower = h->pxlPower;
  a.centWeight = h->d_cw.p;
  a.centWeightDim = h->centWeightDim;
  a.cob = h->correlationCentroiding == 5 ? 1 : h->correlationCentroiding;
  a.fitSize = h->parabolicFit + h->gaussianFit;
  a.gaussianFit = h->gaussianFit;
  a.gMin = h->gMin;
  a.gRep = h->gRep;
  a.fitMx = h->d_fitMx.p;
  a.calData = h->haveCalData ? h->d_calData.p : nullptr;
  a.calBounds = h->d_calBounds.p;
  a.calSteps = h->d_calSteps.p;
  a.calNSteps = h->calNSteps;
  a.calCoeff = h->haveCalCoeff ? h->d_calCoeff.p : nullptr;
  a.calNCoeff = h->calNCoeff;
  a.refCents = h->haveRef ? h->d_ref.p : nullptr;
  a.bimg = bimg;
  a.bimgFrameStride = (long long)h->nsubaps * h->nimg * h->nimg;
  a.cents = cents;
  a.centsFrameStride = (long long)h->nsubaps * 2;
  a.poisFlag = h->d_poisFlag.p;
  a.seed = h->seed;
  set_philox_keys(a);
  a.frame0 = h->framesRead;
  a.frameCtr = h->graphCtr;
  a.poisTab = h->poisTab;
  a.skipCents = corr_active(h) ? 1 : 0;
  a.mode = mode;
  return a;
}

// operand format and split-product passes of a tensor-core form
int form_fmt(int form) {
  return form == SHWFS_FORM_FP16 ? kFmtFP16 : (form == SHWFS_FORM_TF32 ? kFmtTF32 : kFmtBF16);
}
int form_passes(int form) { return form == SHWFS_FORM_BF16X3 ? 3 : 1; }

// GEMM-DFT form: eligibility and device constants.  Configurations outside the
// GEMM kernel (per-subaperture PSFs, phase+amplitude, optical binning,
// reference-stream noise, phasesize > 16, nimg > 16, no staging that fits
// shared memory) run the FP32 form.
bool gemm_static_ok(const shwfs_handle* h, GemmGeom* g, GemmSpec* sp) {
  if (h->psfDim == 4 || h->phaseAmp) return false;
  sp->p = h->phasesize;
  sp->N = h->fftsize;
  sp->padded = h->padded;
  sp->rs = h->padded > h->fftsize ? (h->padded - h->fftsize) / 2 : 0;
  sp->ro = h->padded > h->fftsize ? 0 : (h->fftsize - h->padded) / 2;
  sp->c = h->padded > h->fftsize ? h->fftsize : h->padded;
  sp->P = h->psfsize;
  sp->C = h->clipsize;
  sp->m = h->nimg;
  sp->preBin = h->preBin;
  sp->psfDim = h->psfDim;
  sp->psf = h->psfHost;
  sp->binT = h->binTHost;
  sp->binN = h->binNHost;
  sp->binIdx = h->binIdxHost;
  return gemm_geometry(*sp, form_fmt(h->form), form_passes(h->form), g);
}

bool gemm_active(const shwfs_handle* h) {
  return h->form != SHWFS_FORM_FP32 && h->gemmBuilt && h->opticalBinning != 1 &&
         h->noiseMode == SHWFS_NOISE_COUNTER;
}

// the W2 and Kc constants of geometry g, in its tensor-core staging order
shwfs_status upload_gemm_consts(shwfs_handle* h, const GemmSpec& sp, const GemmGeom& g) {
  std::vector<uint8_t> w2, kc2;
  std::vector<double> kc;
  gemm_build_w2(sp, g, w2);
  gemm_kc_matrix(sp, kc);
  gemm_build_kc(sp, g, kc, kc2);
  CK(h->d_w2.upload(w2.data(), w2.size()));
  CK(h->d_kc2.upload(kc2.data(), kc2.size()));
  return SHWFS_OK;
}

shwfs_status build_gemm(shwfs_handle* h) {
  h->gemmBuilt = false;
  h->gemmCandidates = 0;
  if (h->form == SHWFS_FORM_FP32) return SHWFS_OK;
  GemmSpec sp;
  GemmGeom g{};
  if (!gemm_static_ok(h, &g, &sp)) return SHWFS_OK;  // falls back to the FP32 form
  {
    // the staging chosen by SHWFS_GEMMSTAGING (or the autotuner)
    const std::vector<GemmGeom> cands = gemm_geometry_candidates(sp, g.fmt, g.passes);
    h->gemmCandidates = (int)cands.size();
    if (h->gemmStaging < 0 || h->gemmStaging >= (int)cands.size()) h->gemmStaging = 0;
    if (!cands.empty()) g = cands[h->gemmStaging];
  }
  if (shwfs_status s = upload_gemm_consts(h, sp, g)) return s;
  if (g.fmt == kFmtFP16) {
    const int pp = h->phasesize * h->phasesize;
    std::vector<float> isc((size_t)h->nsubaps, 1.f);
    for (int i = 0; i < h->nsubaps; i++) {
      double s = 0;
      for (int k = 0; k < pp; k++) s += h->pup[(size_t)i * pp + k];
      if (s > 0) isc[i] = (float)(1.0 / (s * s));
    }
    CK(h->d_iscale.upload(isc.data(), isc.size()));
  }
  {
    // pupil of the lit subapertures grouped by 8 pixels, so that the field
    // warps' loads (one lit subaperture per lane) are contiguous
    const int pp = h->phasesize * h->phasesize, ng8 = ((pp + 7) & ~7) / 8;
    const size_t nl = h->lit.size();
    std::vector<float> pt((size_t)ng8 * nl * 8, 0.f);
    for (int gi = 0; gi < ng8; gi++)
      for (size_t li = 0; li < nl; li++)
        for (int e = 0; e < 8; e++) {
          const int k = gi * 8 + e;
          if (k < pp) pt[((size_t)gi * nl + li) * 8 + e] = h->pup[(size_t)h->lit[li] * pp + k];
        }
    if (!pt.empty()) CK(h->d_pupT.upload(pt.data(), pt.size()));
  }
  h->gemm = g;
  h->gemmBuilt = true;
  return SHWFS_OK;
}

// device buffer the correlation images of a frame go to
float* corrimg_dev(shwfs_handle* h) {
  if (!is_none(h->corrimg) && h->corrimg.on_device) return (float*)h->corrimg.data;
  return h->d_corrimg.p;
}

// correlation images and centroids from the final images in bimg
shwfs_status enqueue_corr(shwfs_handle* h, float* cents, float* bimg, int nframes, cudaStream_t st) {
  if (!corr_active(h) || h->lit.empty()) return SHWFS_OK;
  const int cs = h->corrPatternSize;
  if (!is_none(h->corrimg) && numel(h->corrimg) < (int64_t)h->nsubaps * cs * cs)
    return fail(SHWFS_ERR_INVALID, "corrimg must hold nsubx*nsubx*corrsize*corrsize values");
  WfsArgs a = make_args(h, nullptr, cents, bimg, nframes, 0, kPost);
  a.centWeight = h->d_cw.p;
  CorrArgs c{};
  c.mode = h->correlationCentroiding;
  c.cs = cs;
  c.thresh = h->corrThresh;
  c.K = h->d_corrK.p;
  c.corrimg = corrimg_dev(h);
  c.corrimgFrameStride = 0;  // one frame at a time
  CK(launch_corr(a, c, h->numSMs, st));
  return SHWFS_OK;
}

// queue one readout over nframes frames (device pointers)
// device-side state a readout needs that is built lazily (the fit matrix);
// run before a graph capture so that nothing allocates while capturing
shwfs_status prepare_readout(shwfs_handle* h) {
  if (shwfs_status s = prepare_corr(h)) return s;
  if (h->fitMxParam != h->parabolicFit + h->gaussianFit && (h->parabolicFit || h->gaussianFit > 0)) {
    int fs = h->parabolicFit + h->gaussianFit;
    shwfs_status s = make_fit_mx(h, fs < 0 ? 3 : (fs < 3 ? 3 : fs));
    if (s) return s;
    h->fitMxParam = h->parabolicFit + h->gaussianFit;
  }
  return SHWFS_OK;
}

// bimgHost (optional): a second destination of the final images (the
// device alias of the caller's pinned host array); *bimgHostDone tells
// whether the launched kernels filled it (lit subapertures, and the unlit
// ones with imageOnly)
shwfs_status enqueue_readout(shwfs_handle* h, const float* phs, float* cents, float* bimg, int nframes,
                             long long phsStride, cudaStream_t st, float* bimgHost = nullptr,
                             bool* bimgHostDone = nullptr) {
  if (bimgHostDone) *bimgHostDone = false;
  if (h->noiseMode == SHWFS_NOISE_REFERENCE || corr_active(h)) bimgHost = nullptr;
  if (h->interp && phs) {
    // resample the input frames to W x W first (interpolatePhase,
    // cmod/src/centmodule.c:1795-1804); the pipeline then reads d_interp
    const long long WW = (long long)h->W * h->W, in2 = (long long)h->inputPhaseSize * h->inputPhaseSize;
    if ((size_t)(WW * nframes) > h->d_interp.n)
      return fail(SHWFS_ERR_STATE, "interpolation buffer holds %zu frames, %d requested", h->d_interp.n / (size_t)WW,
                  nframes);
    CK(launch_interp_phase(phs, phsStride ? phsStride : in2, h->inputPhaseSize, h->d_interp.p, WW, h->W, nframes, st));
    if (nframes == 1 && !is_none(h->interpOut) && h->interpOut.on_device)
      CK(launch_copy_lit_blocks(h->d_interp.p, (float*)h->interpOut.data, h->d_lit.p, (int)h->lit.size(), h->nsubx,
                                h->phasesize, st));
    phs = h->d_interp.p;
    phsStride = WW;
  }
  const int nlit = (int)h->lit.size();
  const long long nwork = (long long)nlit * nframes;
  const long long ntiles = (nwork + h->TS - 1) / h->TS;
  const int grid = (int)std::max<long long>(1, std::min<long long>(ntiles, (long long)h->numSMs * h->ctasPerSM));
  if (shwfs_status s = prepare_readout(h)) return s;
  if (corr_active(h) && nframes != 1)
    return fail(SHWFS_ERR_UNSUPPORTED, "correlation centroiding runs one frame at a time");
  if (h->noiseMode == SHWFS_NOISE_REFERENCE) {
    if (nframes != 1) return fail(SHWFS_ERR_UNSUPPORTED, "reference-stream noise runs one frame at a time");
    if (nlit) {
      WfsArgs a = make_args(h, phs, cents, bimg, 1, phsStride, kForm | kStorePreNoise);
      CK(h->entry->launch(a, grid, h->smem, st));
    }
    RefNoiseArgs r{};
    r.nthreads = h->nthreads;
    r.subapStart = h->d_subapStart.p;
    r.subflag = h->d_subflag.p;
    r.poisFlag = h->d_poisFlag.p;
    r.bimg = bimg;
    r.m = h->nimg;
    r.nexp = h->opticalBinning == 1 ? 2 * h->ncen : h->nimg * h->nimg;
    r.readNoise = h->readNoise;
    r.readBg = h->readBg;
    r.floorv = h->noiseFloor;
    r.threshType = h->threshType;
    r.addPoisson = h->addPoisson;
    r.calsource = h->calsource;
    r.imageOnly = h->imageOnly;
    CK(launch_refnoise(r, h->d_rng.p, h->d_status.p, st));
    if (nlit) {
      WfsArgs a = make_args(h, phs, cents, bimg, 1, phsStride, kPost);
      CK(h->entry->launch(a, grid, h->smem, st));
    }
    if (!h->unlit.empty() && !h->imageOnly) {
      WfsArgs a = make_args(h, phs, cents, bimg, 1, phsStride, 0);
      CK(launch_unlit(a, h->d_unlit.p, (int)h->unlit.size(), st));
    }
  } else {
    unsigned postDone = 0;
    bool plainDirect = false;
    if (nlit && gemm_active(h)) {
      // tensor-core image formation into bimg, then noise + post stages
      WfsArgs a = make_args(h, phs, cents, bimg, nframes, phsStride, kForm);
      GemmGeom g = h->gemm;
      g.w2 = h->d_w2.p;
      g.kc2 = h->d_kc2.p;
      g.pupT = h->d_pupT.p;
      CK(launch_gemm(a, g, g.fmt == kFmtFP16 ? h->d_iscale.p : nullptr, h->numSMs, h->d_status.p, st));
      if (h->splitEvent) CK(cudaEventRecord(h->splitEvent, st));
      a.mode = kNoiseCounter | kPost;
      a.bimgOut = bimgHost;
      a.statusIn = h->d_status.p;
      a.statusOut = h->h_statusDev;
      CK(launch_post(a, h->numSMs, st, &postDone));
    } else if (nlit) {
      // the fused kernel writes each final image once: straight to the
      // host array when there is one
      plainDirect = bimgHost != nullptr;
      if (plainDirect) bimg = bimgHost;
      WfsArgs a = make_args(h, phs, cents, bimg, nframes, phsStride, kForm | kNoiseCounter | kPost);
      if (h->plainSink && !plainDirect)
        h->plainSink->push_back(DeferredPlain{h, a, ntiles});
      else
        CK(h->entry->launch(a, grid, h->smem, st));
    }
    if (!h->unlit.empty() && !(postDone & kPostDidUnlit)) {
      WfsArgs a = make_args(h, phs, cents, bimg, nframes, phsStride, 0);
      CK(launch_unlit(a, h->d_unlit.p, (int)h->unlit.size(), st));
    }
    if (bimgHostDone && bimgHost) {
      if (plainDirect || !nlit)
        *bimgHostDone = plainDirect || h->unlit.empty() || !h->imageOnly;
      else
        *bimgHostDone = (postDone & kPostDidOut) && (h->unlit.empty() || !h->imageOnly);
    }
  }
  return enqueue_corr(h, cents, bimg, 1, st);
}

// the integration state machine of centroidsFromPhase (cmod/src/centmodule.c:
// 1774-1788) and py_run's advance (:3221-3223); returns 1 on a readout frame
int readout_frame(const shwfs_handle* h) {
  if (h->curInteg == 0) return 1 == h->nintegrations + h->nlatency ? 1 : 0;
  if (h->curInteg + 1 < h->nintegrations) return 0;
  if (h->curInteg + 1 < h->nintegrations + h->nlatency) return 0;
  return 1;
}

// caller-supplied pre-noise images (and optionally caller-drawn noise) of
// shwfs_run_prenoise
struct PrenoiseIn {
  const shwfs_array* images;
  const shwfs_array* shot;
  const shwfs_array* readn;
};

// the reference's state of this frame (cmod/src/centmodule.c:1774-1788):
// 0 start of an exposure, 1 middle, 2 readout, -1 start and readout,
// 3 frame transfer (no exposure)
int integ_state(const shwfs_handle* h) {
  if (h->curInteg == 0) return h->nintegrations + h->nlatency == 1 ? -1 : 0;
  if (h->curInteg + 1 < h->nintegrations) return 1;
  if (h->curInteg + 1 < h->nintegrations + h->nlatency) return 3;
  return 2;
}

shwfs_status enqueue_prenoise(shwfs_handle* h, const PrenoiseIn& in, cudaStream_t st);

// physical integration, one exposed frame (state 0, 1, 2 or -1) of device
// phase phs: this sub-exposure's normalised, sky-added images into d_sub,
// added to the exposure's sum; at the readout the sum becomes the mean and
// goes through noise, threshold and the post stages (as shwfs_run_prenoise)
shwfs_status enqueue_physical(shwfs_handle* h, const float* phs, int state, cudaStream_t st) {
  if (h->interp || h->phaseAmp || h->opticalBinning == 1)
    return fail(SHWFS_ERR_UNSUPPORTED,
                "physical integration with phase interpolation, phase+amplitude or optical binning");
  const size_t n = (size_t)h->nsubaps * h->nimg * h->nimg;
  for (DevBuf<float>* b : {&h->d_sub, &h->d_accum}) {
    if (b->n < n) {
      CK(b->alloc(n));
      CK(cudaMemsetAsync(b->p, 0, n * sizeof(float), st));  // unlit subapertures stay 0
    }
  }
  const int nlit = (int)h->lit.size();
  if (nlit) {
    if (gemm_active(h)) {
      WfsArgs a = make_args(h, phs, h->d_cents.p, h->d_sub.p, 1, 0, kForm);
      GemmGeom g = h->gemm;
      g.w2 = h->d_w2.p;
      g.kc2 = h->d_kc2.p;
      g.pupT = h->d_pupT.p;
      CK(launch_gemm(a, g, g.fmt == kFmtFP16 ? h->d_iscale.p : nullptr, h->numSMs, h->d_status.p, st));
    } else {
      const long long ntiles = ((long long)nlit + h->TS - 1) / h->TS;
      const int grid =
          (int)std::max<long long>(1, std::min<long long>(ntiles, (long long)h->numSMs * h->ctasPerSM));
      WfsArgs a = make_args(h, phs, h->d_cents.p, h->d_sub.p, 1, 0, kForm | kStorePreNoise);
      CK(h->entry->launch(a, grid, h->smem, st));
    }
  }
  const bool first = state == 0 || state == -1, ro = state == 2 || state == -1;
  h->accumCount = first ? 1 : h->accumCount + 1;
  CK(launch_accumulate(h->d_accum.p, h->d_sub.p, (long long)n, first ? 1 : 0, ro ? 1.0f / (float)h->accumCount : 1.0f,
                       st));
  if (!ro) return SHWFS_OK;
  shwfs_array acc{};
  acc.data = h->d_accum.p;
  acc.ndim = 1;
  acc.shape[0] = (int64_t)n;
  acc.dtype = SHWFS_F32;
  acc.on_device = 1;
  const shwfs_array none{};
  PrenoiseIn in{&acc, &none, &none};
  return enqueue_prenoise(h, in, st);
}

// publish exactly what the reference writes on a readout frame: every
// centroid unless imageOnly; every image with imageOnly, else the lit ones
shwfs_status publish_outputs(shwfs_handle* h, cudaStream_t st, bool* sync) {
  if (h->interp && !is_none(h->interpOut) && !h->interpOut.on_device) {
    // interpolated phase of the lit subapertures to a host array
    h->interpStage.resize((size_t)h->W * h->W);
    CK(cudaMemcpyAsync(h->interpStage.data(), h->d_interp.p, h->interpStage.size() * sizeof(float),
                       cudaMemcpyDeviceToHost, st));
    h->scatterPending = true;
    *sync = true;
  }
  if (corr_active(h) && !is_none(h->corrimg) && !h->corrimg.on_device) {
    // the reference writes the correlation images of lit subapertures
    const size_t nc = (size_t)h->nsubaps * h->corrPatternSize * h->corrPatternSize;
    h->corrimgStage.resize(nc);
    CK(cudaMemcpyAsync(h->corrimgStage.data(), h->d_corrimg.p, nc * sizeof(float), cudaMemcpyDeviceToHost, st));
    h->scatterPending = true;
    *sync = true;
  }
  if (!h->cents.on_device && !h->imageOnly && !h->centsDirect)
    CK(cudaMemcpyAsync((void*)h->cents.data, h->d_cents.p, (size_t)h->nsubaps * 2 * sizeof(float),
                       cudaMemcpyDeviceToHost, st));
  if (!h->bimg.on_device && !h->bimgDirect) {
    const size_t nb = (size_t)h->nsubaps * h->nimg * h->nimg;
    if (h->imageOnly || h->unlit.empty()) {
      CK(cudaMemcpyAsync((void*)h->bimg.data, h->d_bimg.p, nb * sizeof(float), cudaMemcpyDeviceToHost, st));
    } else if (h->bimgMapped) {
      CK(launch_publish(h->d_bimg.p, h->bimgMapped, h->d_lit.p, (int)h->lit.size(), h->nimg * h->nimg, st));
    } else {
      h->bimgStage.resize(nb);
      CK(cudaMemcpyAsync(h->bimgStage.data(), h->d_bimg.p, nb * sizeof(float), cudaMemcpyDeviceToHost, st));
      h->scatterPending = true;
      *sync = true;
    }
  }
  return SHWFS_OK;
}

// queue one image-input frame (centroidsFromImage)
shwfs_status enqueue_slope(shwfs_handle* h, cudaStream_t st) {
  if (shwfs_status s = prepare_readout(h)) return s;
  // zero-copy host I/O as for phase frames (counter noise, no correlation):
  // the image kernel reads the pinned detector frame and, with the unlit
  // kernel, writes the centroids and images into the pinned host arrays
  const bool zc = h->noiseMode != SHWFS_NOISE_REFERENCE && !corr_active(h);
  const bool zcOut = zc && (h->hostIO & SHWFS_HOSTIO_OUTPUTS);
  const float* img = (const float*)h->inputImage.data;
  if (!h->inputImage.on_device) {
    if (zc && (h->hostIO & SHWFS_HOSTIO_PHASE) && h->imageMapped) {
      img = h->imageMapped;
      h->inDirect = true;
    } else {
      CK(cudaMemcpyAsync(h->d_image.p, h->inputImage.data, (size_t)numel(h->inputImage) * sizeof(float),
                         cudaMemcpyHostToDevice, st));
      img = h->d_image.p;
    }
  }
  h->centsDirect = !h->cents.on_device && zcOut && h->centsMapped && !h->imageOnly;
  h->bimgDirect = !h->bimg.on_device && zcOut && h->bimgMapped;
  float* cents = h->cents.on_device ? (float*)h->cents.data : (h->centsDirect ? h->centsMapped : h->d_cents.p);
  float* bimg = h->bimg.on_device ? (float*)h->bimg.data : (h->bimgDirect ? h->bimgMapped : h->d_bimg.p);
  const int mm = h->nimg * h->nimg;
  if (!h->lit.empty()) {
    WfsArgs a = make_args(h, nullptr, cents, bimg, 1, 0, kPost);
    a.TS = std::max(1, std::min(64, 4096 / mm));
    CK(launch_image(a, img, h->imageDims, h->imageCols, h->d_subapLoc.p, h->numSMs, st));
  }
  if (!h->unlit.empty()) {
    WfsArgs a = make_args(h, nullptr, cents, bimg, 1, 0, 0);
    if (h->noiseMode == SHWFS_NOISE_REFERENCE && h->imageOnly) {
      RefNoiseArgs r{};
      r.nthreads = h->nthreads;
      r.subapStart = h->d_subapStart.p;
      r.subflag = h->d_subflag.p;
      r.poisFlag = h->d_poisFlag.p;
      r.bimg = bimg;
      r.m = h->nimg;
      r.nexp = mm;
      r.readNoise = h->readNoise;
      r.readBg = h->readBg;
      r.floorv = h->noiseFloor;
      r.threshType = h->threshType;
      r.addPoisson = h->addPoisson;
      r.calsource = h->calsource;
      r.imageOnly = h->imageOnly;
      r.imageInput = 1;
      CK(launch_refnoise(r, h->d_rng.p, h->d_status.p, st));
    } else {
      CK(launch_unlit(a, h->d_unlit.p, (int)h->unlit.size(), st));
    }
  }
  return enqueue_corr(h, cents, bimg, 1, st);
}


// one readout from pre-noise images: the noise, threshold and post stages of
// centroidsFromPhase (cmod/src/centmodule.c:1879-1981) on the caller's images
shwfs_status enqueue_prenoise(shwfs_handle* h, const PrenoiseIn& in, cudaStream_t st) {
  if (shwfs_status s = prepare_readout(h)) return s;
  const size_t mm = (size_t)h->nimg * h->nimg, n = (size_t)h->nsubaps * mm;
  float* cents = h->cents.on_device ? (float*)h->cents.data : h->d_cents.p;
  float* bimg = h->bimg.on_device ? (float*)h->bimg.data : h->d_bimg.p;
  CK(cudaMemcpyAsync(bimg, in.images->data, n * sizeof(float),
                     in.images->on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  const int nlit = (int)h->lit.size();
  const long long ntiles = ((long long)nlit + h->TS - 1) / h->TS;
  const int grid = (int)std::max<long long>(1, std::min<long long>(ntiles, (long long)h->numSMs * h->ctasPerSM));
  const bool inject = !is_none(*in.shot) || !is_none(*in.readn);
  if (inject || h->noiseMode == SHWFS_NOISE_REFERENCE)
    CK(launch_pois_flag(h->nsubaps, h->d_totsig.p, h->d_frac.p, h->sky, h->skyIsArr ? 1 : 0, h->d_poisFlag.p, st));
  if (inject) {
    if (h->d_inj.n < 2 * n) CK(h->d_inj.alloc(2 * n));
    InjectArgs g{};
    g.nsubaps = h->nsubaps;
    g.m = h->nimg;
    g.subflag = h->d_subflag.p;
    g.poisFlag = h->d_poisFlag.p;
    g.bimg = bimg;
    const shwfs_array* src[2] = {in.shot, in.readn};
    for (int k = 0; k < 2; k++) {
      if (is_none(*src[k])) continue;
      CK(cudaMemcpyAsync(h->d_inj.p + k * n, src[k]->data, n * sizeof(float),
                         src[k]->on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    }
    g.shot = is_none(*in.shot) ? nullptr : h->d_inj.p;
    g.readn = is_none(*in.readn) ? nullptr : h->d_inj.p + n;
    g.readNoise = h->readNoise;
    g.readBg = h->readBg;
    g.floorv = h->noiseFloor;
    g.threshType = h->threshType;
    g.addPoisson = h->addPoisson;
    g.calsource = h->calsource;
    g.imageOnly = h->imageOnly;
    CK(launch_inject_noise(g, st));
  } else if (h->noiseMode == SHWFS_NOISE_REFERENCE) {
    RefNoiseArgs r{};
    r.nthreads = h->nthreads;
    r.subapStart = h->d_subapStart.p;
    r.subflag = h->d_subflag.p;
    r.poisFlag = h->d_poisFlag.p;
    r.bimg = bimg;
    r.m = h->nimg;
    r.nexp = (int)mm;
    r.readNoise = h->readNoise;
    r.readBg = h->readBg;
    r.floorv = h->noiseFloor;
    r.threshType = h->threshType;
    r.addPoisson = h->addPoisson;
    r.calsource = h->calsource;
    r.imageOnly = h->imageOnly;
    CK(launch_refnoise(r, h->d_rng.p, h->d_status.p, st));
  } else {
    // counter streams on the caller's images, then the post stages
    unsigned postDone = 0;
    if (nlit) {
      WfsArgs a = make_args(h, nullptr, cents, bimg, 1, 0, kNoiseCounter | kPost);
      CK(launch_post(a, h->numSMs, st, &postDone));
    }
    if (!h->unlit.empty() && !(postDone & kPostDidUnlit)) {
      WfsArgs a = make_args(h, nullptr, cents, bimg, 1, 0, 0);
      CK(launch_unlit(a, h->d_unlit.p, (int)h->unlit.size(), st));
    }
    return enqueue_corr(h, cents, bimg, 1, st);
  }
  if (nlit) {
    WfsArgs a = make_args(h, nullptr, cents, bimg, 1, 0, kPost);
    CK(h->entry->launch(a, grid, h->smem, st));
  }
  if (!h->unlit.empty() && !h->imageOnly) {
    WfsArgs a = make_args(h, nullptr, cents, bimg, 1, 0, 0);
    CK(launch_unlit(a, h->d_unlit.p, (int)h->unlit.size(), st));
  }
  return enqueue_corr(h, cents, bimg, 1, st);
}

shwfs_status run_impl(shwfs_handle* h, cudaStream_t st, bool sync, float* elapsed, bool slope = false,
                      const PrenoiseIn* pre = nullptr) {
  auto t0 = std::chrono::steady_clock::now();
  CK(cudaSetDevice(h->device));
  if (!st) st = h->stream;
  if (slope && is_none(h->inputImage)) return fail(SHWFS_ERR_STATE, "centmodule - inputImage is NULL");
  if (!slope && !pre && is_none(h->phs))
    return fail(SHWFS_ERR_STATE, "no phase array is bound (image-input handle)");
  const bool readout = slope || pre || readout_frame(h);
  h->centsDirect = h->bimgDirect = h->inDirect = false;
  const int istate = integ_state(h);
  const bool physical = h->integMode == SHWFS_INTEG_PHYSICAL && !slope && !pre;
  if (physical && istate != 3) {
    // physical integration: every exposed frame forms its images on the
    // device; the readout frame also draws the noise and centroids
    const float* phs = (const float*)h->phs.data;
    if (!h->phs.on_device) {
      CK(cudaMemcpyAsync(h->d_phs.p, h->phs.data, (size_t)numel(h->phs) * sizeof(float), cudaMemcpyHostToDevice,
                         st));
      phs = h->d_phs.p;
    }
    shwfs_status s = enqueue_physical(h, phs, istate, st);
    if (s) return s;
    if (readout) {
      if ((s = publish_outputs(h, st, &sync))) return s;
      h->framesRead++;
    }
  } else if (readout && !physical) {
    shwfs_status s;
    if (slope) {
      s = enqueue_slope(h, st);
    } else if (pre) {
      s = enqueue_prenoise(h, *pre, st);
    } else {
      const size_t nph = (size_t)numel(h->phs);
      const float* phs = (const float*)h->phs.data;
      // zero-copy host I/O (counter noise, no correlation): the kernels
      // read / write the pinned host arrays through their device aliases
      const bool zc = h->noiseMode != SHWFS_NOISE_REFERENCE && !corr_active(h);
      if (!h->phs.on_device) {
        if (zc && !h->interp && (h->hostIO & SHWFS_HOSTIO_PHASE) && h->phsMapped) {
          phs = h->phsMapped;
          h->inDirect = true;
        } else {
          CK(cudaMemcpyAsync(h->d_phs.p, h->phs.data, nph * sizeof(float), cudaMemcpyHostToDevice, st));
          phs = h->d_phs.p;
        }
      }
      const bool zcOut = zc && (h->hostIO & SHWFS_HOSTIO_OUTPUTS);
      h->centsDirect = !h->cents.on_device && zcOut && h->centsMapped && !h->imageOnly;
      float* cents = h->cents.on_device ? (float*)h->cents.data : (h->centsDirect ? h->centsMapped : h->d_cents.p);
      float* bimg = h->bimg.on_device ? (float*)h->bimg.data : h->d_bimg.p;
      float* bimgHost = !h->bimg.on_device && zcOut ? h->bimgMapped : nullptr;
      s = enqueue_readout(h, phs, cents, bimg, 1, 0, st, bimgHost, &h->bimgDirect);
    }
    if (s) return s;
    if ((s = publish_outputs(h, st, &sync))) return s;
    h->framesRead++;
  }
  if (!slope && !pre) {
    // py_run advances the integration counter; py_runSlope does not
    h->curInteg++;
    if (h->curInteg >= h->nintegrations + h->nlatency) h->curInteg = 0;
  }
  // the kernels' status word comes back in stream order with the outputs:
  // the tensor-core forms' noise/centroid kernel writes it to the pinned
  // host word, the reference-stream path copies it
  const bool checkStatus =
      sync && readout && (h->noiseMode == SHWFS_NOISE_REFERENCE || (gemm_active(h) && !slope && !pre && !physical));
  if (checkStatus && h->noiseMode == SHWFS_NOISE_REFERENCE)
    CK(cudaMemcpyAsync(h->h_status, h->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (sync) {
    CK(cudaStreamSynchronize(st));
    if (h->scatterPending) {
      if (!h->bimgStage.empty() && !h->bimg.on_device) {
        const size_t mm = (size_t)h->nimg * h->nimg;
        float* dst = (float*)h->bimg.data;
        for (int i : h->lit) memcpy(dst + i * mm, h->bimgStage.data() + i * mm, mm * sizeof(float));
        h->bimgStage.clear();
      }
      if (!h->interpStage.empty()) {
        const int W = h->W, p = h->phasesize;
        float* dst = (float*)h->interpOut.data;
        for (int i : h->lit) {
          const int sy = i / h->nsubx, sx = i - sy * h->nsubx;
          for (int r = 0; r < p; r++)
            memcpy(dst + (size_t)(sy * p + r) * W + sx * p, h->interpStage.data() + (size_t)(sy * p + r) * W + sx * p,
                   p * sizeof(float));
        }
        h->interpStage.clear();
      }
      if (!h->corrimgStage.empty()) {
        const size_t cc = (size_t)h->corrPatternSize * h->corrPatternSize;
        float* dst = (float*)h->corrimg.data;
        for (int i : h->lit) memcpy(dst + i * cc, h->corrimgStage.data() + i * cc, cc * sizeof(float));
        h->corrimgStage.clear();
      }
      h->scatterPending = false;
    }
    if (checkStatus) {
      const int status = *(volatile int*)h->h_status;
      if (status & 1) return fail(SHWFS_ERR_STATE, "reference-stream Poisson sampler hit its iteration limit");
      if (status & 2) return fail(SHWFS_ERR_STATE, "tensor-core pipeline wait timed out (results invalid)");
    }
  }
  if (elapsed) *elapsed = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
  return SHWFS_OK;
}

}  // namespace

extern "C" {

const char* shwfs_last_error(void) { return g_err.c_str(); }

const char* shwfs_version(void) { return "shwfs-gb300 0.1 (sm_103a)"; }

shwfs_status shwfs_initialise(const shwfs_init* in, shwfs_handle** out) {
  g_err.clear();
  if (!in || !out) return fail(SHWFS_ERR_INVALID, "null argument");
  *out = nullptr;
  auto h = new (std::nothrow) shwfs_handle();
  if (!h) return fail(SHWFS_ERR_NOMEM, "handle allocation failed");
  struct Guard {
    shwfs_handle* h;
    ~Guard() { delete h; }
  } guard{h};

  if (in->nsubaps <= 0 || in->phasesize <= 0 || in->fftsize <= 0 || in->clipsize <= 0 || in->nimg <= 0)
    return fail(SHWFS_ERR_INVALID, "sizes must be positive");
  h->nsubaps = in->nsubaps;
  h->nsubx = (int)sqrtf((float)in->nsubaps);
  if (h->nsubx * h->nsubx != h->nsubaps) return fail(SHWFS_ERR_INVALID, "nsubaps must be nsubx^2");
  h->ncen = in->ncen;
  h->fftsize = in->fftsize;
  h->clipsize = in->clipsize;
  h->nimg = in->nimg;
  h->phasesize = in->phasesize;
  h->preBinOrig = in->preBinningFactor;
  h->parabolicFit = in->parabolicFit;
  h->gaussianFit = in->gaussianFit;
  h->gMin = in->gaussianMinVal;
  h->gRep = in->gaussianReplaceVal;
  if (h->phasesize > h->fftsize) return fail(SHWFS_ERR_INVALID, "phasesize must not exceed fftsize");
  if (h->nimg > h->clipsize) return fail(SHWFS_ERR_INVALID, "nimg must not exceed clipsize");
  if (h->ncen < 1 || h->ncen > h->nimg) return fail(SHWFS_ERR_INVALID, "ncen must be in [1, nimg]");
  if ((h->parabolicFit != 0 || h->gaussianFit > 0) && h->parabolicFit + h->gaussianFit > h->ncen)
    return fail(SHWFS_ERR_INVALID, "fit size %d larger than the centroid window %d", h->parabolicFit + h->gaussianFit,
                h->ncen);
  if ((h->parabolicFit < 0 || h->gaussianFit > 0) && h->ncen < 3)
    return fail(SHWFS_ERR_INVALID, "a fit needs a centroid window of at least 3 pixels");
  // arrays: validation as py_initialise, plus size checks the C code trusts;
  // everything that needs no GPU is checked before the first CUDA call
  const int p = h->phasesize, nsa = h->nsubaps, m = h->nimg;
  if (is_none(in->cents) || check_f32(in->cents, "cents")) return fail(SHWFS_ERR_INVALID, "cents must be float and contiguous");
  if (numel(in->cents) < 2LL * nsa) return fail(SHWFS_ERR_INVALID, "cents must hold nsubaps*2 values");
  const int W = h->nsubx * p;
  h->W = W;
  if (!is_none(in->phs)) {
    if (check_f32(in->phs, "phs")) return SHWFS_ERR_INVALID;
    if (in->phs.ndim == 2)
      h->phaseAmp = 0;
    else if (in->phs.ndim == 3 && in->phs.shape[0] == 2)
      h->phaseAmp = 1;
    else
      return fail(SHWFS_ERR_INVALID, "phase should be 2D or 3D (for phase+amp)");
    const int64_t ny = in->phs.shape[h->phaseAmp], nx = in->phs.shape[h->phaseAmp + 1];
    if (ny != W || nx != W) {
      // interpolatePhase (cmod/src/centmodule.c:2929-2933): the reference
      // takes the input as square (dims[0] both ways) and reads the
      // amplitude plane at the output-size offset, so only square
      // phase-only inputs have a defined meaning
      if (h->phaseAmp)
        return fail(SHWFS_ERR_UNSUPPORTED, "phase+amplitude of size %lldx%lld would need interpolation to %dx%d; "
                    "the reference reads its amplitude plane at the %dx%d offset, which is not reproduced",
                    (long long)ny, (long long)nx, W, W, W, W);
      if (ny != nx) return fail(SHWFS_ERR_INVALID, "phase of size %lldx%lld: interpolation needs a square phase", (long long)ny, (long long)nx);
      if (ny < 4) return fail(SHWFS_ERR_INVALID, "phase of size %lldx%lld is too small to interpolate", (long long)ny, (long long)nx);
      h->interp = true;
      h->inputPhaseSize = (int)ny;
    }
  }
  // image input (cmod/src/centmodule.c:3117-3157)
  if (!is_none(in->inputImage)) {
    const shwfs_array& im = in->inputImage;
    if (check_f32(im, "inputImage")) return fail(SHWFS_ERR_INVALID, "inputImage array must be float and contiguous");
    if (im.ndim == 2) {
      if (im.shape[0] * im.shape[1] != (int64_t)m * m * nsa)
        return fail(SHWFS_ERR_INVALID, "inputImage should be %d x %d (is %lld x %lld)", m * h->nsubx, m * h->nsubx,
                    (long long)im.shape[0], (long long)im.shape[1]);
      h->imageDims = 2;
      h->imageRows = (int)im.shape[0];
      h->imageCols = (int)im.shape[1];
    } else if (im.ndim == 4) {
      if (im.shape[0] * im.shape[1] != nsa || im.shape[2] != m || im.shape[3] != m)
        return fail(SHWFS_ERR_INVALID, "inputImage should be %dx%dx%dx%d", h->nsubx, h->nsubx, m, m);
      h->imageDims = 4;
      h->imageRows = h->imageCols = m;
    } else {
      return fail(SHWFS_ERR_INVALID, "inputImage should be 2D or 4D");
    }
  }
  if (!is_none(in->subapLocation)) {
    const shwfs_array& sl = in->subapLocation;
    if (sl.dtype != SHWFS_I32) return fail(SHWFS_ERR_INVALID, "subapLocation array must be int32 and contiguous");
    if (numel(sl) != 4LL * nsa)
      return fail(SHWFS_ERR_INVALID, "subapLocation array should be of size %d (is %lld)", nsa * 4, (long long)numel(sl));
    h->subapLoc = to_host<int>(sl);
  }
  if (h->imageDims == 2) {
    // every window must lie inside the image and fit the nimg x nimg image
    for (int i = 0; i < nsa; i++) {
      int r0, r1, c0, c1;
      if (!h->subapLoc.empty()) {
        r0 = h->subapLoc[i * 4];
        r1 = h->subapLoc[i * 4 + 1];
        c0 = h->subapLoc[i * 4 + 2];
        c1 = h->subapLoc[i * 4 + 3];
      } else {
        r0 = (i / h->nsubx) * m;
        r1 = r0 + m;
        c0 = (i % h->nsubx) * m;
        c1 = c0 + m;
      }
      if (r0 < 0 || c0 < 0 || r1 < r0 || c1 < c0 || r1 - r0 > m || c1 - c0 > m || r1 > h->imageRows ||
          c1 > h->imageCols)
        return fail(SHWFS_ERR_INVALID, "subaperture %d window [%d:%d,%d:%d] does not fit the image or nimg", i, r0, r1,
                    c0, c1);
    }
  }
  if (is_none(in->pupfn) || check_f32(in->pupfn, "pupfn")) return fail(SHWFS_ERR_INVALID, "pupfn must be float and contiguous");
  if (numel(in->pupfn) != (int64_t)nsa * p * p) return fail(SHWFS_ERR_INVALID, "pupfn must be (nsubx,nsubx,phasesize,phasesize)");
  if (is_none(in->subflag) || in->subflag.dtype != SHWFS_I32) return fail(SHWFS_ERR_INVALID, "subflag must be int32 and contiguous");
  if (numel(in->subflag) != nsa) return fail(SHWFS_ERR_INVALID, "subflag must have nsubaps entries");
  if (is_none(in->bimg) || check_f32(in->bimg, "bimg")) return fail(SHWFS_ERR_INVALID, "bimg must be float and contiguous");
  if (numel(in->bimg) < (int64_t)nsa * m * m) return fail(SHWFS_ERR_INVALID, "bimg must hold nsubaps*nimg*nimg values");
  if (is_none(in->fracSubArea) || check_f32(in->fracSubArea, "fracSubArea"))
    return fail(SHWFS_ERR_INVALID, "fracSubArea must be float and contiguous");
  if (numel(in->fracSubArea) != nsa) return fail(SHWFS_ERR_INVALID, "fracSubArea must have nsubaps entries");

  h->readNoise = in->readnoise;
  h->readBg = in->readbg;
  h->threshType = in->threshType;
  h->addPoisson = in->addPoisson;
  h->noiseFloor = in->noiseFloor;
  h->calsource = in->calsource;
  h->pxlPower = in->pxlPower;
  h->nintegrations = in->nintegrations;
  h->nlatency = in->nlatency;
  h->seed = in->seed;
  h->opticalBinning = in->opticalBinning;
  h->imageOnly = in->imageOnly;
  h->corrThresh = in->corrThresh;
  h->correlationCentroiding = in->correlationCentroiding;
  if (h->nintegrations < 1) return fail(SHWFS_ERR_INVALID, "nintegrations must be >= 1");
  if (h->nlatency < 0) return fail(SHWFS_ERR_INVALID, "nlatency must be >= 0");
  if (in->nthreads < 1) return fail(SHWFS_ERR_INVALID, "nthreads must be >= 1");
  if (!is_none(in->sigArr) && (check_f32(in->sigArr, "sig array") || in->sigArr.ndim != 1 ||
                               in->sigArr.shape[0] != nsa))
    return fail(SHWFS_ERR_INVALID, "sig arr dimensions must be 1D (nsubx^2)");
  if (!is_none(in->skybrightnessArr) &&
      (check_f32(in->skybrightnessArr, "skybrightness") || in->skybrightnessArr.ndim != 3 ||
       in->skybrightnessArr.shape[0] != nsa || in->skybrightnessArr.shape[1] != m ||
       in->skybrightnessArr.shape[2] != m))
    return fail(SHWFS_ERR_INVALID, "skybrightness should be 3D array shape nsubaps,nimg,nimg");
  if (!is_none(in->useBrightestArr) && (in->useBrightestArr.dtype != SHWFS_I32 ||
                                        in->useBrightestArr.ndim != 1 || in->useBrightestArr.shape[0] != nsa))
    return fail(SHWFS_ERR_INVALID, "useBrightest array should be 1D int32 of shape nsubaps (nsubx^2)");
  if (!is_none(in->spotpsf)) {
    const shwfs_array& ps = in->spotpsf;
    if (ps.ndim != 2 && ps.ndim != 4) return fail(SHWFS_ERR_INVALID, "spotpsf not 2d or 4d");
    if (check_f32(ps, "spotpsf")) return SHWFS_ERR_INVALID;
    const int P = (int)ps.shape[ps.ndim - 1];
    if (ps.shape[ps.ndim - 2] != P) return fail(SHWFS_ERR_INVALID, "spotpsf must be square");
    if (ps.ndim == 4 && ps.shape[0] * ps.shape[1] != nsa)
      return fail(SHWFS_ERR_INVALID, "spotpsf 4d must be (nsubx,nsubx,P,P)");
    if (P < h->clipsize) return fail(SHWFS_ERR_INVALID, "spotpsf dimensions should be at least clipsize");
  }
  if (!is_none(in->centWeight)) {
    const shwfs_array& cw = in->centWeight;
    if (cw.ndim != 2 && cw.ndim != 4) return fail(SHWFS_ERR_INVALID, "centWeight not 2d or 4d");
    if (check_f32(cw, "centWeight")) return SHWFS_ERR_INVALID;
    if (cw.shape[cw.ndim - 2] != m || cw.shape[cw.ndim - 1] != m)
      return fail(SHWFS_ERR_INVALID, "centweight array not correct dimensions (need to be nsubx,nsubx,corrsize,corrsize)");
  }

  CK(cudaGetDevice(&h->device));
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(cudaDeviceGetAttribute(&h->numSMs, cudaDevAttrMultiProcessorCount, h->device));

  shwfs_status s;
  if ((s = set_sig(h, in->sig, &in->sigArr))) return s;
  if ((s = set_sky(h, in->skybrightness, &in->skybrightnessArr))) return s;
  if ((s = set_use_brightest(h, in->useBrightest, &in->useBrightestArr))) return s;

  h->subflag = to_host<int>(in->subflag);
  h->pup = to_host<float>(in->pupfn);
  h->frac = to_host<float>(in->fracSubArea);
  for (int i = 0; i < nsa; i++) (h->subflag[i] == 1 ? h->lit : h->unlit).push_back(i);
  CK(h->d_subflag.upload(h->subflag.data(), nsa));
  CK(h->d_lit.upload(h->lit.data(), h->lit.size()));
  CK(h->d_unlit.upload(h->unlit.data(), h->unlit.size()));
  CK(h->d_pup.upload(h->pup.data(), h->pup.size()));
  CK(h->d_frac.upload(h->frac.data(), nsa));
  CK(h->d_poisFlag.alloc(nsa));
  CK(pois_table_device(&h->poisTab));
  CK(h->d_status.alloc(1));
  if (h->interp) CK(h->d_interp.alloc((size_t)h->W * h->W));
  CK(cudaMemset(h->d_status.p, 0, sizeof(int)));
  CK(cudaHostAlloc((void**)&h->h_status, sizeof(int), cudaHostAllocMapped));
  *h->h_status = 0;
  CK(cudaHostGetDevicePointer((void**)&h->h_statusDev, h->h_status, 0));

  // tiltfn (cmod/src/centmodule.c:3074-3081)
  std::vector<float> tilt((size_t)p * p);
  const float tmp = (float)(M_PI / h->fftsize * (h->fftsize + 1.));
  for (int i = 0; i < p; i++)
    for (int j = 0; j < p; j++) tilt[i * p + j] = tmp * (float)(i + j + 1 - p);
  CK(h->d_tilt.upload(tilt.data(), tilt.size()));

  if ((s = set_spot_psf(h, in->spotpsf))) return s;
  if ((s = load_corr_pattern(h, in->corrPattern))) return s;
  if (!is_none(in->corrimg)) {
    if (check_f32(in->corrimg, "corrimg")) return fail(SHWFS_ERR_INVALID, "corrimg must be float and contiguous");
    h->corrimg = in->corrimg;
  }
  if ((s = set_cent_weight(h, in->centWeight))) return s;
  if ((s = setup_threads(h, in->nthreads))) return s;
  if ((s = prepare_bin(h))) return s;
  if ((s = update_totsig(h))) return s;
  if ((s = plan(h))) return s;

  if (!is_none(in->phs)) {
    const size_t nph = (size_t)numel(in->phs);
    if ((s = bind_io(h, h->phs, in->phs, h->d_phs, nph, false))) return s;
  }
  if (!is_none(in->inputImage)) {
    if ((s = bind_io(h, h->inputImage, in->inputImage, h->d_image, (size_t)numel(in->inputImage), false))) return s;
  }
  if (!h->subapLoc.empty()) CK(h->d_subapLoc.upload(h->subapLoc.data(), h->subapLoc.size()));
  if ((s = bind_io(h, h->cents, in->cents, h->d_cents, (size_t)nsa * 2, true))) return s;
  if ((s = bind_io(h, h->bimg, in->bimg, h->d_bimg, (size_t)nsa * m * m, true))) return s;

  guard.h = nullptr;
  *out = h;
  return SHWFS_OK;
}

shwfs_status shwfs_run(shwfs_handle* h, float* elapsed_s) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  return run_impl(h, nullptr, true, elapsed_s);
}

shwfs_status shwfs_run_async(shwfs_handle* h, void* stream) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  return run_impl(h, (cudaStream_t)stream, false, nullptr);
}

shwfs_status shwfs_run_slope(shwfs_handle* h, float* elapsed_s) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  return run_impl(h, nullptr, true, elapsed_s, true);
}

shwfs_status shwfs_run_prenoise(shwfs_handle* h, const shwfs_array* images, const shwfs_array* shot,
                                const shwfs_array* readn, float* elapsed_s) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  const shwfs_array none{};
  if (!shot) shot = &none;
  if (!readn) readn = &none;
  const int64_t n = (int64_t)h->nsubaps * h->nimg * h->nimg;
  if (!images || is_none(*images)) return fail(SHWFS_ERR_INVALID, "pre-noise images are required");
  const shwfs_array* arrs[3] = {images, shot, readn};
  const char* names[3] = {"images", "shot", "readn"};
  for (int k = 0; k < 3; k++) {
    if (is_none(*arrs[k])) continue;
    if (arrs[k]->dtype != SHWFS_F32 || numel(*arrs[k]) != n)
      return fail(SHWFS_ERR_INVALID, "%s must be float32 with nsubaps*nimg*nimg = %lld values", names[k],
                  (long long)n);
  }
  if (h->opticalBinning == 1)
    return fail(SHWFS_ERR_UNSUPPORTED, "pre-noise images with optical binning (images are binned before noise)");
  if (h->phaseAmp)
    return fail(SHWFS_ERR_UNSUPPORTED, "pre-noise images on a phase+amplitude handle (its Poisson flag needs the amplitude)");
  const bool drawsShot = h->addPoisson == 1 && h->calsource == 0;
  const bool drawsRead = h->readNoise != 0.f && h->calsource == 0;
  const bool inject = !is_none(*shot) || !is_none(*readn);
  if (inject && ((drawsShot && is_none(*shot)) || (drawsRead && is_none(*readn))))
    return fail(SHWFS_ERR_INVALID, "injected noise needs %s for this configuration",
                drawsShot && is_none(*shot) ? "shot (Poisson draws)" : "readn (read-noise draws)");
  PrenoiseIn in{images, shot, readn};
  return run_impl(h, nullptr, true, elapsed_s, false, &in);
}

shwfs_status shwfs_run_batch(shwfs_handle* h, int nframes, const float* phs, int64_t phs_frame_stride, float* cents,
                             float* bimg, void* stream) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  if (nframes < 1 || !phs || !cents || !bimg) return fail(SHWFS_ERR_INVALID, "bad batch arguments");
  if (h->interp && (size_t)nframes * h->W * h->W > h->d_interp.n) {
    CK(cudaSetDevice(h->device));
    CK(h->d_interp.alloc((size_t)nframes * h->W * h->W));  // grows; cudaFree waits for work in flight
  }
  if (h->noiseMode == SHWFS_NOISE_REFERENCE && nframes != 1)
    return fail(SHWFS_ERR_UNSUPPORTED, "reference-stream noise runs one frame at a time");
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  shwfs_status s = enqueue_readout(h, phs, cents, bimg, nframes, phs_frame_stride, st);
  if (s) return s;
  h->framesRead += nframes;
  return SHWFS_OK;
}

shwfs_status shwfs_set_io(shwfs_handle* h, const shwfs_array* phs, const shwfs_array* cents, const shwfs_array* bimg) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  h->version++;
  shwfs_status s;
  if (phs) {
    if (numel(*phs) != numel(h->phs) || phs->dtype != SHWFS_F32) return fail(SHWFS_ERR_INVALID, "phs shape mismatch");
    if ((s = bind_io(h, h->phs, *phs, h->d_phs, (size_t)numel(*phs), false))) return s;
  }
  if (cents) {
    if (numel(*cents) < 2LL * h->nsubaps || cents->dtype != SHWFS_F32) return fail(SHWFS_ERR_INVALID, "cents shape mismatch");
    if ((s = bind_io(h, h->cents, *cents, h->d_cents, (size_t)h->nsubaps * 2, true))) return s;
  }
  if (bimg) {
    if (numel(*bimg) < (int64_t)h->nsubaps * h->nimg * h->nimg || bimg->dtype != SHWFS_F32)
      return fail(SHWFS_ERR_INVALID, "bimg shape mismatch");
    if ((s = bind_io(h, h->bimg, *bimg, h->d_bimg, (size_t)h->nsubaps * h->nimg * h->nimg, true))) return s;
  }
  return SHWFS_OK;
}

shwfs_status shwfs_update(shwfs_handle* h, int code, const shwfs_value* v) {
  if (!h || !v) return fail(SHWFS_ERR_INVALID, "null argument");
  g_err.clear();
  h->version++;
  CK(cudaSetDevice(h->device));
  auto need = [&](int kind, const char* what) -> shwfs_status {
    if (v->kind != kind) return fail(SHWFS_ERR_INVALID, "centmodule: Error extracting %s value", what);
    return SHWFS_OK;
  };
  auto num = [&](const char* what, double* out) -> shwfs_status {
    if (v->kind == SHWFS_VAL_FLOAT) {
      *out = v->dval;
      return SHWFS_OK;
    }
    if (v->kind == SHWFS_VAL_INT) {
      *out = (double)v->ival;
      return SHWFS_OK;
    }
    return fail(SHWFS_ERR_INVALID, "centmodule: Error extracting float value for %s", what);
  };
  shwfs_status s = SHWFS_OK;
  double d = 0;
  switch (code) {
    case SHWFS_CALSOURCE:
      if ((s = need(SHWFS_VAL_INT, "integer"))) return s;
      h->calsource = (int)v->ival;
      break;
    case SHWFS_SIG:
      if (v->kind == SHWFS_VAL_ARRAY) return set_sig(h, 0, &v->arr[0]);
      if ((s = num("sig", &d))) return s;
      h->sig = (float)d;
      return update_totsig(h);
    case SHWFS_ADDPOISSON:
      if ((s = need(SHWFS_VAL_INT, "integer"))) return s;
      h->addPoisson = (int)v->ival;
      break;
    case SHWFS_NCEN:
      if ((s = need(SHWFS_VAL_INT, "integer"))) return s;
      if (v->ival < 1 || v->ival > h->nimg) return fail(SHWFS_ERR_INVALID, "ncen must be in [1, nimg]");
      h->ncen = (int)v->ival;
      break;
    case SHWFS_READNOISE:
      if ((s = num("readnoise", &d))) return s;
      h->readNoise = (float)d;
      break;
    case SHWFS_READBG:
      if ((s = num("readbg", &d))) return s;
      h->readBg = (float)d;
      break;
    case SHWFS_NOISEFLOOR:
      if ((s = num("noisefloor", &d))) return s;
      h->noiseFloor = (float)d;
      break;
    case SHWFS_SKYBRIGHTNESS:
      if (v->kind == SHWFS_VAL_ARRAY) return set_sky(h, 0, &v->arr[0]);
      if ((s = num("skybrightness", &d))) return s;
      return set_sky(h, d, nullptr);
    case SHWFS_PXLPOWER:
      if ((s = num("pxlpower", &d))) return s;
      h->pxlPower = (float)d;
      break;
    case SHWFS_SPOTPSF: {
      shwfs_array none{};
      if ((s = set_spot_psf(h, v->kind == SHWFS_VAL_ARRAY ? v->arr[0] : none))) return s;
      if ((s = update_totsig(h))) return s;
      if ((s = plan(h))) return s;
      h->gemmStaging = 0;
      return build_gemm(h);
    }
    case SHWFS_NTHREADS:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      return setup_threads(h, (int)v->ival);
    case SHWFS_OPTICALBINNING:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      h->opticalBinning = (int)v->ival;
      break;
    case SHWFS_CENTWEIGHT: {
      shwfs_array none{};
      if ((s = set_cent_weight(h, v->kind == SHWFS_VAL_ARRAY ? v->arr[0] : none))) return s;
      return plan(h);
    }
    case SHWFS_CORRELATIONCENTROIDING:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      if (v->ival < 0 || v->ival > 5) return fail(SHWFS_ERR_INVALID, "correlationCentroiding must be 0..5");
      h->correlationCentroiding = (int)v->ival;
      // centWeight of the wrong size is dropped, as the reference does
      if (h->centWeightDim && h->cwSize != corr_size(h)) {
        h->centWeightDim = 0;
        h->d_cw.reset();
      }
      return plan(h);
    case SHWFS_CORRTHRESH:
      if ((s = num("corrThresh", &d))) return s;
      h->corrThresh = (float)d;
      break;
    case SHWFS_CORRPATTERN: {
      shwfs_array none{};
      const bool arr = v->kind == SHWFS_VAL_ARRAY;
      if (arr && h->corrPatternSize && v->arr[0].ndim == 4 && v->arr[0].shape[2] != h->corrPatternSize)
        return fail(SHWFS_ERR_INVALID, "centmodule - corrPattern has changed size - please don't do that");
      return set_corr_pattern(h, arr ? v->arr[0] : none);
    }
    case SHWFS_CALDATA: {
      if (v->kind == SHWFS_VAL_NONE) {
        h->haveCalData = false;
        h->calNSteps = 0;
        break;
      }
      if (v->kind != SHWFS_VAL_TUPLE3) return fail(SHWFS_ERR_INVALID, "centmodule - calibration stuff not a tuple");
      const shwfs_array &cd = v->arr[0], &cb = v->arr[1], &cs = v->arr[2];
      if (check_f32(cd, "calData") || check_f32(cs, "calStep")) return fail(SHWFS_ERR_INVALID, "calData/calStep should be float32 contiguous");
      if (cb.dtype != SHWFS_I32) return fail(SHWFS_ERR_INVALID, "calBounds should be int32 contiguous");
      if (cs.ndim != 1) return fail(SHWFS_ERR_INVALID, "calStep should be 1d");
      const int nsteps = (int)cs.shape[0];
      if (cd.ndim != 4 || cd.shape[0] != 2 || cd.shape[1] * cd.shape[2] != h->nsubaps || cd.shape[3] != nsteps)
        return fail(SHWFS_ERR_INVALID, "calData should be 4d, (2,nsubx,nsubx,steps)");
      if (cb.ndim != 4 || cb.shape[0] != 2 || cb.shape[1] * cb.shape[2] != h->nsubaps || cb.shape[3] != 2)
        return fail(SHWFS_ERR_INVALID, "calBounds should be 4d (2,nsubx,nsubx,2)");
      std::vector<float> vd = to_host<float>(cd), vs = to_host<float>(cs);
      std::vector<int> vb = to_host<int>(cb);
      for (int k : vb)
        if (k < 0 || k >= nsteps) return fail(SHWFS_ERR_INVALID, "calBounds entries must index calSteps");
      CK(h->d_calData.upload(vd.data(), vd.size()));
      CK(h->d_calSteps.upload(vs.data(), vs.size()));
      CK(h->d_calBounds.upload(vb.data(), vb.size()));
      h->calNSteps = nsteps;
      h->haveCalData = true;
      break;
    }
    case SHWFS_REFCENTS:
      if (v->kind == SHWFS_VAL_ARRAY) {
        if (check_f32(v->arr[0], "refCents")) return fail(SHWFS_ERR_INVALID, "refCents must be float contig array");
        if (numel(v->arr[0]) < 2LL * h->nsubaps) return fail(SHWFS_ERR_INVALID, "refCents must hold nsubaps*2 values");
        std::vector<float> r = to_host<float>(v->arr[0]);
        CK(h->d_ref.upload(r.data(), (size_t)h->nsubaps * 2));
        h->haveRef = true;
      } else {
        h->haveRef = false;
      }
      break;
    case SHWFS_CALCOEFF:
      if (v->kind == SHWFS_VAL_ARRAY) {
        const shwfs_array& c = v->arr[0];
        if (check_f32(c, "calCoeff")) return fail(SHWFS_ERR_INVALID, "calCoeff should be float32 contiguous");
        if (c.ndim != 4 || c.shape[2] != 2 || c.shape[0] * c.shape[1] != h->nsubaps)
          return fail(SHWFS_ERR_INVALID, "calCoeff should be 4d (nsubx,nsubx,2,ncoeff)");
        std::vector<float> vc = to_host<float>(c);
        CK(h->d_calCoeff.upload(vc.data(), vc.size()));
        h->calNCoeff = (int)c.shape[3];
        h->haveCalCoeff = true;
      } else if (v->kind == SHWFS_VAL_NONE) {
        h->haveCalCoeff = false;
        h->calNCoeff = 0;
      } else {
        return fail(SHWFS_ERR_INVALID, "centmodule: Error in setCalCoeff");
      }
      break;
    case SHWFS_USEBRIGHTEST:
      if (v->kind == SHWFS_VAL_INT) return set_use_brightest(h, (int)v->ival, nullptr);
      if (v->kind == SHWFS_VAL_ARRAY) return set_use_brightest(h, 0, &v->arr[0]);
      return fail(SHWFS_ERR_INVALID, "centmodule: Error in set useBrightest");
    case SHWFS_INTEGSTEPS:
      if ((s = need(SHWFS_VAL_INT, "int"))) return fail(SHWFS_ERR_INVALID, "centmodule: Error in set integsteps");
      if (v->ival < 1) return fail(SHWFS_ERR_INVALID, "integsteps must be >= 1");
      h->nintegrations = (int)v->ival;
      break;
    case SHWFS_OUTPUTPHASEARR:
      // interpolatedPhaseOutput (cmod/src/centmodule.c:1745-1755): written
      // only while the phase is interpolated, lit subapertures only
      if (v->kind == SHWFS_VAL_ARRAY) {
        const shwfs_array& ar = v->arr[0];
        if (check_f32(ar, "interpolated phase output")) return SHWFS_ERR_INVALID;
        if (numel(ar) < (int64_t)h->W * h->W)
          return fail(SHWFS_ERR_INVALID, "interpolated phase output must hold %dx%d values", h->W, h->W);
        h->interpOut = ar;
      } else {
        h->interpOut = shwfs_array{};
      }
      break;
    case SHWFS_FORM:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      if (v->ival < SHWFS_FORM_FP32 || v->ival > SHWFS_FORM_TF32)
        return fail(SHWFS_ERR_INVALID, "unknown compute form %lld", (long long)v->ival);
      h->form = (int)v->ival;
      h->gemmStaging = 0;
      return build_gemm(h);
    case SHWFS_GEMMSTAGING:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      if (v->ival < 0 || (h->gemmCandidates > 0 && v->ival >= h->gemmCandidates))
        return fail(SHWFS_ERR_INVALID, "staging index %lld outside [0, %d)", (long long)v->ival,
                    h->gemmCandidates);
      h->gemmStaging = (int)v->ival;
      return build_gemm(h);
    case SHWFS_TILESUBAPS:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      if (v->ival < 0 || v->ival > 64) return fail(SHWFS_ERR_INVALID, "tile size must be in [0, 64]");
      h->tileOverride = (int)v->ival;
      return plan(h);
    case SHWFS_HOSTIO:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      if (v->ival < 0 || v->ival > (SHWFS_HOSTIO_OUTPUTS | SHWFS_HOSTIO_PHASE))
        return fail(SHWFS_ERR_INVALID, "unknown host I/O switches %lld", (long long)v->ival);
      h->hostIO = (int)v->ival;
      break;
    case SHWFS_INTEGMODE:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      if (v->ival != SHWFS_INTEG_COMPAT && v->ival != SHWFS_INTEG_PHYSICAL)
        return fail(SHWFS_ERR_INVALID, "unknown integration mode %lld", (long long)v->ival);
      if (v->ival == SHWFS_INTEG_PHYSICAL && (h->interp || h->phaseAmp || h->opticalBinning == 1))
        return fail(SHWFS_ERR_UNSUPPORTED,
                    "physical integration with phase interpolation, phase+amplitude or optical binning");
      h->integMode = (int)v->ival;
      h->curInteg = 0;  // a new exposure starts
      break;
    case SHWFS_NOISEMODE:
      if ((s = need(SHWFS_VAL_INT, "int"))) return s;
      if (v->ival != SHWFS_NOISE_COUNTER && v->ival != SHWFS_NOISE_REFERENCE)
        return fail(SHWFS_ERR_INVALID, "unknown noise mode %lld", (long long)v->ival);
      h->noiseMode = (int)v->ival;
      break;
    default:
      return fail(SHWFS_ERR_INVALID, "centmodule: Code %d not recognised, nothing updated", code);
  }
  return SHWFS_OK;
}

shwfs_status shwfs_free(shwfs_handle* h) {
  if (!h) return SHWFS_OK;
  cudaSetDevice(h->device);
  // work of this handle may be queued on the caller's streams (run_async,
  // run_batch, batch graphs) and write into its pinned host words and
  // aliases: let the device drain before they are freed and unregistered
  cudaDeviceSynchronize();
  delete h;
  return SHWFS_OK;
}

shwfs_status shwfs_test_correlation(int n, const float* img, float* corr) {
  if (n < 1 || n > 4096 || !img || !corr) return fail(SHWFS_ERR_INVALID, "centmodule - corr/img wrong shape");
  const size_t nn = (size_t)n * n;
  // the pattern's unnormalised inverse transform, as load_corr_pattern
  std::vector<double> k;
  hc2r_2d(corr, n, k);
  std::vector<float> kf(nn);
  for (size_t i = 0; i < nn; i++) kf[i] = (float)k[i];
  float *dImg = nullptr, *dK = nullptr, *dOut = nullptr;
  cudaError_t e = cudaMalloc((void**)&dImg, nn * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&dK, nn * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&dOut, nn * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dImg, img, nn * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dK, kf.data(), nn * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_test_corr(n, dImg, dK, dOut, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(corr, dOut, nn * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dImg);
  cudaFree(dK);
  cudaFree(dOut);
  if (e != cudaSuccess) return fail(SHWFS_ERR_CUDA, "testcorrelation: %s", cudaGetErrorString(e));
  return SHWFS_OK;
}

shwfs_status shwfs_get_info(const shwfs_handle* h, shwfs_info* info) {
  if (!h || !info) return fail(SHWFS_ERR_INVALID, "null argument");
  info->nsubx = h->nsubx;
  info->nsubaps = h->nsubaps;
  info->nlit = (int)h->lit.size();
  info->fftsize = h->fftsize;
  info->psfsize = h->psfsize;
  info->clipsize = h->clipsize;
  info->nimg = h->nimg;
  info->phasesize = h->phasesize;
  info->tile_subaps = h->TS;
  info->smem_bytes = h->smem;
  const long long ntiles = ((long long)h->lit.size() + h->TS - 1) / h->TS;
  info->grid_ctas = (int)std::max<long long>(1, std::min<long long>(ntiles, (long long)h->numSMs * h->ctasPerSM));
  info->noise_mode = h->noiseMode;
  info->cur_integ = h->curInteg;
  info->frames_read = h->framesRead;
  info->form = h->form;
  info->form_active = gemm_active(h) ? h->form : SHWFS_FORM_FP32;
  info->host_io_direct = (h->centsDirect ? 1 : 0) | (h->bimgDirect ? 2 : 0) | (h->inDirect ? 4 : 0);
  info->gemm_kcb = h->gemmBuilt ? h->gemm.KCB : 0;
  info->gemm_nw = h->gemmBuilt ? h->gemm.NW : 0;
  info->gemm_nk = h->gemmBuilt ? h->gemm.NK : 0;
  info->gemm_dbuf = h->gemmBuilt ? (h->gemm.dbE ? 1 : 0) | (h->gemm.dbA2 ? 2 : 0) : 0;
  info->gemm_cw = h->gemmBuilt ? h->gemm.CW : 0;
  info->gemm_staging = h->gemmBuilt ? h->gemmStaging : 0;
  info->gemm_candidates = h->gemmBuilt ? h->gemmCandidates : 0;
  return SHWFS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batches: one CUDA graph per readout frame of several handles
// ---------------------------------------------------------------------------

struct shwfs_batch {
  std::vector<shwfs_handle*> hs;
  std::vector<uint64_t> versions;   // handle versions the graph was captured at
  std::vector<uint64_t> ctrFrames;  // frame index each device counter holds
  int device = 0;
  cudaStream_t cap = nullptr;  // capture origin and default launch stream
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> ev;  // ev[0] fork, ev[1 + i] join of branch i
  // the multi-handle fused-kernel launches' branch and its join
  cudaStream_t multiBranch = nullptr;
  cudaEvent_t multiJoin = nullptr;
  int multiLaunches = 0;  // multi-handle launches in the captured graph
  bool multiEnabled = false;  // shwfs_batch_set_multi
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  DevBuf<unsigned long long*> d_ctrs;

  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  ~shwfs_batch() {
    cudaSetDevice(device);
    if (cap) cudaStreamSynchronize(cap);
    drop_graph();
    for (cudaStream_t s : branch) cudaStreamDestroy(s);
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (multiBranch) cudaStreamDestroy(multiBranch);
    if (multiJoin) cudaEventDestroy(multiJoin);
    if (cap) cudaStreamDestroy(cap);
  }
};

namespace {

// record every handle's readout on its own branch of one graph, then the
// counter bump; the handles' launches read their frame index from the
// device counters, so a replay needs no host-side argument change
shwfs_status batch_capture(shwfs_batch* b) {
  b->drop_graph();
  for (shwfs_handle* h : b->hs)
    if (shwfs_status s = prepare_readout(h)) return s;
  // handles whose readout is one fused FP32 kernel plus independent work
  // (counter noise, no correlation, no phase interpolation) and that share
  // an instantiation with another such handle: their fused kernels run as
  // one multi-handle launch on a branch of their own
  std::vector<DeferredPlain> deferred;
  for (shwfs_handle* h : b->hs) {
    h->plainSink = nullptr;
    const bool ok = b->multiEnabled && h->entry && !gemm_active(h) && h->noiseMode == SHWFS_NOISE_COUNTER && !corr_active(h) &&
                    !h->interp && !h->lit.empty();
    if (!ok) continue;
    // same instantiation and the same shared-memory footprint (so that the
    // multi-handle launch keeps each handle's occupancy)
    int same = 0;
    for (shwfs_handle* o : b->hs)
      same += (o->entry == h->entry && o->smem == h->smem && !gemm_active(o) && o->noiseMode == SHWFS_NOISE_COUNTER &&
               !corr_active(o) && !o->interp && !o->lit.empty())
                  ? 1
                  : 0;
    if (same >= 2) h->plainSink = &deferred;
  }
  b->multiLaunches = 0;
  CK(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed));
  auto body = [&]() -> shwfs_status {
    CK(cudaEventRecord(b->ev[0], b->cap));
    for (size_t i = 0; i < b->hs.size(); i++) {
      shwfs_handle* h = b->hs[i];
      CK(cudaStreamWaitEvent(b->branch[i], b->ev[0], 0));
      h->graphCtr = h->d_frameCtr.p;
      shwfs_status s = enqueue_readout(h, (const float*)h->phs.data, (float*)h->cents.data, (float*)h->bimg.data, 1,
                                       0, b->branch[i]);
      h->graphCtr = nullptr;
      if (s) return s;
      CK(cudaEventRecord(b->ev[1 + i], b->branch[i]));
      CK(cudaStreamWaitEvent(b->cap, b->ev[1 + i], 0));
    }
    if (!deferred.empty()) {
      CK(cudaStreamWaitEvent(b->multiBranch, b->ev[0], 0));
      // groups of one instantiation, at most kPlainMulti handles each
      std::vector<bool> done(deferred.size(), false);
      for (size_t i = 0; i < deferred.size(); i++) {
        if (done[i]) continue;
        std::vector<size_t> grp;
        for (size_t j = i; j < deferred.size() && grp.size() < (size_t)kPlainMulti; j++)
          if (!done[j] && deferred[j].h->entry == deferred[i].h->entry && deferred[j].h->smem == deferred[i].h->smem)
            grp.push_back(j);
        int smem = 0, numSMs = deferred[i].h->numSMs;
        for (size_t j : grp) {
          done[j] = true;
          smem = std::max(smem, deferred[j].h->smem);
        }
        int ctas = 0;
        CK(deferred[i].h->entry->occupancy_multi(&ctas, smem));
        if (ctas < 1) return fail(SHWFS_ERR_UNSUPPORTED, "multi-handle kernel cannot be resident");
        // each handle gets the CTAs a launch of its own would have (the
        // block scheduler then balances the union as it balances
        // concurrent launches)
        const long long perHandle = (long long)numSMs * ctas;
        PlainMulti m{};
        m.n = (int)grp.size();
        m.ctaStart[0] = 0;
        for (size_t k = 0; k < grp.size(); k++) {
          const long long t = deferred[grp[k]].ntiles;
          const long long c = std::max<long long>(1, std::min<long long>(t, perHandle));
          m.a[k] = deferred[grp[k]].a;
          m.ctaStart[k + 1] = m.ctaStart[k] + (int)c;
        }
        CK(deferred[i].h->entry->launch_multi(m, smem, b->multiBranch));
        b->multiLaunches++;
      }
      CK(cudaEventRecord(b->multiJoin, b->multiBranch));
      CK(cudaStreamWaitEvent(b->cap, b->multiJoin, 0));
    }
    CK(launch_bump_counters(b->d_ctrs.p, (int)b->hs.size(), b->cap));
    return SHWFS_OK;
  };
  const shwfs_status s = body();
  for (shwfs_handle* h : b->hs) h->plainSink = nullptr;
  const std::string err = g_err;
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->cap, &g);
  if (s) {
    if (g) cudaGraphDestroy(g);
    g_err = err;
    return s;
  }
  if (e != cudaSuccess) return fail(SHWFS_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
  b->graph = g;
  CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
  for (size_t i = 0; i < b->hs.size(); i++) b->versions[i] = b->hs[i]->version;
  return SHWFS_OK;
}

shwfs_status batch_check(const shwfs_handle* h) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle in batch");
  if (h->noiseMode == SHWFS_NOISE_REFERENCE)
    return fail(SHWFS_ERR_UNSUPPORTED, "batches need the counter-based noise streams");
  if (is_none(h->phs) || !h->phs.on_device || !h->cents.on_device || !h->bimg.on_device)
    return fail(SHWFS_ERR_INVALID, "batched handles need device-resident phs, cents and bimg");
  return SHWFS_OK;
}

}  // namespace

extern "C" {

shwfs_status shwfs_batch_create(shwfs_handle* const* handles, int n, shwfs_batch** out) {
  if (!handles || !out || n < 1) return fail(SHWFS_ERR_INVALID, "bad batch arguments");
  *out = nullptr;
  g_err.clear();
  for (int i = 0; i < n; i++) {
    if (shwfs_status s = batch_check(handles[i])) return s;
    if (handles[i]->device != handles[0]->device) return fail(SHWFS_ERR_INVALID, "batched handles share one device");
    for (int j = 0; j < i; j++)
      if (handles[j] == handles[i]) return fail(SHWFS_ERR_INVALID, "handle %d appears twice in the batch", i);
  }
  shwfs_batch* b = new shwfs_batch;
  b->device = handles[0]->device;
  auto init = [&]() -> shwfs_status {
    CK(cudaSetDevice(b->device));
    CK(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
    std::vector<unsigned long long*> ptrs;
    for (int i = 0; i < n; i++) {
      shwfs_handle* h = handles[i];
      b->hs.push_back(h);
      if (!h->d_frameCtr.p) CK(h->d_frameCtr.alloc(1));
      const unsigned long long f0 = h->framesRead;
      CK(cudaMemcpy(h->d_frameCtr.p, &f0, sizeof(f0), cudaMemcpyHostToDevice));
      b->ctrFrames.push_back(h->framesRead);
      b->versions.push_back(h->version);
      ptrs.push_back(h->d_frameCtr.p);
      cudaStream_t s = nullptr;
      CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
      b->branch.push_back(s);
    }
    for (int i = 0; i <= n; i++) {
      cudaEvent_t e = nullptr;
      CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      b->ev.push_back(e);
    }
    CK(cudaStreamCreateWithFlags(&b->multiBranch, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&b->multiJoin, cudaEventDisableTiming));
    CK(b->d_ctrs.upload(ptrs.data(), ptrs.size()));
    return batch_capture(b);
  };
  if (shwfs_status s = init()) {
    const std::string err = g_err;
    delete b;
    g_err = err;
    return s;
  }
  *out = b;
  return SHWFS_OK;
}

shwfs_status shwfs_batch_set_multi(shwfs_batch* b, int on) {
  if (!b) return fail(SHWFS_ERR_INVALID, "null batch");
  CK(cudaSetDevice(b->device));
  if (b->multiEnabled == (on != 0)) return SHWFS_OK;
  CK(cudaStreamSynchronize(b->cap));
  b->multiEnabled = on != 0;
  const shwfs_status s = batch_capture(b);
  if (s) {
    // keep a usable graph: back to the previous setting
    const std::string err = g_err;
    b->multiEnabled = !b->multiEnabled;
    batch_capture(b);
    g_err = err;
  }
  return s;
}

shwfs_status shwfs_batch_multi_launches(const shwfs_batch* b, int* n) {
  if (!b || !n) return fail(SHWFS_ERR_INVALID, "null batch or output");
  *n = b->multiLaunches;
  return SHWFS_OK;
}

shwfs_status shwfs_batch_run(shwfs_batch* b, void* stream) {
  if (!b) return fail(SHWFS_ERR_INVALID, "null batch");
  CK(cudaSetDevice(b->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : b->cap;
  // no graph after a failed re-capture: capture again before launching
  bool stale = b->exec == nullptr;
  for (size_t i = 0; i < b->hs.size(); i++) {
    if (shwfs_status s = batch_check(b->hs[i])) return s;
    stale |= b->versions[i] != b->hs[i]->version;
  }
  if (stale)
    if (shwfs_status s = batch_capture(b)) return s;
  // a handle run on its own since the last replay advanced its host frame
  // index: bring the device counter to it, in stream order
  for (size_t i = 0; i < b->hs.size(); i++) {
    shwfs_handle* h = b->hs[i];
    if (b->ctrFrames[i] != h->framesRead) CK(launch_set_counter(h->d_frameCtr.p, h->framesRead, st));
  }
  CK(cudaGraphLaunch(b->exec, st));
  for (size_t i = 0; i < b->hs.size(); i++) {
    b->hs[i]->framesRead++;
    b->ctrFrames[i] = b->hs[i]->framesRead;
  }
  if (!stream) {
    // the tensor-core forms' noise/centroid kernels wrote each status word
    // to its pinned host copy
    CK(cudaStreamSynchronize(st));
    for (shwfs_handle* h : b->hs) {
      if (!gemm_active(h)) continue;
      const int status = *(volatile int*)h->h_status;
      if (status & 2) return fail(SHWFS_ERR_STATE, "tensor-core pipeline wait timed out (results invalid)");
    }
  }
  return SHWFS_OK;
}

shwfs_status shwfs_sample_noise(int kind, const float* lam, int64_t n, uint64_t seed, uint64_t frame, float* out,
                                void* stream) {
  if (n < 0 || n > (1LL << 32) || !out || (kind != 1 && !lam) || kind < 0 || kind > 2)
    return fail(SHWFS_ERR_INVALID, "bad noise-sampling arguments");
  cudaStream_t st = (cudaStream_t)stream;
  CK(launch_sample_noise(lam, n, seed, frame, kind, out, st));
  if (!stream) CK(cudaStreamSynchronize(st));
  return SHWFS_OK;
}

shwfs_status shwfs_selftest_bounded_wait(int64_t max_cycles, int* timed_out, int* abort_raised) {
  if (!timed_out || !abort_raised || max_cycles <= 0 || max_cycles > (int64_t)1 << 36)
    return fail(SHWFS_ERR_INVALID, "bad self-test arguments");
  DevBuf<int> out;
  CK(out.alloc(3));
  CK(cudaMemset(out.p, 0, 3 * sizeof(int)));
  CK(launch_bounded_wait_selftest((long long)max_cycles, out.p, 0));
  CK(cudaDeviceSynchronize());
  int h[3];
  CK(cudaMemcpy(h, out.p, sizeof(h), cudaMemcpyDeviceToHost));
  *timed_out = h[0];
  *abort_raised = h[1];
  return SHWFS_OK;
}

shwfs_status shwfs_batch_free(shwfs_batch* b) {
  delete b;
  return SHWFS_OK;
}

shwfs_status shwfs_set_split_event(shwfs_handle* h, void* event) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  h->splitEvent = (cudaEvent_t)event;
  h->version++;
  return SHWFS_OK;
}

shwfs_status autotune_gemm(shwfs_handle* h);

shwfs_status shwfs_autotune(shwfs_handle* h, int* best_tile) {
  if (!h) return fail(SHWFS_ERR_INVALID, "null handle");
  g_err.clear();
  CK(cudaSetDevice(h->device));
  if (!h->lit.empty() && !is_none(h->phs) && gemm_active(h)) {
    shwfs_status s = autotune_gemm(h);
    if (best_tile) *best_tile = h->TS;
    return s;
  }
  if (h->lit.empty() || is_none(h->phs) || h->noiseMode == SHWFS_NOISE_REFERENCE) {
    // nothing to choose: no phase-input launches on this handle
    if (best_tile) *best_tile = h->TS;
    return SHWFS_OK;
  }
  if (shwfs_status s = prepare_readout(h)) return s;
  const int nlit = (int)h->lit.size();
  const size_t mm = (size_t)h->nimg * h->nimg;
  // enough frames that every candidate fills the GPU several times over
  const int nf = (int)std::max<long long>(1, std::min<long long>(64, (16LL * 64 * h->numSMs + nlit - 1) / nlit));
  DevBuf<float> ph, ce, bi;
  const float* phs = (const float*)h->phs.data;
  if (!h->phs.on_device) {
    CK(ph.upload(phs, (size_t)numel(h->phs)));
    phs = ph.p;
  }
  CK(ce.alloc((size_t)nf * h->nsubaps * 2));
  CK(bi.alloc((size_t)nf * h->nsubaps * mm));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int saved = h->tileOverride;
  const int cands[] = {0, 4, 6, 8, 10, 12, 14, 16, 20, 24, 32};
  float bestMs = 1e30f;
  int bestOverride = saved;
  shwfs_status s = SHWFS_OK;
  for (int c : cands) {
    h->tileOverride = c;
    if (plan(h) != SHWFS_OK) continue;
    float ms = 0.f;
    for (int rep = 0; rep < 2 && !s; rep++) {  // rep 0 warms up
      if (cudaEventRecord(e0, h->stream) != cudaSuccess) s = fail(SHWFS_ERR_CUDA, "event record failed");
      for (int k = 0; k < 3 && !s; k++) s = enqueue_readout(h, phs, ce.p, bi.p, nf, 0, h->stream);
      if (!s && cudaEventRecord(e1, h->stream) != cudaSuccess) s = fail(SHWFS_ERR_CUDA, "event record failed");
      if (!s && cudaEventSynchronize(e1) != cudaSuccess) s = fail(SHWFS_ERR_CUDA, "autotune launch failed");
      if (!s) cudaEventElapsedTime(&ms, e0, e1);
    }
    if (s) break;
    if (ms < bestMs) {
      bestMs = ms;
      bestOverride = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->tileOverride = s ? saved : bestOverride;
  h->version++;
  const std::string err = g_err;
  const shwfs_status sp = plan(h);
  if (s) {
    g_err = err;
    return s;
  }
  if (sp) return sp;
  if (best_tile) *best_tile = h->TS;
  return SHWFS_OK;
}

shwfs_status shwfs_gemm_stagings(int form, int phasesize, int crop, int nimg, int* rows, int cap, int* n) {
  if (!n || cap < 0 || (cap > 0 && !rows) || phasesize < 1 || crop < 1 || nimg < 1 || form < SHWFS_FORM_BF16 ||
      form > SHWFS_FORM_TF32)
    return fail(SHWFS_ERR_INVALID, "bad staging query arguments");
  g_err.clear();
  // the geometry depends on the phase, crop and image sizes only
  GemmSpec sp{};
  sp.p = phasesize;
  sp.c = crop;
  sp.m = nimg;
  const std::vector<GemmGeom> cands = gemm_geometry_candidates(sp, form_fmt(form), form_passes(form));
  *n = (int)cands.size();
  for (int i = 0; i < cap && i < (int)cands.size(); i++) {
    const GemmGeom& g = cands[i];
    int* r = rows + (size_t)i * SHWFS_STAGING_FIELDS;
    uint32_t tmem = gemm_d2_col(g) + (uint32_t)g.N2;
    for (int b = 0; b < g.nd1; b++) tmem = std::max(tmem, gemm_d1_col(g, b) + 2u * (uint32_t)g.CW);
    r[SHWFS_STG_CW] = g.CW;
    r[SHWFS_STG_NOC] = g.noc;
    r[SHWFS_STG_KCB] = g.KCB;
    r[SHWFS_STG_NKC] = g.nkc;
    r[SHWFS_STG_DBE] = g.dbE;
    r[SHWFS_STG_DBA2] = g.dbA2;
    r[SHWFS_STG_NK] = g.NK;
    r[SHWFS_STG_NW] = g.NW;
    r[SHWFS_STG_ND1] = g.nd1;
    r[SHWFS_STG_K1] = g.K1;
    r[SHWFS_STG_N2] = g.N2;
    r[SHWFS_STG_SMEM] = gemm_smem_bytes(g);
    r[SHWFS_STG_TMEM] = (int)tmem;
  }
  return SHWFS_OK;
}

// tensor-core forms: time every staging of the GEMM kernel that fits
// (gemm_geometry_candidates) on this handle's own phase and keep the fastest
// with its constants.  The MMAs see the same k-steps in the same order
// whatever the staging, so the results do not change.
shwfs_status autotune_gemm(shwfs_handle* h) {
  GemmSpec sp;
  GemmGeom g0{};
  if (!gemm_static_ok(h, &g0, &sp)) return SHWFS_OK;
  const std::vector<GemmGeom> cands = gemm_geometry_candidates(sp, g0.fmt, g0.passes);
  if (cands.size() < 2) return SHWFS_OK;
  if (shwfs_status s = prepare_readout(h)) return s;
  const int nlit = (int)h->lit.size();
  const size_t mm = (size_t)h->nimg * h->nimg;
  const int nf = (int)std::max<long long>(1, std::min<long long>(64, (16LL * 128 * h->numSMs + nlit - 1) / nlit));
  DevBuf<float> ph, ce, bi;
  const float* phs = (const float*)h->phs.data;
  if (!h->phs.on_device) {
    CK(ph.upload(phs, (size_t)numel(h->phs)));
    phs = ph.p;
  }
  CK(ce.alloc((size_t)nf * h->nsubaps * 2));
  CK(bi.alloc((size_t)nf * h->nsubaps * mm));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const GemmGeom saved = h->gemm;
  float bestMs = 1e30f;
  size_t best = 0;
  shwfs_status s = SHWFS_OK;
  for (size_t c = 0; c < cands.size() && !s; c++) {
    if ((s = upload_gemm_consts(h, sp, cands[c]))) break;
    h->gemm = cands[c];
    float ms = 0.f;
    for (int rep = 0; rep < 2 && !s; rep++) {  // rep 0 warms up
      if (cudaEventRecord(e0, h->stream) != cudaSuccess) s = fail(SHWFS_ERR_CUDA, "event record failed");
      for (int k = 0; k < 3 && !s; k++) s = enqueue_readout(h, phs, ce.p, bi.p, nf, 0, h->stream);
      if (!s && cudaEventRecord(e1, h->stream) != cudaSuccess) s = fail(SHWFS_ERR_CUDA, "event record failed");
      if (!s && cudaEventSynchronize(e1) != cudaSuccess) s = fail(SHWFS_ERR_CUDA, "autotune launch failed");
      if (!s) cudaEventElapsedTime(&ms, e0, e1);
    }
    if (!s && ms < bestMs) {
      bestMs = ms;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const std::string err = g_err;
  const GemmGeom keep = s ? saved : cands[best];
  if (!s) h->gemmStaging = (int)best;
  const shwfs_status su = upload_gemm_consts(h, sp, keep);
  h->gemm = keep;
  h->version++;
  if (s) {
    g_err = err;
    return s;
  }
  return su;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// hooks for the native runtime (engine_internal.h)
// ---------------------------------------------------------------------------
namespace shwfs {

shwfs_status engine_frame(shwfs_handle* h, const float* phs_dev, cudaStream_t st, int* readout) {
  *readout = readout_frame(h);
  if (h->integMode == SHWFS_INTEG_PHYSICAL) {
    const int state = integ_state(h);
    if (state != 3) {
      if (!h->cents.on_device || !h->bimg.on_device)
        return fail(SHWFS_ERR_STATE, "engine_frame needs device-resident cents and bimg");
      if (shwfs_status s = enqueue_physical(h, phs_dev, state, st)) return s;
    }
    if (*readout) h->framesRead++;
  } else if (*readout) {
    if (!h->cents.on_device || !h->bimg.on_device)
      return fail(SHWFS_ERR_STATE, "engine_frame needs device-resident cents and bimg");
    if (shwfs_status s = enqueue_readout(h, phs_dev, (float*)h->cents.data, (float*)h->bimg.data, 1, 0, st))
      return s;
    h->framesRead++;
  }
  h->curInteg++;
  if (h->curInteg >= h->nintegrations + h->nlatency) h->curInteg = 0;
  return SHWFS_OK;
}

int64_t engine_device_bytes(const shwfs_handle* h) {
  int64_t b = 0;
  auto add = [&](const auto& buf) { b += (int64_t)buf.n * (int64_t)sizeof(*buf.p); };
  add(h->d_pup); add(h->d_tilt); add(h->d_frac); add(h->d_totsig); add(h->d_sigArr); add(h->d_skyArr);
  add(h->d_cw); add(h->d_ref); add(h->d_calData); add(h->d_calSteps); add(h->d_calCoeff); add(h->d_fitMx);
  add(h->d_binT); add(h->d_binN); add(h->d_psf); add(h->d_lit); add(h->d_unlit); add(h->d_binII);
  add(h->d_binLo); add(h->d_binHi); add(h->d_ubArr); add(h->d_calBounds); add(h->d_subflag);
  add(h->d_subapStart); add(h->d_status); add(h->d_psfSpec); add(h->d_phs); add(h->d_cents); add(h->d_bimg);
  add(h->d_sub); add(h->d_accum); add(h->d_inj);
  add(h->d_image); add(h->d_subapLoc); add(h->d_poisFlag); add(h->d_rng); add(h->d_w2); add(h->d_kc2);
  add(h->d_iscale); add(h->d_pupT); add(h->d_interp); add(h->d_frameCtr);
  return b;
}

const int* engine_status_ptr(const shwfs_handle* h) { return h->d_status.p; }
int engine_nsubaps(const shwfs_handle* h) { return h->nsubaps; }
shwfs_status engine_fail(shwfs_status st, const char* msg) { return fail(st, "%s", msg); }

}  // namespace shwfs
