// Reference-stream noise state and launcher (see wfs_refnoise.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace shwfs {

constexpr int kMtN = 624, kMtM = 397;

// one reference worker thread's generators: PCG32 (Poisson) + MT19937 (read noise)
struct RefRng {
  uint64_t pcg_state, pcg_inc;
  uint32_t mt[kMtN];
  int mti;
  int pad;
};

struct RefNoiseArgs {
  int nthreads;
  const int* subapStart;  // nthreads + 1
  const int* subflag;
  const unsigned char* poisFlag;
  float* bimg;
  int m, nexp;
  float readNoise, readBg, floorv;
  int threshType, addPoisson, calsource, imageOnly;
  int imageInput;  // 1: runSlope frame -- lit subapertures draw nothing
};

// host-side seeding: pcg32_srandom_r(seed_t, 1) and gsl_rng_set(mt, seed_t)
// (cmod/src/centmodule.c:91-98, 2556-2562)
inline void seed_ref_rng(RefRng* r, uint64_t seed_t) {
  auto next = [r]() {
    uint64_t old = r->pcg_state;
    r->pcg_state = old * 6364136223846793005ULL + r->pcg_inc;
  };
  r->pcg_state = 0u;
  r->pcg_inc = (1ull << 1u) | 1u;
  next();
  r->pcg_state += seed_t;
  next();
  uint64_t s = seed_t;
  if (s == 0) s = 4357;
  r->mt[0] = (uint32_t)(s & 0xffffffffULL);
  for (int i = 1; i < kMtN; i++) r->mt[i] = (uint32_t)(1812433253UL * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + i);
  r->mti = kMtN;
  r->pad = 0;
}

cudaError_t launch_refnoise(const RefNoiseArgs& a, RefRng* rng, int* status, cudaStream_t stream);

// Poisson flag of every subaperture for frames whose pre-noise images come
// from the caller: the reference poissonises subaperture i only when
// totsig > 0, sky * fracSubArea > 0 or a sky array is set
// (cmod/src/centmodule.c:1879), here from the handle's totals.
cudaError_t launch_pois_flag(int nsubaps, const float* totsig, const float* frac, float sky, int skyArr,
                             unsigned char* poisFlag, cudaStream_t stream);

// Noise from caller-drawn values: shot[k] replaces the Poisson draw of pixel
// k where the reference poissonises, readn[k] replaces (float)gsl_ran_gaussian
// where readCCD draws (readNoise != 0 and no calibration source), then
// readCCD's background and threshold (cmod/src/centmodule.c:785-817,
// 1879-1881); unlit subapertures with imageOnly get readCCD of a zero image
// (:1972-1976).  Either array may be null where the configuration draws
// nothing from it.
struct InjectArgs {
  int nsubaps, m;
  const int* subflag;
  const unsigned char* poisFlag;
  float* bimg;
  const float* shot;
  const float* readn;
  float readNoise, readBg, floorv;
  int threshType, addPoisson, calsource, imageOnly;
};
cudaError_t launch_inject_noise(const InjectArgs& a, cudaStream_t stream);

}  // namespace shwfs
