// Device copy of the Poisson CDF tables used by the tabulated sampler
// (poisson_tab in shwfs_dev.cuh), built on the host in double precision once
// per device.
#include <cuda_runtime.h>
#include <string.h>

#include <cmath>
#include <mutex>
#include <set>
#include <vector>

#include "shwfs_dev.cuh"

namespace shwfs {

__device__ PoisTab g_poistab;

namespace {

bool build_host_table(PoisTab* t) {
  memset(t, 0, sizeof(*t));
  int pos = 0;
  t->off[0] = 0;
  t->len[0] = 1;
  t->cdf[pos++] = 1.0f;  // Poisson(0) = 0
  for (int L = 1; L < kPoisTabL; L++) {
    std::vector<float> C;
    double p = std::exp(-(double)L), c = p;
    C.push_back((float)c);
    for (int k = 1; 1.0 - c > 9.3e-10 && k < 400; k++) {  // tail below 2^-30
      p *= (double)L / k;
      c += p;
      C.push_back((float)(c < 1.0 ? c : 1.0));
    }
    if (C.back() < 1.0f) C.push_back(1.0f);  // the search always ends inside the table
    if (pos + (int)C.size() > kPoisCdfMax) return false;
    t->off[L] = (uint16_t)pos;
    t->len[L] = (uint16_t)C.size();
    for (float v : C) t->cdf[pos++] = v;
    for (int j = 0; j < kPoisGuide; j++) {
      const float target = (float)j / (float)kPoisGuide;
      int k = 0;
      while (k < (int)C.size() - 1 && C[k] < target) k++;
      t->guide[L][j] = (uint8_t)k;
    }
  }
  return true;
}

std::mutex g_mu;
std::set<int> g_ready;

}  // namespace

cudaError_t pois_table_device(const PoisTab** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ready.count(dev)) {
    static PoisTab host;
    static bool built = false;
    if (!built) {
      if (!build_host_table(&host)) return cudaErrorInvalidValue;
      built = true;
    }
    e = cudaMemcpyToSymbol(g_poistab, &host, sizeof(host));
    if (e != cudaSuccess) return e;
    g_ready.insert(dev);
  }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_poistab);
  if (e != cudaSuccess) return e;
  *out = static_cast<const PoisTab*>(p);
  return cudaSuccess;
}

}  // namespace shwfs
