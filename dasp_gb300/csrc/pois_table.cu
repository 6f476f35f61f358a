// Device copy of the Poisson alias tables used by the tabulated sampler
// (poisson_tab in shwfs_dev.cuh), built on the host in double precision once
// per device.
#include <cuda_runtime.h>
#include <string.h>

#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>
#include <set>
#include <vector>

#include "shwfs_dev.cuh"

namespace shwfs {

__device__ PoisTab g_poistab;

namespace {

// keep threshold of a column kept with probability q: the 32-bit coin keeps
// the column when it is below round(q 2^32) (q = 1: always, up to 2^-32)
uint32_t keep32(double q) {
  if (q >= 1.0) return 0xffffffffu;
  if (q <= 0.0) return 0u;
  const double t = std::floor(q * 4294967296.0 + 0.5);
  return t >= 4294967295.0 ? 0xffffffffu : (uint32_t)t;
}

// Walker/Vose alias table of Poisson(L) over 0..n-1 into prob/alias[o..o+n)
void alias_table(const std::vector<double>& P, uint32_t* prob, uint8_t* alias) {
  const int n = (int)P.size();
  std::vector<double> q(n);
  std::vector<int> small, large;
  for (int k = 0; k < n; k++) {
    q[k] = P[k] * n;
    (q[k] < 1.0 ? small : large).push_back(k);
  }
  for (int k = 0; k < n; k++) {
    prob[k] = 0xffffffffu;
    alias[k] = (uint8_t)k;
  }
  while (!small.empty() && !large.empty()) {
    const int l = small.back(), g = large.back();
    small.pop_back();
    large.pop_back();
    prob[l] = keep32(q[l]);
    alias[l] = (uint8_t)g;
    q[g] = (q[g] + q[l]) - 1.0;
    (q[g] < 1.0 ? small : large).push_back(g);
  }
  // what is left has q = 1 up to rounding: keeps its own column
}

bool build_host_table(PoisTab* t) {
  memset(t, 0, sizeof(*t));
  int pos = 0;
  t->offlen[0] = 1u;  // entry 0, one column: Poisson(0) = 0
  t->prob[pos] = 0xffffffffu;
  t->alias[pos++] = 0;
  for (int L = 1; L < kPoisTabL; L++) {
    std::vector<double> P;
    double p = std::exp(-(double)L), c = p;
    P.push_back(p);
    for (int k = 1; 1.0 - c > 9.3e-10 && k < 255; k++) {  // upper tail below 2^-30
      p *= (double)L / k;
      c += p;
      P.push_back(p);
    }
    P.back() += 1.0 - c;  // the last entry takes the remaining mass
    if (pos + (int)P.size() > kPoisCdfMax || P.size() > 255) return false;
    t->offlen[L] = ((uint32_t)pos << 8) | (uint32_t)P.size();
    alias_table(P, t->prob + pos, t->alias + pos);
    pos += (int)P.size();
  }
  return true;
}

std::mutex g_mu;
std::map<int, const PoisTab*> g_ready;  // device -> table address

std::mutex g_launch_mu;
std::map<std::pair<int, const void*>, int> g_smemAttr;           // (device, kernel) -> its dynamic smem limit
std::map<std::tuple<int, const void*, int, int>, int> g_occupancy;  // (device, kernel, smem, threads) -> CTAs/SM

}  // namespace

cudaError_t pois_table_device(const PoisTab** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_ready.find(dev);
  if (it == g_ready.end()) {
    static PoisTab host;
    static bool built = false;
    if (!built) {
      if (!build_host_table(&host)) return cudaErrorInvalidValue;
      built = true;
    }
    e = cudaMemcpyToSymbol(g_poistab, &host, sizeof(host));
    if (e != cudaSuccess) return e;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_poistab);
    if (e != cudaSuccess) return e;
    it = g_ready.emplace(dev, static_cast<const PoisTab*>(p)).first;
  }
  *out = it->second;
  return cudaSuccess;
}

cudaError_t kernel_smem_setup(const void* kern, int smem, int threads, int* ctasPerSM) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_launch_mu);
  // the limit is a property of the kernel: only ever raised, so a launch
  // with less shared memory than an earlier one never lowers it under a
  // later, larger launch
  auto at = g_smemAttr.find(std::make_pair(dev, kern));
  if (at == g_smemAttr.end() || at->second < smem) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    g_smemAttr[std::make_pair(dev, kern)] = smem;
  }
  if (!ctasPerSM) return cudaSuccess;
  const auto key = std::make_tuple(dev, kern, smem, threads);
  auto it = g_occupancy.find(key);
  if (it == g_occupancy.end()) {
    int ctas = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, kern, threads, (size_t)smem);
    if (e != cudaSuccess) return e;
    it = g_occupancy.emplace(key, ctas).first;
  }
  *ctasPerSM = it->second;
  return cudaSuccess;
}

}  // namespace shwfs
