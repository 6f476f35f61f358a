// Centroids from a detector image with no memory allocation at all.
//
// Who needs this: a real-time controller thread that reads a camera frame
// every millisecond or so and must never call cudaMalloc/cudaFree in its
// loop (an allocation can block the whole device while it synchronises), and
// systems whose device memory is entirely owned by another allocator.  Such a
// caller cannot create a shwfs handle (which allocates device copies of its
// configuration), so this entry point takes everything as caller-owned device
// buffers and keeps its only working memory -- the lists of lit and unlit
// subapertures -- in a fixed static device array compiled into the library.
//
// The scratch array is shared by every call on a device and keeps the last
// call's contents; each call rebuilds both lists and their counts from the
// caller's subflag before using them, so nothing has to start at zero.  Two
// calls whose GPU work overlaps (different streams, or different host
// threads) race on the array and must not be issued.  The first call on a
// device looks up the array's device address with that device current (once
// per device); that first call should come before any stream capture.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>

#include "../../include/shwfs.h"
#include "wfs_plain.cuh"

namespace {

// counts[2] followed by the lit list and the unlit list
constexpr int kScratchInts = 2 + 2 * SHWFS_NOALLOC_MAX_SUBAPS;
static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
int* g_scratch_ptr[kMaxDevices];  // device address of g_noalloc_scratch per device

// copy a message into the caller's buffer (if any) and return the status
shwfs_status report(char* err, size_t errlen, shwfs_status st, const char* msg) {
  if (err && errlen) {
    strncpy(err, msg, errlen - 1);
    err[errlen - 1] = 0;
  }
  return st;
}

// Ordered split of subflag into lit / unlit index lists (one CTA): every
// thread counts its contiguous chunk, a block scan gives the offsets, then
// each thread writes its indices in order.  Writes both counts.
__global__ void split_subaps_kernel(const int* __restrict__ subflag, int n, int* scratch) {
  __shared__ int s_lit[1024];
  __shared__ int s_unlit[1024];
  const int t = threadIdx.x, nt = blockDim.x;
  const int chunk = (n + nt - 1) / nt;
  const int lo = min(n, t * chunk), hi = min(n, lo + chunk);
  int nl = 0;
  for (int i = lo; i < hi; i++) nl += subflag[i] == 1;
  s_lit[t] = nl;
  s_unlit[t] = (hi - lo) - nl;
  __syncthreads();
  // inclusive scans (Hillis-Steele)
  for (int off = 1; off < nt; off <<= 1) {
    int a = t >= off ? s_lit[t - off] : 0;
    int b = t >= off ? s_unlit[t - off] : 0;
    __syncthreads();
    s_lit[t] += a;
    s_unlit[t] += b;
    __syncthreads();
  }
  int* lit = scratch + 2;
  int* unlit = scratch + 2 + SHWFS_NOALLOC_MAX_SUBAPS;
  int pl = s_lit[t] - nl, pu = s_unlit[t] - ((hi - lo) - nl);
  for (int i = lo; i < hi; i++) {
    if (subflag[i] == 1)
      lit[pl++] = i;
    else
      unlit[pu++] = i;
  }
  if (t == nt - 1) {
    scratch[0] = s_lit[t];
    scratch[1] = s_unlit[t];
  }
}

}  // namespace

extern "C" shwfs_status shwfs_image_centroids_noalloc(const shwfs_image_job* job, void* stream, char* err,
                                                      size_t errlen) {
  if (err && errlen) err[0] = 0;
  if (!job) return report(err, errlen, SHWFS_ERR_INVALID, "null job");
  const int nsubx = job->nsubx, m = job->nimg;
  if (nsubx < 1 || m < 1) return report(err, errlen, SHWFS_ERR_INVALID, "nsubx and nimg must be positive");
  const long long nsub = (long long)nsubx * nsubx;
  if (nsub > SHWFS_NOALLOC_MAX_SUBAPS)
    return report(err, errlen, SHWFS_ERR_INVALID,
                        "too many subapertures for the allocation-free call: at most SHWFS_NOALLOC_MAX_SUBAPS "
                        "(65536, i.e. 256x256)");
  if (job->ncen < 1 || job->ncen > m) return report(err, errlen, SHWFS_ERR_INVALID, "ncen must be in [1, nimg]");
  if (!job->image || !job->subflag || !job->cents || !job->bimg)
    return report(err, errlen, SHWFS_ERR_INVALID, "image, subflag, cents and bimg must be device pointers");
  int npxlx;
  if (job->image_ndim == 2) {
    if (job->image_rows < (long long)nsubx * m || job->image_cols < (long long)nsubx * m)
      return report(err, errlen, SHWFS_ERR_INVALID, "2-D image smaller than nsubx*nimg in a dimension");
    npxlx = (int)job->image_cols;
  } else if (job->image_ndim == 4) {
    npxlx = m;
  } else {
    return report(err, errlen, SHWFS_ERR_INVALID, "image_ndim must be 2 or 4");
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return report(err, errlen, SHWFS_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return report(err, errlen, SHWFS_ERR_UNSUPPORTED, "device ordinal out of range");
  {
    // once per device, with that device current: the device address of the
    // static scratch array (host code cannot use the symbol itself)
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) return report(err, errlen, SHWFS_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
      g_scratch_ptr[dev] = (int*)p;
    }
  }
  int* scratch = g_scratch_ptr[dev];
  cudaStream_t st = (cudaStream_t)stream;
  split_subaps_kernel<<<1, 1024, 0, st>>>(job->subflag, (int)nsub, scratch);
  if ((e = cudaGetLastError()) != cudaSuccess) return report(err, errlen, SHWFS_ERR_CUDA, cudaGetErrorString(e));
  int counts[2] = {0, 0};
  if ((e = cudaMemcpyAsync(counts, scratch, sizeof(counts), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return report(err, errlen, SHWFS_ERR_CUDA, cudaGetErrorString(e));
  int numSMs = 1;
  cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev);

  shwfs::WfsArgs a;
  memset(&a, 0, sizeof(a));
  a.nsubx = nsubx;
  a.nsubaps = (int)nsub;
  a.m = m;
  a.ncen = job->ncen;
  a.nframes = 1;
  a.TS = m * m <= 4096 ? (4096 / (m * m) < 64 ? 4096 / (m * m) : 64) : 1;
  a.floorv = job->noiseFloor;
  a.threshType = job->threshType;
  a.calsource = job->calsource;
  a.useBrightest = job->useBrightest;
  a.pxlPower = job->pxlPower;
  a.imageOnly = job->imageOnly;
  a.readNoise = job->readNoise;
  a.readBg = job->readBg;
  a.seed = job->seed;
  set_philox_keys(a);
  a.frame0 = job->frame;
  a.refCents = job->refCents;
  a.cents = job->cents;
  a.centsFrameStride = nsub * 2;
  a.bimg = job->bimg;
  a.bimgFrameStride = nsub * m * m;
  if (counts[0] > 0) {
    a.lit = scratch + 2;
    a.nlit = counts[0];
    e = shwfs::launch_image(a, job->image, job->image_ndim, npxlx, nullptr, numSMs, st);
    if (e != cudaSuccess) return report(err, errlen, SHWFS_ERR_CUDA, cudaGetErrorString(e));
  }
  if (counts[1] > 0) {
    e = shwfs::launch_unlit(a, scratch + 2 + SHWFS_NOALLOC_MAX_SUBAPS, counts[1], st);
    if (e != cudaSuccess) return report(err, errlen, SHWFS_ERR_CUDA, cudaGetErrorString(e));
  }
  return SHWFS_OK;
}
