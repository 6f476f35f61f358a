// Infinite phase screen resident on the device (science/infScrn.py
// addNewColumnOnEnd :747-791, addNewRowOnEnd :825-855, addNewColumnOnStart
// :793-823, addNewRowOnStart :857-887): each new column (row) is
// A Z + coeff B n + step, Z the last two columns (rows) stacked oldest first,
// n standard normals; A and B come from the host in float64.  At the start
// of the screen the reference uses AStart, A with its two column blocks in
// reverse order (:722-731), on the first two lines stacked first line first:
// that is A applied with the second line in A's first block and the edge
// line in its second, which is how the kernel pairs them.
// The screen is a circular buffer in both axes: logical (y, x) lives at
// ((rs + y) % ny, (cs + x) % nx), so appending overwrites the oldest column
// (row) in place instead of shifting the screen as the reference does.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/shwfs.h"
#include "engine_internal.h"
#include "shwfs_dev.cuh"

struct shwfs_screen {
  int ny = 0, nx = 0;
  int rs = 0, cs = 0;             // circular starts (rows, columns)
  float* scr = nullptr;           // ny x nx, physical order
  double* a[2] = {nullptr, nullptr};  // [0] columns: ny x 2ny; [1] rows: nx x 2nx
  double* b[2] = {nullptr, nullptr};  // [0] ny x ny; [1] nx x nx
  double* noise = nullptr;        // max(ny, nx)
  shwfs::PhiloxKeys keys{};
  unsigned long long added = 0;   // extrusions so far (the noise stream's frame index)
  cudaStream_t stream = nullptr;
};

namespace shwfs {

namespace {

constexpr int kScrWarps = 8;

// standard normals for one extrusion: element j from the stream of
// (seed, extrusion, j, purpose 3)
__global__ void screen_noise_kernel(PhiloxKeys keys, unsigned long long ext, int n, double* out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    KeyedStream st(keys, ext, j, 0, 3);
    out[j] = (double)normal_counter(st);
  }
}

// one new column (axis 0) or row (axis 1): warp per output element
__global__ void screen_extrude_kernel(float* __restrict__ scr, int ny, int nx, int rs, int cs, int axis, int start,
                                      const double* __restrict__ A, const double* __restrict__ B,
                                      const double* __restrict__ noise, double coeff, double step) {
  const int len = axis == 0 ? ny : nx;  // output length; Z has 2 len entries
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kScrWarps + (threadIdx.x >> 5);
  if (i >= len) return;
  // logical element k of line l of A's block l: at the end, 0 the older of
  // the last two lines and 1 the last; at the start, 0 the second line and
  // 1 the first (the edge)
  auto z = [&](int l, int k) {
    if (axis == 0) {
      const int x = start ? 1 - l : nx - 2 + l;
      return (double)scr[(long long)((rs + k) % ny) * nx + (cs + x) % nx];
    }
    const int y = start ? 1 - l : ny - 2 + l;
    return (double)scr[(long long)((rs + y) % ny) * nx + (cs + k) % nx];
  };
  const double* ar = A + (long long)i * 2 * len;
  const double* br = B + (long long)i * len;
  double az = 0.0, bn = 0.0;
  for (int j = lane; j < 2 * len; j += 32) az += ar[j] * z(j / len, j % len);
  for (int j = lane; j < len; j += 32) bn += br[j] * noise[j];
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    az += __shfl_xor_sync(0xffffffffu, az, o);
    bn += __shfl_xor_sync(0xffffffffu, bn, o);
  }
  if (lane == 0) {
    const double v = az + bn * coeff + step;
    // the new line replaces the one dropped: at the end the first line
    // (physical column cs, row rs), at the start the last
    const int pc = start ? (cs + nx - 1) % nx : cs, pr = start ? (rs + ny - 1) % ny : rs;
    if (axis == 0)
      scr[(long long)((rs + i) % ny) * nx + pc] = (float)v;
    else
      scr[(long long)pr * nx + (cs + i) % nx] = (float)v;
  }
}

__global__ void screen_window_kernel(const float* __restrict__ scr, int ny, int nx, int rs, int cs, int y0, int x0,
                                     int h, int w, float* __restrict__ out, long long stride) {
  const long long total = (long long)h * w;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(k / w), x = (int)(k - (long long)y * w);
    out[(long long)y * stride + x] = scr[(long long)((rs + y0 + y) % ny) * nx + (cs + x0 + x) % nx];
  }
}

// one pupil-phase layer: the window of a screen and its sub-pixel shift
struct LayerWin {
  const float* scr;
  int ny, nx, rs, cs;  // the screen's size and circular starts
  int y0, x0;          // logical top-left of the (npup+1) square window
  float s1, s2, s3, s4;  // bilinear weights (1-x)(1-y), (1-x)y, x(1-y), xy
};
constexpr int kMaxLayers = 16;
// threads per block of both pupil-phase kernels (their reductions assume it)
constexpr int kPupilThreads = 256;
struct LayerSet {
  LayerWin l[kMaxLayers];
  int n;
};

// createPupilPhs (util/atmos.py:678-733) for sources at infinity: each
// layer's window shifted by linearshift (cmod/src/interpmodule.c:1234-1300,
// float products and sums in its order, no contraction) and the layers
// added in order; then (second kernel) the piston over the pupil removed
// and the result multiplied by the pupil and scaled (:818-833)
__global__ void pupil_layers_kernel(const LayerSet L, int npup, float* __restrict__ out,
                                    const float* __restrict__ pfn, double* __restrict__ partial) {
  __shared__ double red[kPupilThreads];
  double acc = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < (long long)npup * npup;
       k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k / npup), j = (int)(k - (long long)i * npup);
    float o = 0.f;
    for (int q = 0; q < L.n; q++) {
      const LayerWin& w = L.l[q];
      auto at = [&](int y, int x) {
        return w.scr[(long long)((w.rs + w.y0 + y) % w.ny) * w.nx + (w.cs + w.x0 + x) % w.nx];
      };
      float f = __fmul_rn(at(i, j), w.s1);
      f = __fadd_rn(f, __fmul_rn(at(i + 1, j), w.s2));
      f = __fadd_rn(f, __fmul_rn(at(i, j + 1), w.s3));
      f = __fadd_rn(f, __fmul_rn(at(i + 1, j + 1), w.s4));
      o = __fadd_rn(o, f);
    }
    out[k] = o;
    acc += (double)o * (double)pfn[k];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int st = blockDim.x / 2; st; st >>= 1) {
    if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void pupil_finish_kernel(float* __restrict__ out, const float* __restrict__ pfn, long long n,
                                    const double* __restrict__ partial, int nparts, double area, int removePiston,
                                    float scale) {
  // every block reduces the partial sums in the same order (a strided sum
  // per thread, then a tree), so all blocks subtract the same piston
  __shared__ double red[kPupilThreads];
  __shared__ float pist;
  double s = 0.0;
  for (int b = threadIdx.x; b < nparts; b += kPupilThreads) s += partial[b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = kPupilThreads / 2; st; st >>= 1) {
    if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) pist = removePiston ? (float)(red[0] / area) : 0.f;
  __syncthreads();
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    out[k] = __fmul_rn(__fmul_rn(__fsub_rn(out[k], pist), pfn[k]), scale);
}

}  // namespace

}  // namespace shwfs

using shwfs::engine_fail;

namespace {

shwfs_status cuda_fail(cudaError_t e, const char* what) {
  return engine_fail(SHWFS_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
}

#define SCK(call, what)                          \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

template <typename T>
cudaError_t upload(T** dst, const T* src, size_t n) {
  cudaError_t e = cudaMalloc((void**)dst, n * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

void release(shwfs_screen* s) {
  cudaFree(s->scr);
  for (int k = 0; k < 2; k++) {
    cudaFree(s->a[k]);
    cudaFree(s->b[k]);
  }
  cudaFree(s->noise);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

}  // namespace

extern "C" {

shwfs_status shwfs_screen_create(int ny, int nx, const float* init, const double* ay, const double* by,
                                 const double* ax, const double* bx, uint64_t seed, shwfs_screen** out) {
  if (!out || !init || ny < 3 || nx < 3 || (int64_t)ny * nx > ((int64_t)1 << 30))
    return engine_fail(SHWFS_ERR_INVALID, "screen_create: bad size or null argument");
  if (!ay && !ax) return engine_fail(SHWFS_ERR_INVALID, "screen_create: give the column and/or row matrices");
  if ((ay && !by) || (ax && !bx)) return engine_fail(SHWFS_ERR_INVALID, "screen_create: A without B");
  shwfs_screen* s = new shwfs_screen;
  s->ny = ny;
  s->nx = nx;
  s->keys = shwfs::PhiloxKeys{};
  {
    shwfs::WfsArgs tmp;
    memset(&tmp, 0, sizeof(tmp));
    tmp.seed = seed;
    shwfs::set_philox_keys(tmp);
    s->keys = tmp.philoxKeys;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = upload(&s->scr, init, (size_t)ny * nx);
  if (e == cudaSuccess && ay) e = upload(&s->a[0], ay, (size_t)ny * 2 * ny);
  if (e == cudaSuccess && by) e = upload(&s->b[0], by, (size_t)ny * ny);
  if (e == cudaSuccess && ax) e = upload(&s->a[1], ax, (size_t)nx * 2 * nx);
  if (e == cudaSuccess && bx) e = upload(&s->b[1], bx, (size_t)nx * nx);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->noise, (size_t)std::max(ny, nx) * sizeof(double));
  if (e != cudaSuccess) {
    release(s);
    return cuda_fail(e, "screen_create");
  }
  *out = s;
  return SHWFS_OK;
}

shwfs_status shwfs_screen_add(shwfs_screen* s, int axis, int n, double coeff_turb, double step, const double* noise,
                              void* stream) {
  if (!s || axis < 0 || axis > 3 || n < 0) return engine_fail(SHWFS_ERR_INVALID, "screen_add: bad arguments");
  const int start = axis >= 2 ? 1 : 0;
  axis &= 1;
  if (!s->a[axis]) return engine_fail(SHWFS_ERR_INVALID, "screen_add: no matrices for this axis");
  cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
  const int len = axis == 0 ? s->ny : s->nx;
  for (int k = 0; k < n; k++) {
    if (noise) {
      SCK(cudaMemcpyAsync(s->noise, noise + (size_t)k * len, len * sizeof(double), cudaMemcpyHostToDevice, st),
          "screen_add noise");
    } else {
      shwfs::screen_noise_kernel<<<(len + 255) / 256, 256, 0, st>>>(s->keys, s->added, len, s->noise);
      SCK(cudaGetLastError(), "screen_noise_kernel");
    }
    const int blocks = (len + shwfs::kScrWarps - 1) / shwfs::kScrWarps;
    shwfs::screen_extrude_kernel<<<blocks, shwfs::kScrWarps * 32, 0, st>>>(
        s->scr, s->ny, s->nx, s->rs, s->cs, axis, start, s->a[axis], s->b[axis], s->noise, coeff_turb,
        k == 0 ? step : 0.0);
    SCK(cudaGetLastError(), "screen_extrude_kernel");
    if (axis == 0)
      s->cs = start ? (s->cs + s->nx - 1) % s->nx : (s->cs + 1) % s->nx;
    else
      s->rs = start ? (s->rs + s->ny - 1) % s->ny : (s->rs + 1) % s->ny;
    s->added++;  // the next extrusion's noise overwrites s->noise in stream order
  }
  if (!stream) SCK(cudaStreamSynchronize(st), "screen_add sync");
  return SHWFS_OK;
}

shwfs_status shwfs_screen_window(shwfs_screen* s, int y0, int x0, int h, int w, float* out, int64_t out_stride,
                                 void* stream) {
  if (!s || !out || y0 < 0 || x0 < 0 || h < 1 || w < 1 || y0 + h > s->ny || x0 + w > s->nx || out_stride < w)
    return engine_fail(SHWFS_ERR_INVALID, "screen_window: window outside the screen");
  cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
  const long long total = (long long)h * w;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 8);
  shwfs::screen_window_kernel<<<blocks, 256, 0, st>>>(s->scr, s->ny, s->nx, s->rs, s->cs, y0, x0, h, w, out,
                                                       (long long)out_stride);
  SCK(cudaGetLastError(), "screen_window_kernel");
  if (!stream) SCK(cudaStreamSynchronize(st), "screen_window sync");
  return SHWFS_OK;
}

shwfs_status shwfs_screens_pupil_phase(shwfs_screen* const* screens, int nlayers, const int* y0, const int* x0,
                                       const float* yshift, const float* xshift, int npup, const float* pupil,
                                       double pupil_area, int remove_piston, float scale, float* out, void* stream) {
  if (!screens || nlayers < 1 || nlayers > shwfs::kMaxLayers || !y0 || !x0 || !yshift || !xshift || npup < 1 ||
      !pupil || !out || !(pupil_area > 0.0))
    return engine_fail(SHWFS_ERR_INVALID, "screens_pupil_phase: bad arguments (1..16 layers, npup >= 1, area > 0)");
  shwfs::LayerSet L{};
  L.n = nlayers;
  for (int q = 0; q < nlayers; q++) {
    const shwfs_screen* s = screens[q];
    if (!s) return engine_fail(SHWFS_ERR_INVALID, "screens_pupil_phase: null screen");
    if (y0[q] < 0 || x0[q] < 0 || y0[q] + npup + 1 > s->ny || x0[q] + npup + 1 > s->nx)
      return engine_fail(SHWFS_ERR_INVALID, "screens_pupil_phase: window (npup+1 square) outside a screen");
    const float xs = xshift[q], ys = yshift[q];
    if (!(xs >= 0.f && xs <= 1.f && ys >= 0.f && ys <= 1.f))
      return engine_fail(SHWFS_ERR_INVALID, "screens_pupil_phase: shifts must be in [0, 1]");
    shwfs::LayerWin& w = L.l[q];
    w.scr = s->scr;
    w.ny = s->ny;
    w.nx = s->nx;
    w.rs = s->rs;
    w.cs = s->cs;
    w.y0 = y0[q];
    w.x0 = x0[q];
    // linearshift's weights in float (cmod/src/interpmodule.c:1277-1280)
    w.s1 = (float)((1.0 - (double)xs) * (1.0 - (double)ys));
    w.s2 = (float)((1.0 - (double)xs) * (double)ys);
    w.s3 = (float)((double)xs * (1.0 - (double)ys));
    w.s4 = xs * ys;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : screens[0]->stream;
  const long long n = (long long)npup * npup;
  const int blocks = (int)std::min<long long>((n + shwfs::kPupilThreads - 1) / shwfs::kPupilThreads, 1024);
  double* partial = nullptr;
  SCK(cudaMallocAsync((void**)&partial, (size_t)blocks * sizeof(double), st), "screens_pupil_phase");
  shwfs::pupil_layers_kernel<<<blocks, shwfs::kPupilThreads, 0, st>>>(L, npup, out, pupil, partial);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    shwfs::pupil_finish_kernel<<<blocks, shwfs::kPupilThreads, 0, st>>>(out, pupil, n, partial, blocks, pupil_area,
                                                                      remove_piston, scale);
    e = cudaGetLastError();
  }
  cudaFreeAsync(partial, st);
  if (e != cudaSuccess) return cuda_fail(e, "pupil phase kernels");
  if (!stream) SCK(cudaStreamSynchronize(st), "screens_pupil_phase sync");
  return SHWFS_OK;
}

shwfs_status shwfs_screen_read(shwfs_screen* s, float* host_out) {
  if (!s || !host_out) return engine_fail(SHWFS_ERR_INVALID, "screen_read: null argument");
  float* d = nullptr;
  SCK(cudaMalloc((void**)&d, (size_t)s->ny * s->nx * sizeof(float)), "screen_read");
  shwfs_status r = shwfs_screen_window(s, 0, 0, s->ny, s->nx, d, s->nx, s->stream);
  if (r == SHWFS_OK) {
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(host_out, d, (size_t)s->ny * s->nx * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) r = cuda_fail(e, "screen_read");
  }
  cudaFree(d);
  return r;
}

shwfs_status shwfs_screen_free(shwfs_screen* s) {
  if (s) {
    cudaStreamSynchronize(s->stream);
    release(s);
  }
  return SHWFS_OK;
}

}  // extern "C"
