// Infinite phase screen resident on the device (science/infScrn.py
// addNewColumnOnEnd :747-791, addNewRowOnEnd :825-855): each new column
// (row) is A Z + coeff B n + step, Z the last two columns (rows) stacked
// oldest first, n standard normals; A and B come from the host in float64.
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
__global__ void screen_extrude_kernel(float* __restrict__ scr, int ny, int nx, int rs, int cs, int axis,
                                      const double* __restrict__ A, const double* __restrict__ B,
                                      const double* __restrict__ noise, double coeff, double step) {
  const int len = axis == 0 ? ny : nx;  // output length; Z has 2 len entries
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kScrWarps + (threadIdx.x >> 5);
  if (i >= len) return;
  // logical element k of line l (0: the older of the last two, 1: the last)
  auto z = [&](int l, int k) {
    if (axis == 0) {
      const int x = nx - 2 + l;
      return (double)scr[(long long)((rs + k) % ny) * nx + (cs + x) % nx];
    }
    const int y = ny - 2 + l;
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
    // the new line replaces the oldest one: physical column cs (row rs)
    if (axis == 0)
      scr[(long long)((rs + i) % ny) * nx + cs] = (float)v;
    else
      scr[(long long)rs * nx + (cs + i) % nx] = (float)v;
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
  if (!s || (axis != 0 && axis != 1) || n < 0) return engine_fail(SHWFS_ERR_INVALID, "screen_add: bad arguments");
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
        s->scr, s->ny, s->nx, s->rs, s->cs, axis, s->a[axis], s->b[axis], s->noise, coeff_turb, k == 0 ? step : 0.0);
    SCK(cudaGetLastError(), "screen_extrude_kernel");
    if (axis == 0)
      s->cs = (s->cs + 1) % s->nx;
    else
      s->rs = (s->rs + 1) % s->ny;
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
