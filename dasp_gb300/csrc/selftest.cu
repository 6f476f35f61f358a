// Self-test of the bounded waits every pipeline kernel uses: one CTA waits
// on an mbarrier that nothing arrives on.  The wait must give up after its
// cycle limit, raise the CTA's abort flag and let the kernel return, so
// that a stalled pipeline ends with an error status the host reads and the
// context stays usable.  Nothing faults and nothing hangs: the limit bounds
// the wait.
#include "tc_sm103.cuh"
#include "wfs_plain.cuh"

namespace shwfs {

namespace {

__global__ void bounded_wait_selftest_kernel(long long max_cycles, int* out) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    abort_flag = 0;
    tc::fence_mbar_init();
  }
  __syncthreads();
  const long long t0 = clock64();
  const bool ok = tc::mbar_wait_abortable(&bar, 0, &abort_flag, max_cycles);
  const long long dt = clock64() - t0;
  __syncthreads();
  if (threadIdx.x == 0) {
    out[0] = ok ? 0 : 1;        // 1: the wait gave up
    out[1] = abort_flag;        // 1: the abort flag was raised
    out[2] = (int)(dt >> 20);  // cycles waited / 2^20
  }
}

}  // namespace

cudaError_t launch_bounded_wait_selftest(long long max_cycles, int* out, cudaStream_t stream) {
  bounded_wait_selftest_kernel<<<1, 32, 0, stream>>>(max_cycles, out);
  return cudaGetLastError();
}

}  // namespace shwfs
