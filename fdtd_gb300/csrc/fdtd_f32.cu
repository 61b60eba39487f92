// float32 and compensated float32 instantiations of the time-step kernels.
#include "fdtd_launch.cuh"

namespace fdtd {
int run_f32(Plan &p, const fdtd_run_args *a, const fdtd_capture_args *cap, cudaStream_t st) {
    return run_impl<PF32>(p, a, cap, st);
}
int run_f32c(Plan &p, const fdtd_run_args *a, const fdtd_capture_args *cap, cudaStream_t st) {
    return run_impl<PF32C>(p, a, cap, st);
}
int prepare_tma_f32(Plan &p) { return prepare_tma_impl<PF32>(p); }
int prepare_tma_f32c(Plan &p) { return prepare_tma_impl<PF32C>(p); }

// Device check of the failure path of every staged pass: wait (bounded, at
// most `limit` polls) on an mbarrier that nothing arrives at, and report the
// expiry through a status word as the passes do (bit 0).  Nothing faults and
// the context stays usable.
__global__ void k_wait_selftest(int *status, unsigned limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(smem_u32(&bar), 1);
    fence_mbar_init();
    if (!mbar_wait_bounded(smem_u32(&bar), 0u, limit)) atomicOr(status, 1);
}

void launch_wait_selftest(int *status, unsigned limit, cudaStream_t st) { k_wait_selftest<<<1, 32, 0, st>>>(status, limit); }

}  // namespace fdtd
