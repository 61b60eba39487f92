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
}  // namespace fdtd
