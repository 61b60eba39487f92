// float64 instantiation of the time-step kernels (reference operation order).
#include "fdtd_launch.cuh"

namespace fdtd {
int run_f64(Plan &p, const fdtd_run_args *a, cudaStream_t st) { return run_impl<PF64>(p, a, st); }
}  // namespace fdtd
