// float64 instantiation of the time-step kernels (reference operation order).
#include "fdtd_launch.cuh"

namespace fdtd {
int run_f64(Plan &p, const fdtd_run_args *a, const fdtd_capture_args *cap, cudaStream_t st) {
    return p.k.scaled ? run_impl<PF64S>(p, a, cap, st) : run_impl<PF64>(p, a, cap, st);
}
int prepare_tma_f64(Plan &p) { return p.k.scaled ? prepare_tma_impl<PF64S>(p) : prepare_tma_impl<PF64>(p); }

size_t tma_stage_bytes(int precision, int tile_rows, int mat_E, int mat_H) {
    switch (precision) {
        case FDTD_FLOAT32:
            return stage_bytes_of<PF32>(tile_rows, mat_E, mat_H);
        case FDTD_FLOAT32C:
            return stage_bytes_of<PF32C>(tile_rows, mat_E, mat_H);
        default:
            return stage_bytes_of<PF64>(tile_rows, mat_E, mat_H);
    }
}
}  // namespace fdtd
