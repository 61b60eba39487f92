// One-pass time step (fdtd_onepass.cuh): float32 instantiations, tensor maps
// and launch.
#include "fdtd_launch.cuh"
#include "fdtd_onepass.cuh"

namespace fdtd {

namespace {

// Dispatch on the tile height and the material modes (H material: values or
// uniform; an H index map runs on the values).
template <template <int, int, int> class F, class... A>
auto one_dispatch(int TY, int mE, int mH, A &&...a) {
    const bool hu = mH == MAT_UNIFORM;
    if (TY == 8) {
        if (mE == MAT_IDS) return hu ? F<8, MAT_IDS, MAT_UNIFORM>::run(a...) : F<8, MAT_IDS, MAT_FULL>::run(a...);
        if (mE == MAT_UNIFORM)
            return hu ? F<8, MAT_UNIFORM, MAT_UNIFORM>::run(a...) : F<8, MAT_UNIFORM, MAT_FULL>::run(a...);
        return hu ? F<8, MAT_FULL, MAT_UNIFORM>::run(a...) : F<8, MAT_FULL, MAT_FULL>::run(a...);
    }
    if (mE == MAT_IDS) return hu ? F<4, MAT_IDS, MAT_UNIFORM>::run(a...) : F<4, MAT_IDS, MAT_FULL>::run(a...);
    if (mE == MAT_UNIFORM)
        return hu ? F<4, MAT_UNIFORM, MAT_UNIFORM>::run(a...) : F<4, MAT_UNIFORM, MAT_FULL>::run(a...);
    return hu ? F<4, MAT_FULL, MAT_UNIFORM>::run(a...) : F<4, MAT_FULL, MAT_FULL>::run(a...);
}

template <int TY, int MATE, int MATH>
struct AllowF {
    static cudaError_t run(size_t bytes) {
        return cudaFuncSetAttribute(k_step_onepass<PF32, TY, MATE, MATH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)bytes);
    }
};

template <int TY, int MATE, int MATH>
struct LaunchF {
    static int run(Plan &p, int dir, const double *wave, cudaStream_t st) {
        const CUtensorMap *m = p.omaps[dir];
        k_step_onepass<PF32, TY, MATE, MATH><<<p.ogrid, p.oblock, p.osmem, st>>>(p.ko[dir], wave, m[0], m[1], m[2],
                                                                                 m[3]);
        return 0;
    }
};

template <int TY, int MATE, int MATH>
struct BytesF {
    static size_t run(int what) {
        using G = OneGeom<float, TY, MATE, MATH>;
        return what == 0 ? (size_t)G::fieldBytes : (size_t)G::xBytes;
    }
};

}  // namespace

size_t onepass_bytes(int precision, int tile_rows, int mat_E, int mat_H, int what) {
    (void)precision;  // float32 only
    return one_dispatch<BytesF>(tile_rows == 8 ? 8 : 4, mat_E, mat_H, what);
}

int prepare_onepass_f32(Plan &p) {
    const GridK &k = p.ko[0];
    const int TY = k.TY, Zc = 32 * PF32::V;
    const int esz = (int)sizeof(float);
    const int boxH = (3 * Zc + 8) * esz / 8, boxE = (3 * Zc + 4) * esz / 8, boxO = 3 * Zc * esz / 8;
    for (int dir = 0; dir < 2; ++dir) {
        // sources of direction 0 are the caller's buffers, of direction 1 the alternates
        const void *Hs = p.ko[1 - dir].H, *Es = p.ko[1 - dir].E;
        CUtensorMap *m = p.omaps[dir];
        bool ok = encode_field_map(&m[0], Hs, k, esz, boxH, TY + 2) && encode_field_map(&m[1], Es, k, esz, boxE, TY + 1);
        if (k.mat_E == MAT_FULL) ok = ok && encode_field_map(&m[2], k.ie, k, esz, boxE, TY + 1);
        else if (k.mat_E == MAT_IDS) ok = ok && encode_index_map(&m[2], k.mid_E, k, Zc + 16, TY + 1);
        else m[2] = m[1];
        if (k.mat_H == MAT_FULL) ok = ok && encode_field_map(&m[3], k.imu, k, esz, boxO, TY);
        else m[3] = m[1];
        if (!ok) return FDTD_ERR_UNSUPPORTED;
    }
    const cudaError_t e = one_dispatch<AllowF>(TY, k.mat_E, k.mat_H, p.osmem);
    if (e != cudaSuccess) {
        set_last_cuda_error((int)e);
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

int onepass_step_f32(Plan &p, int dir, const double *wave, cudaStream_t st) {
    const GridK &k = p.ko[dir];
    one_dispatch<LaunchF>(k.TY, k.mat_E, k.mat_H, p, dir, wave, st);
    if (p.onepass_hcopy) {
        // periodic x after the H half: H[nx-1] = H[0] in the buffer just written
        const int blocks = grid_stride_blocks((long)k.ny * k.nz * 3);
        k_plane_copy<float, false><<<blocks, kThreads, 0, st>>>((float *)k.H, nullptr, k.nx, k.ny, k.nz, 0,
                                                                k.nx - 1, 0);
    }
    return FDTD_OK;
}

}  // namespace fdtd
