// The rotation-based M2L launchers (the kernels are in m2l_rot.cuh,
// instantiated by m2l_rot_f32.cu, m2l_rot_f64.cu and m2l_rot_tf*.cu).
#include <cstdint>

#include "m2l_rot.cuh"

namespace edfmm {

// Rotation-based M2L for expansion orders 1..8 (FP32: pairs with a source
// scale above 256x the target's are left to the caller's generic kernel).
// Rows of instances inactive under ``mask`` are skipped (their locals are
// left as they were).
int launch_m2l_rot(int dtype, int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows,
                   const void *tcen,
                   const void *thal, const void *cen, const void *hal, const void *Mx, void *Lx, int nc_pad,
                   const InstMask &mask, cudaStream_t s) {
    if (M <= 0) return EDFMM_OK;
    // the FP32 kernel reads rows two coefficients (16 bytes) at a time
    if (dtype != EDFMM_F64 && ((reinterpret_cast<uintptr_t>(Mx) & 15) != 0 || (nc_pad & 1) != 0))
        return EDFMM_ERR_ARG;
    return dtype == EDFMM_F64 ? m2l_rot_f64(p, M, off, src, rows, tcen, thal, cen, hal, Mx, Lx, nc_pad, mask, s)
                              : m2l_rot_f32(p, M, off, src, rows, tcen, thal, cen, hal, Mx, Lx, nc_pad, mask, s);
}

// Two-float M2L of an FP64 plan (orders 6..8); returns EDFMM_ERR_UNSUPPORTED
// for other orders (the caller then runs the FP64 kernel).
int launch_m2l_rot_tf(int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows,
                      const void *tnodes, const void *thal,
                      const void *snodes, const void *hal, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                      int block, bool packed, cudaStream_t s) {
    if (M <= 0) return EDFMM_OK;
    switch (p) {
        case 6: return m2l_rot_tf6(packed, M, off, src, rows, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s);
        case 7: return m2l_rot_tf7(packed, M, off, src, rows, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s);
        case 8:
            return block == 256 ? m2l_rot_tf8w(packed, M, off, src, rows, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s)
                                : m2l_rot_tf8(packed, M, off, src, rows, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s);
        default: return EDFMM_ERR_UNSUPPORTED;
    }
}

}  // namespace edfmm
