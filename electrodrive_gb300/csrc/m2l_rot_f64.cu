// Rotation-based M2L kernels, FP64, orders 1..8.
#include "m2l_rot.cuh"

namespace edfmm {

int m2l_rot_f64(int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s) {
    switch (p) {
        case 1: return launch_rot<double, 1, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 2: return launch_rot<double, 2, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 3: return launch_rot<double, 3, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 4: return launch_rot<double, 4, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 5: return launch_rot<double, 5, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 6: return launch_rot<double, 6, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 7: return launch_rot<double, 7, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 8: return launch_rot<double, 8, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        default: return fail(EDFMM_ERR_UNSUPPORTED, "rotation M2L supports orders 1..8");
    }
}

}  // namespace edfmm
