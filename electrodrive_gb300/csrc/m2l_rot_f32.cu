// Rotation-based M2L kernels, FP32, orders 1..8.
#include "m2l_rot.cuh"

namespace edfmm {

int m2l_rot_f32(int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s) {
    switch (p) {
        case 1: return launch_rot<float, 1, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 2: return launch_rot<float, 2, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 3: return launch_rot<float, 3, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 4: return launch_rot<float, 4, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 5: return launch_rot<float, 5, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 6: return launch_rot<float, 6, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 7: return launch_rot<float, 7, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        case 8: return launch_rot<float, 8, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
        default: return fail(EDFMM_ERR_UNSUPPORTED, "rotation M2L supports orders 1..8");
    }
}

}  // namespace edfmm
