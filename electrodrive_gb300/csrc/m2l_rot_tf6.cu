// Two-float rotation M2L kernels, order 6, 128 threads per block (packed and scalar matrices).
#include "m2l_rot.cuh"

namespace edfmm {

int m2l_rot_tf6(bool packed, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s) {
    return packed ? launch_rot_tf<6, 128, true>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s)
                  : launch_rot_tf<6, 128, false>(M, off, src, rows, a, b, c, d, Mx, Lx, nc_pad, mask, s);
}

}  // namespace edfmm
