// Tensor-grid conductor meshes on the GPU (electrodrive/core/bem_mesh.py:27-212).
//
// The host supplies the 1-D coordinate tables the reference builds with
// numpy (linspace values and their sines and cosines: O(n_a + n_b) numbers);
// the device forms every vertex, the triangle index lists, and the panel
// geometry (centroid, cross product, area, degenerate-panel removal, unit
// normal) of the whole, possibly multi-conductor, mesh.  Each product, sum
// and quotient is evaluated in numpy's order with the _rn intrinsics (no
// contraction into FMA) and sqrt is correctly rounded on both sides, so the
// arrays are bit-identical to the host meshers' for the same tables.
#include "edfmm_internal.cuh"

namespace edfmm {
namespace {

inline unsigned nb(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// vertices of one grid (row-major over (a, b)) and its raw triangles
__global__ void k_grid_vertices(int kind, double p0, double p1, double p2, double p3, double p4,
                                const double *__restrict__ ta, int64_t na, const double *__restrict__ tb, int64_t nb_,
                                double *__restrict__ V) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= na * nb_) return;
    const int64_t i = k / nb_, j = k % nb_;
    double x, y, z;
    if (kind == EDFMM_MESH_SPHERE) {
        // (cx + r sin(t) cos(p), cy + r sin(t) sin(p), cz + r cos(t)); ta = (sin t, cos t), tb = (sin p, cos p)
        const double st = ta[2 * i], ct = ta[2 * i + 1], sp = tb[2 * j], cp = tb[2 * j + 1];
        const double rs = __dmul_rn(p3, st);
        x = __dadd_rn(p0, __dmul_rn(rs, cp));
        y = __dadd_rn(p1, __dmul_rn(rs, sp));
        z = __dadd_rn(p2, __dmul_rn(p3, ct));
    } else if (kind == EDFMM_MESH_TORUS) {
        // ((R + a cos v) cos u + cx, (R + a cos v) sin u + cy, a sin v + cz); ta = (sin u, cos u), tb = (sin v, cos v)
        const double su = ta[2 * i], cu = ta[2 * i + 1], sv = tb[2 * j], cv = tb[2 * j + 1];
        const double w = __dadd_rn(p3, __dmul_rn(p4, cv));
        x = __dadd_rn(__dmul_rn(w, cu), p0);
        y = __dadd_rn(__dmul_rn(w, su), p1);
        z = __dadd_rn(__dmul_rn(p4, sv), p2);
    } else {
        // plane patch: (x_i, y_j, z); ta = x, tb = y
        x = ta[i];
        y = tb[j];
        z = p0;
    }
    V[3 * k] = x;
    V[3 * k + 1] = y;
    V[3 * k + 2] = z;
}

__global__ void k_grid_triangles(int kind, int64_t na, int64_t nb_, int64_t voff, int32_t cid, int32_t *__restrict__ T,
                                 int32_t *__restrict__ C) {
    // two triangles per cell, cells row-major, the reference's vertex order
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t ncell_a, ncell_b;
    if (kind == EDFMM_MESH_SPHERE) {
        ncell_a = na - 1;
        ncell_b = nb_;
    } else if (kind == EDFMM_MESH_TORUS) {
        ncell_a = na;
        ncell_b = nb_;
    } else {
        ncell_a = na - 1;
        ncell_b = nb_ - 1;
    }
    if (k >= ncell_a * ncell_b) return;
    const int64_t i = k / ncell_b, j = k % ncell_b;
    int64_t t0[3], t1[3];
    if (kind == EDFMM_MESH_SPHERE) {
        const int64_t jn = (j + 1) % nb_;
        const int64_t a = i * nb_ + j, b = i * nb_ + jn, c = (i + 1) * nb_ + j, d = (i + 1) * nb_ + jn;
        t0[0] = a, t0[1] = b, t0[2] = c;
        t1[0] = b, t1[1] = d, t1[2] = c;
    } else if (kind == EDFMM_MESH_TORUS) {
        const int64_t in = (i + 1) % na, jn = (j + 1) % nb_;
        const int64_t A = i * nb_ + j, B = i * nb_ + jn, Cc = in * nb_ + j, D = in * nb_ + jn;
        t0[0] = A, t0[1] = B, t0[2] = Cc;
        t1[0] = B, t1[1] = D, t1[2] = Cc;
    } else {
        const int64_t n1 = nb_;  // n + 1 points per row
        const int64_t idx = i * n1 + j;
        t0[0] = idx, t0[1] = idx + 1, t0[2] = idx + n1;
        t1[0] = idx + 1, t1[1] = idx + n1 + 1, t1[2] = idx + n1;
    }
    for (int q = 0; q < 3; ++q) {
        T[6 * k + q] = (int32_t)(t0[q] + voff);
        T[6 * k + 3 + q] = (int32_t)(t1[q] + voff);
    }
    C[2 * k] = cid;
    C[2 * k + 1] = cid;
}

// panel geometry of every raw triangle: area and the keep flag (area > 1e-16)
__global__ void k_panel_area(const double *__restrict__ V, const int32_t *__restrict__ T, int64_t nt,
                             double *__restrict__ cross, double *__restrict__ area, int32_t *__restrict__ keep) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const double *a = V + 3 * (int64_t)T[3 * t], *b = V + 3 * (int64_t)T[3 * t + 1], *c = V + 3 * (int64_t)T[3 * t + 2];
    const double u0 = __dsub_rn(b[0], a[0]), u1 = __dsub_rn(b[1], a[1]), u2 = __dsub_rn(b[2], a[2]);
    const double w0 = __dsub_rn(c[0], a[0]), w1 = __dsub_rn(c[1], a[1]), w2 = __dsub_rn(c[2], a[2]);
    // numpy.cross: u1 w2 - u2 w1, u2 w0 - u0 w2, u0 w1 - u1 w0 (rounded products)
    const double x = __dsub_rn(__dmul_rn(u1, w2), __dmul_rn(u2, w1));
    const double y = __dsub_rn(__dmul_rn(u2, w0), __dmul_rn(u0, w2));
    const double z = __dsub_rn(__dmul_rn(u0, w1), __dmul_rn(u1, w0));
    // 0.5 * numpy.linalg.norm(cross, axis=1): sqrt((x^2 + y^2) + z^2)
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    const double ar = __dmul_rn(0.5, __dsqrt_rn(s));
    cross[3 * t] = x;
    cross[3 * t + 1] = y;
    cross[3 * t + 2] = z;
    area[t] = ar;
    keep[t] = ar > 1e-16 ? 1 : 0;
}

__global__ void k_panel_emit(const double *__restrict__ V, const int32_t *__restrict__ T, const int32_t *__restrict__ C,
                             const double *__restrict__ cross, const double *__restrict__ area,
                             const int32_t *__restrict__ keep, const int32_t *__restrict__ pos, int64_t nt,
                             int32_t *__restrict__ To, int32_t *__restrict__ Co, double *__restrict__ cen,
                             double *__restrict__ nrm, double *__restrict__ ao) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt || !keep[t]) return;
    const int64_t o = pos[t];
    const double *a = V + 3 * (int64_t)T[3 * t], *b = V + 3 * (int64_t)T[3 * t + 1], *c = V + 3 * (int64_t)T[3 * t + 2];
    const double ar = area[t];
    const double den = __dadd_rn(__dmul_rn(2.0, ar), 1e-30);
    for (int q = 0; q < 3; ++q) {
        To[3 * o + q] = T[3 * t + q];
        // (v0 + v1 + v2) / 3
        cen[3 * o + q] = __ddiv_rn(__dadd_rn(__dadd_rn(a[q], b[q]), c[q]), 3.0);
        nrm[3 * o + q] = __ddiv_rn(cross[3 * t + q], den);
    }
    Co[o] = C[t];
    ao[o] = ar;
}

}  // namespace
}  // namespace edfmm

using namespace edfmm;

extern "C" {

int edfmm_mesh_grid(int kind, const double *params_host, const double *tab_a_dev, int64_t na,
                    const double *tab_b_dev, int64_t nb_, int64_t vertex_offset, int32_t conductor_id,
                    double *vertices_dev, int32_t *triangles_dev, int32_t *conductor_ids_dev, void *stream) {
    if (kind != EDFMM_MESH_SPHERE && kind != EDFMM_MESH_TORUS && kind != EDFMM_MESH_PLANE)
        return fail(EDFMM_ERR_ARG, "kind must be EDFMM_MESH_SPHERE, EDFMM_MESH_TORUS or EDFMM_MESH_PLANE");
    if (!params_host || na < 2 || nb_ < 2 || vertex_offset < 0)
        return fail(EDFMM_ERR_ARG, "need parameters and at least two entries per table");
    if (!tab_a_dev || !tab_b_dev || !vertices_dev || !triangles_dev || !conductor_ids_dev)
        return fail(EDFMM_ERR_ARG, "NULL table or output");
    if (vertex_offset + na * nb_ > INT32_MAX) return fail(EDFMM_ERR_ARG, "vertex indices exceed int32");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const double *p = params_host;
    const int64_t nv = na * nb_;
    k_grid_vertices<<<nb(nv, 256), 256, 0, s>>>(kind, p[0], p[1], p[2], p[3], p[4], tab_a_dev, na, tab_b_dev, nb_,
                                                 vertices_dev);
    EDFMM_LAUNCH_CHECK("k_grid_vertices");
    const int64_t ncell = kind == EDFMM_MESH_TORUS ? na * nb_ : (kind == EDFMM_MESH_SPHERE ? (na - 1) * nb_ : (na - 1) * (nb_ - 1));
    k_grid_triangles<<<nb(ncell, 256), 256, 0, s>>>(kind, na, nb_, vertex_offset, conductor_id, triangles_dev,
                                                     conductor_ids_dev);
    EDFMM_LAUNCH_CHECK("k_grid_triangles");
    return EDFMM_OK;
}

int edfmm_mesh_finish(const double *vertices_dev, int64_t n_vertices, const int32_t *triangles_dev,
                      const int32_t *conductor_ids_dev, int64_t n_triangles, int32_t *triangles_out_dev,
                      int32_t *conductor_ids_out_dev, double *centroids_dev, double *normals_dev, double *areas_dev,
                      int64_t *n_out_host, void *stream) {
    if (!n_out_host) return fail(EDFMM_ERR_ARG, "n_out_host is NULL");
    *n_out_host = 0;
    if (n_triangles < 0 || n_vertices < 0) return fail(EDFMM_ERR_ARG, "negative size");
    if (n_triangles == 0) return EDFMM_OK;
    if (!vertices_dev || !triangles_dev || !conductor_ids_dev || !triangles_out_dev || !conductor_ids_out_dev ||
        !centroids_dev || !normals_dev || !areas_dev)
        return fail(EDFMM_ERR_ARG, "NULL argument");
    if (n_triangles > INT32_MAX) return fail(EDFMM_ERR_ARG, "too many triangles");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DevBuf cross, area, keep, pos, tmp, total;
    int rc;
    if ((rc = cross.reserve(24 * (size_t)n_triangles)) || (rc = area.reserve(8 * (size_t)n_triangles)) ||
        (rc = keep.reserve(4 * (size_t)n_triangles)) || (rc = pos.reserve(4 * (size_t)n_triangles)) ||
        (rc = tmp.reserve(scan_tmp_bytes(n_triangles))) || (rc = total.reserve(8)))
        return rc;
    k_panel_area<<<nb(n_triangles, 256), 256, 0, s>>>(vertices_dev, triangles_dev, n_triangles, dptr<double>(cross),
                                                      dptr<double>(area), dptr<int32_t>(keep));
    EDFMM_LAUNCH_CHECK("k_panel_area");
    if ((rc = scan_exclusive(dptr<int32_t>(keep), dptr<int32_t>(pos), n_triangles, dptr<int64_t>(total), tmp.p, s)))
        return rc;
    k_panel_emit<<<nb(n_triangles, 256), 256, 0, s>>>(vertices_dev, triangles_dev, conductor_ids_dev, dptr<double>(cross),
                                                      dptr<double>(area), dptr<int32_t>(keep), dptr<int32_t>(pos),
                                                      n_triangles, triangles_out_dev, conductor_ids_out_dev,
                                                      centroids_dev, normals_dev, areas_dev);
    EDFMM_LAUNCH_CHECK("k_panel_emit");
    int64_t n_out = 0;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&n_out, total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    *n_out_host = n_out;
    return EDFMM_OK;
}

}  // extern "C"
