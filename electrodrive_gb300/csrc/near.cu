// Singular and near-singular panel quadrature of the single-layer operator.
//
// Restates (paths inside the reference project):
//   * standard_triangle_quadrature      core/bem_quadrature.py:79-150
//       order 1: centroid; order 2: barycentric permutations of (2/3, 1/6, 1/6),
//       weights w_ref * area, area = |(v1 - v0) x (v2 - v0)| / 2
//   * near_singular_quadrature          core/bem_quadrature.py:217-308
//       `depth` times: split (4-way, edge midpoints) the subtriangle whose
//       centroid is nearest the target (first on ties, list order kept by
//       pop + append), then apply the base rule on every leaf
//   * self integrals                    core/bem.py:1781-1805
//       I_i = sum_k K_E w_k / max(|C_i - y_k|, 1e-12) at the panel's own centroid
//   * near pairs                        core/bem.py:475-555
//       0 < |C_i - C_j| <= f (R_i + R_j), R = sqrt(A / pi), evaluated with the
//       same FP64 roundings as numpy (no fused multiply-add), found with a
//       uniform grid instead of the reference's O(N^2) scan; CSR by target i,
//       sources j ascending (the reference's row-major order)
//   * correction weights                core/bem.py:558-667
//       delta_ij = sum_k K_E w_k / max(|C_i - y_k|, 1e-12) - K_E A_j / max(|C_i - C_j|, 1e-12)
//       on panel j refined uniformly `depth` times
//   * application                       core/bem.py:675-734
//       V_i += sum_j sigma_j delta_ij (row sums in column order: deterministic)
//   * on-the-fly module                 core/bem_near_cuda_kernel.cu:110-232
//       the same correction with the unrefined rule of `quad_order`, weights
//       recomputed per call, here one warp per target row instead of one
//       thread per pair with atomics.
// All geometry work is FP64 (it runs once per mesh); the application kernel
// runs in the solve dtype.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "edfmm_internal.cuh"
#include "twofloat.cuh"

namespace edfmm {
namespace {

inline unsigned nb(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct V3 {
    double x, y, z;
};
__device__ __forceinline__ V3 ld3(const double *p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 mid(V3 a, V3 b) {
    return V3{__dmul_rn(0.5, __dadd_rn(a.x, b.x)), __dmul_rn(0.5, __dadd_rn(a.y, b.y)),
              __dmul_rn(0.5, __dadd_rn(a.z, b.z))};
}
// numpy-order norm of a difference: sqrt((dx*dx + dy*dy) + dz*dz), no FMA
__device__ __forceinline__ double dist_np(V3 a, V3 b) {
    const double dx = __dsub_rn(a.x, b.x), dy = __dsub_rn(a.y, b.y), dz = __dsub_rn(a.z, b.z);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}
__device__ __forceinline__ double tri_area(V3 a, V3 b, V3 c) {
    const double e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z;
    const double e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
    const double cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
    return 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
}
__device__ __forceinline__ V3 centroid3(V3 a, V3 b, V3 c) {
    return V3{(a.x + b.x + c.x) / 3.0, (a.y + b.y + c.y) / 3.0, (a.z + b.z + c.z) / 3.0};
}

// sum_k K_E w_k / max(|t - y_k|, 1e-12) of the base rule on triangle (a, b, c)
__device__ __forceinline__ double rule_sum(V3 a, V3 b, V3 c, V3 t, int order, double ke) {
    const double area = tri_area(a, b, c);
    if (!(area > 0.0)) return 0.0;
    if (order <= 1) {
        const V3 y = centroid3(a, b, c);
        return ke / fmax(dist_np(t, y), 1e-12) * area;
    }
    const double p = 2.0 / 3.0, q = 1.0 / 6.0, w = area / 3.0;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double l0 = k == 0 ? p : q, l1 = k == 1 ? p : q, l2 = k == 2 ? p : q;
        const V3 y{l0 * a.x + l1 * b.x + l2 * c.x, l0 * a.y + l1 * b.y + l2 * c.y, l0 * a.z + l1 * b.z + l2 * c.z};
        s += ke / fmax(dist_np(t, y), 1e-12) * w;
    }
    return s;
}

constexpr int kMaxAdaptiveDepth = 8;

// adaptive near-singular rule (list of at most 3 depth + 1 triangles)
__device__ double adaptive_sum(V3 v0, V3 v1, V3 v2, V3 t, int order, int depth, double ke) {
    V3 tri[3 * kMaxAdaptiveDepth + 1][3];
    int n = 1;
    tri[0][0] = v0;
    tri[0][1] = v1;
    tri[0][2] = v2;
    for (int d = 0; d < depth; ++d) {
        int best = 0;
        double bd = INFINITY;
        for (int i = 0; i < n; ++i) {
            const V3 c = centroid3(tri[i][0], tri[i][1], tri[i][2]);
            const double dd = dist_np(c, t);
            if (dd < bd) {
                bd = dd;
                best = i;
            }
        }
        const V3 a = tri[best][0], b = tri[best][1], c = tri[best][2];
        for (int i = best; i < n - 1; ++i) {  // pop(best), keeping order
            tri[i][0] = tri[i + 1][0];
            tri[i][1] = tri[i + 1][1];
            tri[i][2] = tri[i + 1][2];
        }
        n -= 1;
        const V3 m01 = mid(a, b), m12 = mid(b, c), m20 = mid(c, a);
        const V3 kids[4][3] = {{a, m01, m20}, {m01, b, m12}, {m20, m12, c}, {m01, m12, m20}};
        for (int k = 0; k < 4; ++k) {
            tri[n][0] = kids[k][0];
            tri[n][1] = kids[k][1];
            tri[n][2] = kids[k][2];
            ++n;
        }
    }
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += rule_sum(tri[i][0], tri[i][1], tri[i][2], t, order, ke);
    return s;
}

__global__ void k_self_integrals(const double *__restrict__ verts, const double *__restrict__ cent, int64_t n,
                                 int order, int depth, double ke, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = adaptive_sum(ld3(verts + 9 * i), ld3(verts + 9 * i + 3), ld3(verts + 9 * i + 6), ld3(cent + 3 * i),
                          order, depth, ke);
}

__device__ __forceinline__ double disk_radius(double a) { return __dsqrt_rn(__ddiv_rn(a > 0.0 ? a : 0.0, M_PI)); }

// Near-field correction of potentials at arbitrary targets
// (_apply_near_quadrature_potentials, electrodrive/core/bem.py:940-1046): for
// target x and every panel j with |C_j - x| <= f R_j, R_j = sqrt(A_j / pi),
// and A_j > 0, sigma_j != 0:
//   V(x) += sigma_j (I_near - K_E A_j / max(|C_j - x|, 1e-12)),
// I_near the adaptive rule of panel j about x (the rule of the self integrals).
// One warp per target; the lanes stride over the panels with a squared-
// distance bound before the exact test (the numpy-order distance against
// f R_j), and a fixed shuffle tree adds the lanes' sums into V(x).
__global__ void k_near_targets(const double *__restrict__ tgt, int64_t m, const double *__restrict__ cent,
                               const double *__restrict__ areas, const double *__restrict__ sigma,
                               const double *__restrict__ verts, int64_t n, double factor, int order, int depth,
                               double ke, double *__restrict__ V) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= m) return;  // uniform over the warp
    const V3 x = ld3(tgt + 3 * w);
    const double f2pi = factor * factor / M_PI * (1.0 + 1e-9);  // bound on (f R)^2, slightly widened
    double acc = 0.0;
    for (int64_t j = lane; j < n; j += 32) {
        const double a = areas[j];
        const double dx = cent[3 * j] - x.x, dy = cent[3 * j + 1] - x.y, dz = cent[3 * j + 2] - x.z;
        if (dx * dx + dy * dy + dz * dz > f2pi * (a > 0.0 ? a : 0.0)) continue;
        const V3 c = ld3(cent + 3 * j);
        const double d = dist_np(c, x);
        if (!(d <= factor * disk_radius(a))) continue;
        const double sj = sigma[j];
        if (!(a > 0.0) || sj == 0.0) continue;
        const double I_near = adaptive_sum(ld3(verts + 9 * j), ld3(verts + 9 * j + 3), ld3(verts + 9 * j + 6), x,
                                           order, depth, ke);
        const double I_far = ke * a / (d < 1e-12 ? 1e-12 : d);
        acc += sj * (I_near - I_far);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) V[w] += acc;
}

// ---------------------------------------------------------------------------
// near pairs by uniform grid
// ---------------------------------------------------------------------------

__global__ void k_radii_bounds(const double *cent, const double *areas, int64_t n, double *radii,
                               unsigned long long *rmax, long long *lo, long long *hi) {
    // per-lane values, reduced over the warp, then one atomic per warp
    // and bound (a block of panels updates the same seven words)
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    constexpr long long kLo = 0x7fffffffffffffffLL, kHi = (long long)0x8000000000000000ULL;
    unsigned long long rm = 0;
    long long l[3] = {kLo, kLo, kLo}, h[3] = {kHi, kHi, kHi};
    if (i < n) {
        const double r = disk_radius(areas[i]);
        radii[i] = r;
        if (isfinite(r)) rm = (unsigned long long)__double_as_longlong(r);
        for (int a = 0; a < 3; ++a) {
            const double v = cent[3 * i + a];
            if (!isfinite(v)) continue;
            long long o = __double_as_longlong(v);
            o = o >= 0 ? o : o ^ 0x7fffffffffffffffLL;
            l[a] = o;
            h[a] = o;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long rr = __shfl_xor_sync(0xffffffffu, rm, o);
        rm = rr > rm ? rr : rm;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const long long lo_o = __shfl_xor_sync(0xffffffffu, l[a], o), hi_o = __shfl_xor_sync(0xffffffffu, h[a], o);
            l[a] = lo_o < l[a] ? lo_o : l[a];
            h[a] = hi_o > h[a] ? hi_o : h[a];
        }
    }
    if ((threadIdx.x & 31) == 0) {
        if (rm) atomicMax(rmax, rm);
        for (int a = 0; a < 3; ++a) {
            if (l[a] != kLo) atomicMin(&lo[a], l[a]);
            if (h[a] != kHi) atomicMax(&hi[a], h[a]);
        }
    }
}

struct Grid {
    double org[3];
    double h;
    int dim[3];
};

__device__ __forceinline__ int cell_of(const Grid &g, const double *c, int a) {
    int k = (int)floor((c[a] - g.org[a]) / g.h);
    return k < 0 ? 0 : (k >= g.dim[a] ? g.dim[a] - 1 : k);
}

__global__ void k_cell_count(const double *cent, int64_t n, Grid g, int32_t *cell, int32_t *count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *c = cent + 3 * i;
    if (!(isfinite(c[0]) && isfinite(c[1]) && isfinite(c[2]))) {
        cell[i] = -1;
        return;
    }
    const int id = (cell_of(g, c, 2) * g.dim[1] + cell_of(g, c, 1)) * g.dim[0] + cell_of(g, c, 0);
    cell[i] = id;
    atomicAdd(&count[id], 1);
}

__global__ void k_cell_fill(int64_t n, const int32_t *cell, int32_t *cursor, int32_t *items) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || cell[i] < 0) return;
    items[atomicAdd(&cursor[cell[i]], 1)] = (int32_t)i;
}

// pass 0: count near neighbours of each i; pass 1: write them
__global__ void k_near_scan(const double *cent, const double *radii, int64_t n, Grid g, double factor,
                            const int32_t *cell_off, const int32_t *items, int pass, int32_t *row_cnt,
                            const int32_t *row_off, int32_t *cols) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *ci = cent + 3 * i;
    int cnt = 0;
    if (isfinite(ci[0]) && isfinite(ci[1]) && isfinite(ci[2]) && isfinite(radii[i])) {
        const int cx = cell_of(g, ci, 0), cy = cell_of(g, ci, 1), cz = cell_of(g, ci, 2);
        const V3 pi = ld3(ci);
        const int base = pass ? row_off[i] : 0;
        for (int dz = -1; dz <= 1; ++dz) {
            const int z = cz + dz;
            if (z < 0 || z >= g.dim[2]) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int y = cy + dy;
                if (y < 0 || y >= g.dim[1]) continue;
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = cx + dx;
                    if (x < 0 || x >= g.dim[0]) continue;
                    const int id = (z * g.dim[1] + y) * g.dim[0] + x;
                    for (int k = cell_off[id]; k < cell_off[id + 1]; ++k) {
                        const int j = items[k];
                        const double rj = radii[j];
                        if (!isfinite(rj)) continue;
                        const double d = dist_np(pi, ld3(cent + 3 * (int64_t)j));
                        const double th = __dmul_rn(factor, __dadd_rn(radii[i], rj));
                        if (isfinite(d) && d > 0.0 && d <= th) {
                            if (pass) cols[base + cnt] = j;
                            ++cnt;
                        }
                    }
                }
            }
        }
    }
    if (!pass) row_cnt[i] = cnt;
}

__global__ void k_set_last32(int32_t *off, int64_t rows, const int64_t *total) { off[rows] = (int32_t)*total; }

// 1 / max(|d - o|, 1e-12) for a lattice point at offset o from the cell corner
__device__ __forceinline__ double lattice_term(V3 d, V3 o) {
    const double dx = d.x - o.x, dy = d.y - o.y, dz = d.z - o.z;
    return rsqrt(fmax(fma(dz, dz, fma(dy, dy, dx * dx)), 1e-24));
}

// The base rule on the 4^depth triangles of uniform midpoint refinement of
// (a, b, c) (the reference refines recursively by edge midpoints).  The
// leaves are the cells of the barycentric grid of step h = 2^-depth: the
// upright cell (i, j) has corners (i, j), (i+1, j), (i, j+1) and the inverted
// one (i+1, j), (i, j+1), (i+1, j+1), in units of the lattice steps
// E1 = h (b - a) and E2 = h (c - a); every leaf has area(a, b, c) / 4^depth.
// The target's offset from a cell corner, t - a - i E1 - j E2, is formed once
// per cell (three FMAs), and each rule point subtracts its fixed offset in
// the cell from it: three subtractions and one FP64 rsqrt per point.
__device__ double uniform_sum(V3 a, V3 b, V3 c, V3 t, int order, int depth, double ke) {
    const double area = tri_area(a, b, c);
    if (!(area > 0.0)) return 0.0;
    const int m = 1 << depth;
    const double h = 1.0 / (double)m;
    const V3 E1{(b.x - a.x) * h, (b.y - a.y) * h, (b.z - a.z) * h};
    const V3 E2{(c.x - a.x) * h, (c.y - a.y) * h, (c.z - a.z) * h};
    const V3 d0{t.x - a.x, t.y - a.y, t.z - a.z};
    auto off = [&](double u, double v) {
        return V3{fma(v, E2.x, u * E1.x), fma(v, E2.y, u * E1.y), fma(v, E2.z, u * E1.z)};
    };
    double s = 0.0;
    if (order <= 1) {
        // leaf centroids: upright (1/3, 1/3), inverted (2/3, 2/3) from the corner
        const V3 ou = off(1.0 / 3.0, 1.0 / 3.0), oi = off(2.0 / 3.0, 2.0 / 3.0);
        for (int i = 0; i < m; ++i) {
            const V3 r{fma(-(double)i, E1.x, d0.x), fma(-(double)i, E1.y, d0.y), fma(-(double)i, E1.z, d0.z)};
            for (int j = 0; i + j < m; ++j) {
                const V3 d{fma(-(double)j, E2.x, r.x), fma(-(double)j, E2.y, r.y), fma(-(double)j, E2.z, r.z)};
                s += lattice_term(d, ou);
                if (i + j < m - 1) s += lattice_term(d, oi);
            }
        }
        return ke * (area * h * h) * s;
    }
    // points 2/3 at one corner, 1/6 at the others: upright cell offsets
    // (q, q), (p, q), (q, p); inverted cell (1-q, 1-q), (1-p, 1-q), (1-q, 1-p)
    const double p = 2.0 / 3.0, q = 1.0 / 6.0;
    const V3 u0 = off(q, q), u1 = off(p, q), u2 = off(q, p);
    const V3 v0 = off(1.0 - q, 1.0 - q), v1 = off(1.0 - p, 1.0 - q), v2 = off(1.0 - q, 1.0 - p);
    for (int i = 0; i < m; ++i) {
        const V3 r{fma(-(double)i, E1.x, d0.x), fma(-(double)i, E1.y, d0.y), fma(-(double)i, E1.z, d0.z)};
        for (int j = 0; i + j < m; ++j) {
            const V3 d{fma(-(double)j, E2.x, r.x), fma(-(double)j, E2.y, r.y), fma(-(double)j, E2.z, r.z)};
            s += lattice_term(d, u0);
            s += lattice_term(d, u1);
            s += lattice_term(d, u2);
            if (i + j < m - 1) {
                s += lattice_term(d, v0);
                s += lattice_term(d, v1);
                s += lattice_term(d, v2);
            }
        }
    }
    return ke * (area * h * h / 3.0) * s;
}

// 1 / sqrt(a) in two-float for a normal positive a: two Newton steps from the
// FP32 estimate (the first leaves a one-signed error of about 1.5 e0^2 =
// 2^-44.6, the second takes it to the two-float rounding level)
__device__ __forceinline__ tf32x2 tf_rsqrt2(tf32x2 a) {
    const tf32x2 y = tf_rsqrt(a, rsqrt_normal(a.hi));
    const tf32x2 h = tf32x2(1.0f, 0.0f) - a * (y * y);
    return tf_fast_two_sum(y.hi, __fadd_rn(y.lo, __fmul_rn(__fmul_rn(0.5f, y.hi), h.hi)));
}

__device__ __forceinline__ tf32x2 lattice_term_tf(const tf32x2 (&d)[3], const tf32x2 (&o)[3]) {
    const tf32x2 dx = d[0] - o[0], dy = d[1] - o[1], dz = d[2] - o[2];
    tf32x2 r2 = fma(dz, dz, fma(dy, dy, dx * dx));
    if (!(r2.hi >= 1e-24f)) r2 = tf32x2(1e-24f, 0.0f);  // 1 / max(r, 1e-12)
    return tf_rsqrt2(r2);
}

// uniform_sum (order >= 2) on the FP32 pipe: the target offsets and the rule
// points' 1 / r in two-float arithmetic (about 2^-44 per term, against the
// FP64 pipe's 1/64 of the FP32 rate on this GPU), each cell's six terms
// summed in two-float and the cells in FP64.  The geometry (area, lattice
// steps, point offsets) is formed in FP64 once per pair.
__device__ double uniform_sum_tf(V3 a, V3 b, V3 c, V3 t, int depth, double ke) {
    const double area = tri_area(a, b, c);
    if (!(area > 0.0)) return 0.0;
    const int m = 1 << depth;
    const double h = 1.0 / (double)m;
    const V3 E1{(b.x - a.x) * h, (b.y - a.y) * h, (b.z - a.z) * h};
    const V3 E2{(c.x - a.x) * h, (c.y - a.y) * h, (c.z - a.z) * h};
    auto tf3 = [](double x, double y, double z, tf32x2 (&o)[3]) {
        o[0] = tf_from_double(x);
        o[1] = tf_from_double(y);
        o[2] = tf_from_double(z);
    };
    auto off = [&](double u, double v, tf32x2 (&o)[3]) {
        tf3(fma(v, E2.x, u * E1.x), fma(v, E2.y, u * E1.y), fma(v, E2.z, u * E1.z), o);
    };
    const double p = 2.0 / 3.0, q = 1.0 / 6.0;
    tf32x2 u0[3], u1[3], u2[3], v0[3], v1[3], v2[3], e1[3], e2[3], d0[3];
    off(q, q, u0);
    off(p, q, u1);
    off(q, p, u2);
    off(1.0 - q, 1.0 - q, v0);
    off(1.0 - p, 1.0 - q, v1);
    off(1.0 - q, 1.0 - p, v2);
    tf3(-E1.x, -E1.y, -E1.z, e1);
    tf3(-E2.x, -E2.y, -E2.z, e2);
    tf3(t.x - a.x, t.y - a.y, t.z - a.z, d0);
    double s = 0.0;
    for (int i = 0; i < m; ++i) {
        tf32x2 r[3];
        const tf32x2 fi((float)i, 0.0f);
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = fma(fi, e1[k], d0[k]);
        for (int j = 0; i + j < m; ++j) {
            tf32x2 d[3];
            const tf32x2 fj((float)j, 0.0f);
#pragma unroll
            for (int k = 0; k < 3; ++k) d[k] = fma(fj, e2[k], r[k]);
            tf32x2 cs = lattice_term_tf(d, u0) + lattice_term_tf(d, u1) + lattice_term_tf(d, u2);
            if (i + j < m - 1) cs = cs + lattice_term_tf(d, v0) + lattice_term_tf(d, v1) + lattice_term_tf(d, v2);
            s += tf_to_double(cs);
        }
    }
    return ke * (area * h * h / 3.0) * s;
}

// one thread per pair k of the CSR rows (rows hold a few pairs each, and a
// pair's rule is ~200 FP64 evaluations at depth 3); its row i is the last
// row starting at or before k
__global__ void k_near_weights_pairs(const double *__restrict__ cent, const double *__restrict__ areas,
                                     const double *__restrict__ verts, int64_t n, int64_t np,
                                     const int32_t *__restrict__ row_off, const int32_t *__restrict__ cols, int order,
                                     int depth, double ke, double *__restrict__ w) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    int64_t lo = 0, hi = n - 1;  // row_off[lo] <= k < row_off[n]
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (row_off[mid] <= k) lo = mid;
        else hi = mid - 1;
    }
    const V3 ci = ld3(cent + 3 * lo);
    const int j = cols[k];
    const double aj = areas[j];
    double v = 0.0;
    if (aj > 0.0) {
        const V3 a = ld3(verts + 9 * (int64_t)j), b = ld3(verts + 9 * (int64_t)j + 3),
                 c = ld3(verts + 9 * (int64_t)j + 6);
        const double inear =
            order <= 1 ? uniform_sum(a, b, c, ci, order, depth, ke) : uniform_sum_tf(a, b, c, ci, depth, ke);
        const double ifar = ke * aj / fmax(dist_np(ci, ld3(cent + 3 * (int64_t)j)), 1e-12);
        v = inear - ifar;
    }
    w[k] = v;
}

template <typename T>
__global__ void k_near_apply(int64_t n, const int32_t *__restrict__ row_off, const int32_t *__restrict__ cols,
                             const T *__restrict__ w, const T *__restrict__ sigma, const T *__restrict__ v_in,
                             T *__restrict__ v_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T acc = 0;
    for (int k = row_off[i]; k < row_off[i + 1]; ++k) acc += w[k] * sigma[cols[k]];
    v_out[i] = (v_in ? v_in[i] : (T)0) + acc;
}

template <typename T>
__global__ void k_cast(const double *in, T *out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (T)in[i];
}

// the reference CUDA module's on-the-fly correction: rule on the unit triangle
// (u, v) with weights normalised to 1, scaled by A_j.  One thread per pair
// (CSR order) for kNearRows consecutive target rows per block, the pairs'
// corrections staged in shared memory and summed per row by one thread in
// pair order (deterministic, no atomics; a row of any length).  1 / r is
// one FP64 reciprocal square root of max(r^2, 1e-24), i.e. 1 / max(r, 1e-12)
// as the reference clamps it, instead of a square root and a division.
constexpr int kNearThreads = 256, kNearRows = 32;

template <typename T>
__device__ __forceinline__ T near_rinv(T r2) {
    if constexpr (sizeof(T) == 8) return rsqrt(r2 < 1e-24 ? 1e-24 : r2);
    else return rsqrtf(r2 < 1e-24f ? 1e-24f : r2);
}

template <typename T>
__global__ void __launch_bounds__(kNearThreads)
    k_near_onthefly(int64_t n, const int32_t *__restrict__ row_off, const int32_t *__restrict__ cols,
                    const T *__restrict__ cent, const T *__restrict__ areas, const T *__restrict__ sigma,
                    const T *__restrict__ verts, int q, T ke, const T *__restrict__ v_far, T *__restrict__ v_out) {
    __shared__ T delta[kNearThreads];
    __shared__ int32_t rows[kNearRows + 1];  // row_off of this block's rows
    const int64_t r0 = (int64_t)blockIdx.x * kNearRows;
    const int nr = (int)(n - r0 < kNearRows ? n - r0 : kNearRows);
    if (threadIdx.x <= nr) rows[threadIdx.x] = row_off[r0 + threadIdx.x];
    __syncthreads();
    const int kb = rows[0], kend = rows[nr];
    T acc = 0;
    int tr = 0;  // summing thread: its row's position in the block's pair range
    for (int base = kb; base < kend; base += kNearThreads) {
        const int k = base + (int)threadIdx.x;
        T d = 0;
        if (k < kend) {
            // the target row of pair k: the last row starting at or before k
            int hi = nr - 1;
            while (tr < hi) {
                const int mid = (tr + hi + 1) >> 1;
                if (rows[mid] <= k) tr = mid;
                else hi = mid - 1;
            }
            const int j = cols[k];
            const T aj = areas[j], sj = sigma[j];
            if (aj > (T)0 && sj != (T)0) {
                const int64_t i = r0 + tr;
                const T cx = cent[3 * i], cy = cent[3 * i + 1], cz = cent[3 * i + 2];
                const T dx = cx - cent[3 * j], dy = cy - cent[3 * j + 1], dz = cz - cent[3 * j + 2];
                const T rfi = near_rinv(dx * dx + dy * dy + dz * dz);
                const T *v = verts + 9 * (int64_t)j;
                const T v0x = v[0], v0y = v[1], v0z = v[2];
                const T e1x = v[3] - v0x, e1y = v[4] - v0y, e1z = v[5] - v0z;
                const T e2x = v[6] - v0x, e2y = v[7] - v0y, e2z = v[8] - v0z;
                T inear = 0;
                for (int kk = 0; kk < q; ++kk) {
                    T u, w, wk;
                    if (q == 1) {
                        u = w = (T)(1.0 / 3.0);
                        wk = (T)1;
                    } else {
                        u = kk == 0 ? (T)(2.0 / 3.0) : (T)(1.0 / 6.0);
                        w = kk == 1 ? (T)(2.0 / 3.0) : (T)(1.0 / 6.0);
                        wk = (T)(1.0 / 3.0);
                    }
                    const T ex = cx - (v0x + u * e1x + w * e2x), ey = cy - (v0y + u * e1y + w * e2y);
                    const T ez = cz - (v0z + u * e1z + w * e2z);
                    inear += ke * near_rinv(ex * ex + ey * ey + ez * ez) * (wk * aj);
                }
                d = sj * (inear - ke * aj * rfi);
            }
        }
        delta[threadIdx.x] = d;
        __syncthreads();
        if ((int)threadIdx.x < nr) {
            const int lo = max(rows[threadIdx.x], base), hi = min(rows[threadIdx.x + 1], base + kNearThreads);
            for (int kk = lo; kk < hi; ++kk) acc += delta[kk - base];
        }
        __syncthreads();
    }
    if ((int)threadIdx.x < nr) v_out[r0 + threadIdx.x] = v_far[r0 + threadIdx.x] + acc;
}

}  // namespace
}  // namespace edfmm

using namespace edfmm;

struct edfmm_near {
    int64_t n = 0;
    int64_t n_pairs = 0;
    int64_t max_row = 0;
    int dtype = EDFMM_F64;
    DevBuf row_off, cols, w64, w;  // CSR by target; FP64 weights and a solve-dtype copy
};

extern "C" {

EDFMM_API int edfmm_self_integrals(const void *panel_vertices_dev, const void *centroids_dev, int64_t n,
                                   int quad_order, int depth, double k_e, void *out_dev, void *stream) {
    if (n < 0 || depth < 0 || depth > kMaxAdaptiveDepth) return fail(EDFMM_ERR_ARG, "bad n or depth (0..8)");
    if (n == 0) return EDFMM_OK;
    if (!panel_vertices_dev || !centroids_dev || !out_dev) return fail(EDFMM_ERR_ARG, "NULL argument");
    k_self_integrals<<<nb(n, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const double *>(panel_vertices_dev), static_cast<const double *>(centroids_dev), n, quad_order,
        depth, k_e, static_cast<double *>(out_dev));
    EDFMM_LAUNCH_CHECK("k_self_integrals");
    return EDFMM_OK;
}

EDFMM_API int edfmm_near_targets_correct(const void *targets_dev, int64_t m, const void *centroids_dev,
                                         const void *areas_dev, const void *sigma_dev,
                                         const void *panel_vertices_dev, int64_t n, double distance_factor,
                                         int quad_order, int depth, double k_e, void *V_dev, void *stream) {
    if (m < 0 || n < 0 || depth < 0 || depth > kMaxAdaptiveDepth)
        return fail(EDFMM_ERR_ARG, "bad m, n or depth (0..8)");
    if (m == 0 || n == 0) return EDFMM_OK;
    if (!targets_dev || !centroids_dev || !areas_dev || !sigma_dev || !panel_vertices_dev || !V_dev)
        return fail(EDFMM_ERR_ARG, "NULL argument");
    k_near_targets<<<nb(m * 32, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const double *>(targets_dev), m, static_cast<const double *>(centroids_dev),
        static_cast<const double *>(areas_dev), static_cast<const double *>(sigma_dev),
        static_cast<const double *>(panel_vertices_dev), n, distance_factor, quad_order, depth, k_e,
        static_cast<double *>(V_dev));
    EDFMM_LAUNCH_CHECK("k_near_targets");
    return EDFMM_OK;
}

EDFMM_API int edfmm_near_create(const void *centroids_dev, const void *areas_dev, const void *panel_vertices_dev,
                                int64_t n, double distance_factor, int quad_order, int depth, double k_e, int dtype,
                                void *stream, edfmm_near **out) {
    if (!out) return fail(EDFMM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n < 0 || depth < 0 || depth > 6) return fail(EDFMM_ERR_ARG, "bad n or depth (0..6)");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "bad dtype");
    if (n > 0 && (!centroids_dev || !areas_dev || !panel_vertices_dev)) return fail(EDFMM_ERR_ARG, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // owned until success: an early return (EDFMM_CUDA_TRY included) frees it
    std::unique_ptr<edfmm_near> owned(new edfmm_near());
    edfmm_near *h = owned.get();
    h->n = n;
    h->dtype = dtype;
    int rc = EDFMM_OK;
    auto done = [&](int r) {
        if (!r) *out = owned.release();
        return r;
    };
    if ((rc = h->row_off.reserve(sizeof(int32_t) * (n + 1)))) return done(rc);
    EDFMM_CUDA_TRY(cudaMemsetAsync(h->row_off.p, 0, sizeof(int32_t) * (n + 1), s));
    if (n <= 1) {
        EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
        return done(EDFMM_OK);
    }
    const double *c = static_cast<const double *>(centroids_dev);
    const double *a = static_cast<const double *>(areas_dev);
    DevBuf radii, bounds, cell, cnt, cell_off, items, tmp, total, rowcnt;
    if ((rc = radii.reserve(8 * n)) || (rc = bounds.reserve(8 * 8)) || (rc = cell.reserve(4 * n)) ||
        (rc = rowcnt.reserve(4 * n)) || (rc = total.reserve(8)))
        return done(rc);
    long long init[7] = {0, 0x7fffffffffffffffLL, 0x7fffffffffffffffLL, 0x7fffffffffffffffLL,
                         (long long)0x8000000000000000ULL, (long long)0x8000000000000000ULL,
                         (long long)0x8000000000000000ULL};
    EDFMM_CUDA_TRY(cudaMemcpyAsync(bounds.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
    long long *bd = dptr<long long>(bounds);
    k_radii_bounds<<<nb(n, 256), 256, 0, s>>>(c, a, n, dptr<double>(radii), (unsigned long long *)bd, bd + 1, bd + 4);
    EDFMM_LAUNCH_CHECK("k_radii_bounds");
    long long hb[7];
    EDFMM_CUDA_TRY(cudaMemcpyAsync(hb, bd, sizeof(hb), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    auto from_ord = [](long long o) {
        long long v = o >= 0 ? o : o ^ 0x7fffffffffffffffLL;
        double d;
        std::memcpy(&d, &v, 8);
        return d;
    };
    double rmax;
    std::memcpy(&rmax, &hb[0], 8);
    Grid g;
    double ext[3];
    for (int k = 0; k < 3; ++k) {
        g.org[k] = from_ord(hb[1 + k]);
        ext[k] = from_ord(hb[4 + k]) - g.org[k];
        if (!std::isfinite(ext[k]) || ext[k] < 0) ext[k] = 0;
    }
    // cell edge >= the largest possible threshold; cap the cell count at 2^22
    double hcell = std::max(2.0 * distance_factor * rmax, 1e-300);
    for (;;) {
        int64_t tot = 1;
        for (int k = 0; k < 3; ++k) {
            g.dim[k] = (int)std::min<double>(std::floor(ext[k] / hcell) + 1, 1 << 20);
            tot *= g.dim[k];
        }
        if (tot <= (1 << 22)) break;
        hcell *= 1.5;
    }
    g.h = hcell;
    const int64_t ncell = (int64_t)g.dim[0] * g.dim[1] * g.dim[2];
    if ((rc = cnt.reserve(4 * ncell)) || (rc = cell_off.reserve(4 * (ncell + 1))) || (rc = items.reserve(4 * n)) ||
        (rc = tmp.reserve(scan_tmp_bytes(std::max<int64_t>(ncell, n)))))
        return done(rc);
    EDFMM_CUDA_TRY(cudaMemsetAsync(cnt.p, 0, 4 * ncell, s));
    k_cell_count<<<nb(n, 256), 256, 0, s>>>(c, n, g, dptr<int32_t>(cell), dptr<int32_t>(cnt));
    EDFMM_LAUNCH_CHECK("k_cell_count");
    if ((rc = scan_exclusive(dptr<int32_t>(cnt), dptr<int32_t>(cell_off), ncell, dptr<int64_t>(total), tmp.p, s)))
        return done(rc);
    k_set_last32<<<1, 1, 0, s>>>(dptr<int32_t>(cell_off), ncell, dptr<int64_t>(total));
    EDFMM_LAUNCH_CHECK("k_set_last32");
    EDFMM_CUDA_TRY(cudaMemcpyAsync(cnt.p, cell_off.p, 4 * ncell, cudaMemcpyDeviceToDevice, s));
    k_cell_fill<<<nb(n, 256), 256, 0, s>>>(n, dptr<int32_t>(cell), dptr<int32_t>(cnt), dptr<int32_t>(items));
    EDFMM_LAUNCH_CHECK("k_cell_fill");
    k_near_scan<<<nb(n, 128), 128, 0, s>>>(c, dptr<double>(radii), n, g, distance_factor, dptr<int32_t>(cell_off),
                                           dptr<int32_t>(items), 0, dptr<int32_t>(rowcnt), nullptr, nullptr);
    EDFMM_LAUNCH_CHECK("k_near_scan");
    if ((rc = scan_exclusive(dptr<int32_t>(rowcnt), dptr<int32_t>(h->row_off), n, dptr<int64_t>(total), tmp.p, s)))
        return done(rc);
    k_set_last32<<<1, 1, 0, s>>>(dptr<int32_t>(h->row_off), n, dptr<int64_t>(total));
    EDFMM_LAUNCH_CHECK("k_set_last32");
    int64_t np = 0;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&np, total.p, 8, cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    if (np >= INT32_MAX) return done(fail(EDFMM_ERR_ARG, "too many near pairs"));
    h->n_pairs = np;
    if ((rc = h->cols.reserve(4 * std::max<int64_t>(np, 1))) || (rc = h->w64.reserve(8 * std::max<int64_t>(np, 1))) ||
        (rc = h->w.reserve((dtype == EDFMM_F64 ? 8 : 4) * std::max<int64_t>(np, 1))))
        return done(rc);
    if (np > 0) {
        k_near_scan<<<nb(n, 128), 128, 0, s>>>(c, dptr<double>(radii), n, g, distance_factor, dptr<int32_t>(cell_off),
                                               dptr<int32_t>(items), 1, nullptr, dptr<int32_t>(h->row_off),
                                               dptr<int32_t>(h->cols));
        EDFMM_LAUNCH_CHECK("k_near_scan");
        // rows sorted by column: the reference's per-target order
        std::vector<int32_t> hoff(n + 1);
        EDFMM_CUDA_TRY(cudaMemcpyAsync(hoff.data(), h->row_off.p, 4 * (n + 1), cudaMemcpyDeviceToHost, s));
        EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
        int64_t mx = 0;
        for (int64_t i = 0; i < n; ++i) mx = std::max<int64_t>(mx, hoff[i + 1] - hoff[i]);
        h->max_row = mx;
        if ((rc = sort_csr_rows(dptr<int32_t>(h->row_off), dptr<int32_t>(h->cols), n, mx, s))) return done(rc);
        k_near_weights_pairs<<<nb(np, 128), 128, 0, s>>>(c, a, static_cast<const double *>(panel_vertices_dev), n, np,
                                                         dptr<int32_t>(h->row_off), dptr<int32_t>(h->cols), quad_order,
                                                         depth, k_e, dptr<double>(h->w64));
        EDFMM_LAUNCH_CHECK("k_near_weights_pairs");
        if (dtype == EDFMM_F64) {
            EDFMM_CUDA_TRY(cudaMemcpyAsync(h->w.p, h->w64.p, 8 * np, cudaMemcpyDeviceToDevice, s));
        } else {
            k_cast<float><<<nb(np, 256), 256, 0, s>>>(dptr<double>(h->w64), dptr<float>(h->w), np);
            EDFMM_LAUNCH_CHECK("k_cast");
        }
    }
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    return done(EDFMM_OK);
}

EDFMM_API int edfmm_near_convert(const edfmm_near *src, int dtype, void *stream, edfmm_near **out) {
    if (!out) return fail(EDFMM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!src) return fail(EDFMM_ERR_ARG, "near handle is NULL");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "bad dtype");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // owned until success: an early return (EDFMM_CUDA_TRY included) frees it
    std::unique_ptr<edfmm_near> owned(new edfmm_near());
    edfmm_near *h = owned.get();
    h->n = src->n;
    h->n_pairs = src->n_pairs;
    h->max_row = src->max_row;
    h->dtype = dtype;
    int rc = EDFMM_OK;
    auto done = [&](int r) {
        if (!r) *out = owned.release();
        return r;
    };
    const int64_t np = src->n_pairs;
    if ((rc = h->row_off.reserve(sizeof(int32_t) * (h->n + 1)))) return done(rc);
    EDFMM_CUDA_TRY(cudaMemcpyAsync(h->row_off.p, src->row_off.p, sizeof(int32_t) * (h->n + 1),
                                   cudaMemcpyDeviceToDevice, s));
    if (src->cols.p) {
        if ((rc = h->cols.reserve(4 * std::max<int64_t>(np, 1))) ||
            (rc = h->w64.reserve(8 * std::max<int64_t>(np, 1))) ||
            (rc = h->w.reserve((dtype == EDFMM_F64 ? 8 : 4) * std::max<int64_t>(np, 1))))
            return done(rc);
    }
    if (np > 0) {
        EDFMM_CUDA_TRY(cudaMemcpyAsync(h->cols.p, src->cols.p, 4 * np, cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(h->w64.p, src->w64.p, 8 * np, cudaMemcpyDeviceToDevice, s));
        if (dtype == EDFMM_F64) {
            EDFMM_CUDA_TRY(cudaMemcpyAsync(h->w.p, src->w64.p, 8 * np, cudaMemcpyDeviceToDevice, s));
        } else {
            k_cast<float><<<nb(np, 256), 256, 0, s>>>(dptr<double>(src->w64), dptr<float>(h->w), np);
            EDFMM_LAUNCH_CHECK("k_cast");
        }
    }
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    return done(EDFMM_OK);
}

EDFMM_API int edfmm_near_destroy(edfmm_near *h) {
    delete h;
    return EDFMM_OK;
}

EDFMM_API int64_t edfmm_near_num_pairs(const edfmm_near *h) { return h ? h->n_pairs : -1; }

EDFMM_API int edfmm_near_export(const edfmm_near *h, int64_t *pairs_dev, double *weights_dev, void *stream) {
    if (!h) return fail(EDFMM_ERR_ARG, "near handle is NULL");
    if (h->n_pairs == 0) return EDFMM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<int32_t> off(h->n + 1), cols(h->n_pairs);
    EDFMM_CUDA_TRY(cudaMemcpyAsync(off.data(), h->row_off.p, 4 * (h->n + 1), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaMemcpyAsync(cols.data(), h->cols.p, 4 * h->n_pairs, cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    if (pairs_dev) {
        std::vector<int64_t> pr(2 * h->n_pairs);
        for (int64_t i = 0; i < h->n; ++i)
            for (int k = off[i]; k < off[i + 1]; ++k) {
                pr[2 * k] = i;
                pr[2 * k + 1] = cols[k];
            }
        EDFMM_CUDA_TRY(cudaMemcpyAsync(pairs_dev, pr.data(), 8 * pr.size(), cudaMemcpyHostToDevice, s));
    }
    if (weights_dev)
        EDFMM_CUDA_TRY(cudaMemcpyAsync(weights_dev, h->w64.p, 8 * h->n_pairs, cudaMemcpyDeviceToDevice, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    return EDFMM_OK;
}

EDFMM_API int edfmm_near_apply(const edfmm_near *h, const void *sigma_dev, const void *v_in_dev, void *v_out_dev,
                               void *stream) {
    if (!h) return fail(EDFMM_ERR_ARG, "near handle is NULL");
    if (h->n == 0) return EDFMM_OK;
    if (!sigma_dev || !v_out_dev) return fail(EDFMM_ERR_ARG, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (h->dtype == EDFMM_F64)
        k_near_apply<double><<<nb(h->n, 256), 256, 0, s>>>(h->n, dptr<int32_t>(h->row_off), dptr<int32_t>(h->cols),
                                                           dptr<double>(h->w), static_cast<const double *>(sigma_dev),
                                                           static_cast<const double *>(v_in_dev),
                                                           static_cast<double *>(v_out_dev));
    else
        k_near_apply<float><<<nb(h->n, 256), 256, 0, s>>>(h->n, dptr<int32_t>(h->row_off), dptr<int32_t>(h->cols),
                                                          dptr<float>(h->w), static_cast<const float *>(sigma_dev),
                                                          static_cast<const float *>(v_in_dev),
                                                          static_cast<float *>(v_out_dev));
    EDFMM_LAUNCH_CHECK("k_near_apply");
    return EDFMM_OK;
}

EDFMM_API int edfmm_near_quadrature_matvec(const void *v_far_dev, const void *sigma_dev, const void *centroids_dev,
                                           const void *areas_dev, const void *panel_vertices_dev,
                                           const int32_t *row_off_dev, const int32_t *cols_dev, int64_t n,
                                           double k_e, int quad_order, int dtype, void *v_out_dev, void *stream) {
    if (n < 0) return fail(EDFMM_ERR_ARG, "n must be >= 0");
    if (n == 0) return EDFMM_OK;
    if (!v_far_dev || !sigma_dev || !centroids_dev || !areas_dev || !panel_vertices_dev || !row_off_dev || !cols_dev ||
        !v_out_dev)
        return fail(EDFMM_ERR_ARG, "NULL argument");
    const int q = quad_order <= 1 ? 1 : 3;
    if (quad_order > 2) return fail(EDFMM_ERR_UNSUPPORTED, "quad_order must be 1 or 2");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (dtype == EDFMM_F64)
        k_near_onthefly<double><<<nb(n, kNearRows), kNearThreads, 0, s>>>(
            n, row_off_dev, cols_dev, (const double *)centroids_dev, (const double *)areas_dev, (const double *)sigma_dev,
            (const double *)panel_vertices_dev, q, k_e, (const double *)v_far_dev, (double *)v_out_dev);
    else
        k_near_onthefly<float><<<nb(n, kNearRows), kNearThreads, 0, s>>>(
            n, row_off_dev, cols_dev, (const float *)centroids_dev, (const float *)areas_dev, (const float *)sigma_dev,
            (const float *)panel_vertices_dev, q, (float)k_e, (const float *)v_far_dev, (float *)v_out_dev);
    EDFMM_LAUNCH_CHECK("k_near_onthefly");
    return EDFMM_OK;
}

EDFMM_API int edfmm_near_rows(const edfmm_near *h, const int32_t **row_off_dev, const int32_t **cols_dev) {
    if (!h) return fail(EDFMM_ERR_ARG, "near handle is NULL");
    if (row_off_dev) *row_off_dev = dptr<int32_t>(h->row_off);
    if (cols_dev) *cols_dev = dptr<int32_t>(h->cols);
    return EDFMM_OK;
}

// V(x) = sum_k K_E q_k / max(|x - r_k|, 1e-12) (core/bem.py:291-320)
}  // extern "C"

namespace edfmm {
namespace {
template <typename T>
__global__ void k_point_charges(const T *pts, int64_t n, const double *charges, int nq, double ke, T *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
    const double x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
    for (int k = 0; k < nq; ++k) {
        const double dx = x - charges[4 * k + 1], dy = y - charges[4 * k + 2], dz = z - charges[4 * k + 3];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        r = r < 1e-12 ? 1e-12 : r;
        acc += ke * charges[4 * k] / r;
    }
    out[i] = (T)acc;
}
}  // namespace
}  // namespace edfmm

extern "C" EDFMM_API int edfmm_point_charge_potential(const void *points_dev, int64_t n, const double *charges_dev,
                                                      int n_charges, double k_e, int dtype, void *out_dev,
                                                      void *stream) {
    if (n < 0 || n_charges < 0) return fail(EDFMM_ERR_ARG, "bad sizes");
    if (n == 0) return EDFMM_OK;
    if (!points_dev || !out_dev || (n_charges > 0 && !charges_dev)) return fail(EDFMM_ERR_ARG, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (dtype == EDFMM_F64)
        k_point_charges<double><<<nb(n, 256), 256, 0, s>>>((const double *)points_dev, n, charges_dev, n_charges, k_e,
                                                           (double *)out_dev);
    else
        k_point_charges<float><<<nb(n, 256), 256, 0, s>>>((const float *)points_dev, n, charges_dev, n_charges, k_e,
                                                          (float *)out_dev);
    EDFMM_LAUNCH_CHECK("k_point_charges");
    return EDFMM_OK;
}
