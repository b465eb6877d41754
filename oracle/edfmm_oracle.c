/*
 * edfmm_oracle.c -- CPU oracle for the FMM-accelerated single-layer BEM
 * matvec.  TEST INFRASTRUCTURE ONLY: this file is the checker that the
 * CUDA path is compared against (by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py).  Nothing in electrodrive_gb300/ links,
 * imports or calls it.
 *
 * Parity status: the tree and interaction-list restatements are pinned
 * bit-exactly against golden fixtures written by the reference itself
 * (tests/golden/make_golden.py); the far field is the analytic
 * solid-harmonic FMM that the reference's least-squares translation
 * operators approximate, pinned against FP64 direct summation and against
 * the reference FMM's own potentials within the reference's error budget.
 *
 * Restated reference behaviour (file:line inside the reference project):
 *   - adaptive octree:       electrodrive/fmm3d/tree.py:801-960
 *       tight bbox per node (tree.py:874-876), leaf rule (tree.py:895-897),
 *       strict '>' octant split (tree.py:914-919), stable counting sort
 *       (tree.py:921-939), DFS pre-order node numbering (tree.py:878-889),
 *       node radius = ||half|| * (1 + 1e-12) (tree.py:331)
 *   - dual-tree lists:       electrodrive/fmm3d/interaction_lists.py:374-528
 *       MAC (interaction_lists.py:273-297), refinement side (:306-337),
 *       dedup + sort by (tgt, src) (:474-485)
 *   - P2P near field:        electrodrive/fmm3d/kernels_cpu.py:83-153, :286-345
 *       q / max(|x_t - x_s|, eps) with the diagonal removed only in the
 *       self leaf pair
 *   - direct sum:            electrodrive/fmm3d/sanity_suite.py:83-121
 *   - matvec assembly:       electrodrive/fmm3d/bem_fmm.py:460-594
 *       q = sigma * area, K_E * (phi_far + phi_near), original order,
 *       + self_integrals * sigma * area, non-finite -> 0
 *
 * torch's CPU vector norm of a 3-vector rounds as
 * sqrt(fma(z, z, fma(y, y, x * x))) in the tensor's dtype; the MAC and the
 * node radii below use exactly that so decisions match bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* Tree                                                                */
/* ------------------------------------------------------------------ */

typedef struct {
    int is_f64;
    int64_t n_points;
    int64_t n_nodes, cap_nodes;
    int leaf_size, max_depth;
    int n_warn_max_depth;
    /* per node (DFS pre-order) */
    double *center;   /* 3 per node, values exactly representable in dtype */
    double *half;     /* 3 per node */
    double *radius;   /* 1 per node */
    int32_t *level;
    int64_t *parent;
    int64_t *children; /* 8 per node */
    int64_t *start, *end;
    uint8_t *is_leaf;
    int64_t *index_map; /* tree position -> original index */
} orc_tree;

static void tree_grow(orc_tree *t) {
    if (t->n_nodes < t->cap_nodes) return;
    int64_t c = t->cap_nodes ? t->cap_nodes * 2 : 1024;
    t->center = realloc(t->center, sizeof(double) * 3 * c);
    t->half = realloc(t->half, sizeof(double) * 3 * c);
    t->radius = realloc(t->radius, sizeof(double) * c);
    t->level = realloc(t->level, sizeof(int32_t) * c);
    t->parent = realloc(t->parent, sizeof(int64_t) * c);
    t->children = realloc(t->children, sizeof(int64_t) * 8 * c);
    t->start = realloc(t->start, sizeof(int64_t) * c);
    t->end = realloc(t->end, sizeof(int64_t) * c);
    t->is_leaf = realloc(t->is_leaf, c);
    t->cap_nodes = c;
}

typedef struct {
    orc_tree *t;
    const float *pf;
    const double *pd;
    int64_t *idx;
    int64_t *scratch;
} build_ctx;

static inline double coord(const build_ctx *b, int64_t i, int a) {
    return b->t->is_f64 ? b->pd[3 * i + a] : (double)b->pf[3 * i + a];
}

static int64_t build_node(build_ctx *b, int64_t start, int64_t end, int level, int64_t parent) {
    orc_tree *t = b->t;
    double mn[3], mx[3], c[3], h[3];
    for (int a = 0; a < 3; ++a) {
        mn[a] = INFINITY;
        mx[a] = -INFINITY;
    }
    for (int64_t i = start; i < end; ++i) {
        int64_t j = b->idx[i];
        for (int a = 0; a < 3; ++a) {
            double v = coord(b, j, a);
            if (v < mn[a]) mn[a] = v;
            if (v > mx[a]) mx[a] = v;
        }
    }
    /* center = 0.5 * (min + max); half = clamp(0.5 * (max - min), 0) in dtype */
    for (int a = 0; a < 3; ++a) {
        if (t->is_f64) {
            c[a] = 0.5 * (mn[a] + mx[a]);
            double hh = 0.5 * (mx[a] - mn[a]);
            h[a] = hh < 0.0 ? 0.0 : hh;
        } else {
            float s = (float)mn[a] + (float)mx[a];
            c[a] = (double)(0.5f * s);
            float d = (float)mx[a] - (float)mn[a];
            float hh = 0.5f * d;
            h[a] = (double)(hh < 0.0f ? 0.0f : hh);
        }
    }
    tree_grow(t);
    int64_t me = t->n_nodes++;
    for (int a = 0; a < 3; ++a) {
        t->center[3 * me + a] = c[a];
        t->half[3 * me + a] = h[a];
    }
    if (t->is_f64) {
        double r = sqrt(fma(h[2], h[2], fma(h[1], h[1], h[0] * h[0])));
        t->radius[me] = r * (1.0 + 1e-12);
    } else {
        float hx = (float)h[0], hy = (float)h[1], hz = (float)h[2];
        float r = sqrtf(fmaf(hz, hz, fmaf(hy, hy, hx * hx)));
        t->radius[me] = (double)(r * (float)(1.0 + 1e-12));
    }
    t->level[me] = level;
    t->parent[me] = parent;
    for (int o = 0; o < 8; ++o) t->children[8 * me + o] = -1;
    t->start[me] = start;
    t->end[me] = end;
    t->is_leaf[me] = 1;

    int64_t n = end - start;
    double hmax = h[0];
    if (h[1] > hmax) hmax = h[1];
    if (h[2] > hmax) hmax = h[2];
    int degenerate = hmax < 1e-7;
    if (n <= t->leaf_size || level >= t->max_depth || degenerate) {
        if (level >= t->max_depth && n > t->leaf_size && !degenerate) t->n_warn_max_depth++;
        return me;
    }
    int64_t cnt[8] = {0}, off[8];
    /* octant id = (x > cx) + 2 (y > cy) + 4 (z > cz); comparisons in dtype */
    for (int64_t i = start; i < end; ++i) {
        int64_t j = b->idx[i];
        int o = (coord(b, j, 0) > c[0]) + 2 * (coord(b, j, 1) > c[1]) + 4 * (coord(b, j, 2) > c[2]);
        cnt[o]++;
    }
    int64_t acc = 0;
    for (int o = 0; o < 8; ++o) {
        off[o] = acc;
        acc += cnt[o];
    }
    int64_t cur[8];
    memcpy(cur, off, sizeof(cur));
    for (int64_t i = start; i < end; ++i) {
        int64_t j = b->idx[i];
        int o = (coord(b, j, 0) > c[0]) + 2 * (coord(b, j, 1) > c[1]) + 4 * (coord(b, j, 2) > c[2]);
        b->scratch[start + cur[o]++] = j;
    }
    memcpy(b->idx + start, b->scratch + start, sizeof(int64_t) * n);
    t->is_leaf[me] = 0;
    for (int o = 0; o < 8; ++o) {
        if (cnt[o] == 0) continue;
        int64_t ch = build_node(b, start + off[o], start + off[o] + cnt[o], level + 1, me);
        t->children[8 * me + o] = ch;
    }
    return me;
}

ORC_API void *orc_tree_build(const void *points, int64_t n, int is_f64, int leaf_size, int max_depth) {
    orc_tree *t = calloc(1, sizeof(orc_tree));
    t->is_f64 = is_f64;
    t->n_points = n;
    t->leaf_size = leaf_size;
    t->max_depth = max_depth;
    t->index_map = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) t->index_map[i] = i;
    if (n > 0) {
        build_ctx b;
        b.t = t;
        b.pf = is_f64 ? NULL : (const float *)points;
        b.pd = is_f64 ? (const double *)points : NULL;
        b.idx = t->index_map;
        b.scratch = malloc(sizeof(int64_t) * n);
        build_node(&b, 0, n, 0, -1);
        free(b.scratch);
    }
    return t;
}

ORC_API int64_t orc_tree_n_nodes(void *h) { return ((orc_tree *)h)->n_nodes; }
ORC_API int orc_tree_n_depth_warnings(void *h) { return ((orc_tree *)h)->n_warn_max_depth; }

/* Export in the reference's SoA layout (tree.py:286-348). */
ORC_API void orc_tree_export(void *h, int64_t *index_map, double *centers, double *half_extents,
                             double *radii, int32_t *levels, int64_t *parents, int64_t *children,
                             int64_t *ranges, uint8_t *is_leaf) {
    orc_tree *t = h;
    int64_t m = t->n_nodes;
    if (index_map) memcpy(index_map, t->index_map, sizeof(int64_t) * t->n_points);
    if (centers) memcpy(centers, t->center, sizeof(double) * 3 * m);
    if (half_extents) memcpy(half_extents, t->half, sizeof(double) * 3 * m);
    if (radii) memcpy(radii, t->radius, sizeof(double) * m);
    if (levels) memcpy(levels, t->level, sizeof(int32_t) * m);
    if (parents) memcpy(parents, t->parent, sizeof(int64_t) * m);
    if (children) memcpy(children, t->children, sizeof(int64_t) * 8 * m);
    if (ranges)
        for (int64_t i = 0; i < m; ++i) {
            ranges[2 * i] = t->start[i];
            ranges[2 * i + 1] = t->end[i];
        }
    if (is_leaf) memcpy(is_leaf, t->is_leaf, m);
}

ORC_API void orc_tree_free(void *h) {
    orc_tree *t = h;
    if (!t) return;
    free(t->center);
    free(t->half);
    free(t->radius);
    free(t->level);
    free(t->parent);
    free(t->children);
    free(t->start);
    free(t->end);
    free(t->is_leaf);
    free(t->index_map);
    free(t);
}

/* ------------------------------------------------------------------ */
/* Interaction lists                                                   */
/* ------------------------------------------------------------------ */

typedef struct {
    int64_t n_p2p, n_m2l;
    int64_t *p2p; /* (src, tgt) pairs, sorted by (tgt, src) */
    int64_t *m2l;
} orc_lists;

typedef struct {
    int64_t *v;
    int64_t n, cap;
} vec2;

static void vpush(vec2 *v, int64_t a, int64_t b) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 4096;
        v->v = realloc(v->v, sizeof(int64_t) * 2 * v->cap);
    }
    v->v[2 * v->n] = a;
    v->v[2 * v->n + 1] = b;
    v->n++;
}

static double node_dist(const orc_tree *t, int64_t s, int64_t g) {
    if (t->is_f64) {
        double dx = t->center[3 * s] - t->center[3 * g];
        double dy = t->center[3 * s + 1] - t->center[3 * g + 1];
        double dz = t->center[3 * s + 2] - t->center[3 * g + 2];
        return sqrt(fma(dz, dz, fma(dy, dy, dx * dx)));
    } else {
        float dx = (float)t->center[3 * s] - (float)t->center[3 * g];
        float dy = (float)t->center[3 * s + 1] - (float)t->center[3 * g + 1];
        float dz = (float)t->center[3 * s + 2] - (float)t->center[3 * g + 2];
        return (double)sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
    }
}

static double node_diam(const orc_tree *t, int64_t i) {
    if (t->is_f64) return 2.0 * t->radius[i];
    return (double)(2.0f * (float)t->radius[i]);
}

static int cmp_tgt_src(const void *a, const void *b) {
    const int64_t *x = a, *y = b;
    if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
    if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
    return 0;
}

ORC_API void *orc_lists_build(void *th, double theta) {
    orc_tree *t = th;
    orc_lists *L = calloc(1, sizeof(orc_lists));
    if (t->n_nodes == 0) return L;
    vec2 p2p = {0}, m2l = {0}, stack = {0};
    vpush(&stack, 0, 0);
    while (stack.n > 0) {
        stack.n--;
        int64_t s = stack.v[2 * stack.n], g = stack.v[2 * stack.n + 1];
        int sl = t->is_leaf[s], gl = t->is_leaf[g];
        if (s != g) {
            double dist = node_dist(t, s, g);
            if (dist != 0.0) {
                double ds = node_diam(t, s), dg = node_diam(t, g);
                double mx = ds >= dg ? ds : dg;
                if (mx / dist < theta) {
                    vpush(&m2l, s, g);
                    continue;
                }
            }
        }
        if (sl && gl) {
            vpush(&p2p, s, g);
            continue;
        }
        int refine_src;
        if (sl && !gl)
            refine_src = 0;
        else if (gl && !sl)
            refine_src = 1;
        else {
            double ds = node_diam(t, s), dg = node_diam(t, g);
            if (ds > dg * 1.01)
                refine_src = 1;
            else if (dg > ds * 1.01)
                refine_src = 0;
            else {
                int64_t ns = t->end[s] - t->start[s], ng = t->end[g] - t->start[g];
                refine_src = ns >= ng;
            }
        }
        int64_t node = refine_src ? s : g;
        for (int o = 0; o < 8; ++o) {
            int64_t c = t->children[8 * node + o];
            if (c < 0) continue;
            if (refine_src)
                vpush(&stack, c, g);
            else
                vpush(&stack, s, c);
        }
    }
    qsort(p2p.v, p2p.n, 2 * sizeof(int64_t), cmp_tgt_src);
    qsort(m2l.v, m2l.n, 2 * sizeof(int64_t), cmp_tgt_src);
    L->n_p2p = p2p.n;
    L->p2p = p2p.v;
    L->n_m2l = m2l.n;
    L->m2l = m2l.v;
    free(stack.v);
    return L;
}

ORC_API int64_t orc_lists_n_p2p(void *h) { return ((orc_lists *)h)->n_p2p; }
ORC_API int64_t orc_lists_n_m2l(void *h) { return ((orc_lists *)h)->n_m2l; }
ORC_API void orc_lists_export(void *h, int64_t *p2p, int64_t *m2l) {
    orc_lists *L = h;
    if (p2p && L->n_p2p) memcpy(p2p, L->p2p, sizeof(int64_t) * 2 * L->n_p2p);
    if (m2l && L->n_m2l) memcpy(m2l, L->m2l, sizeof(int64_t) * 2 * L->n_m2l);
}
ORC_API void orc_lists_free(void *h) {
    orc_lists *L = h;
    if (!L) return;
    free(L->p2p);
    free(L->m2l);
    free(L);
}

/* ------------------------------------------------------------------ */
/* P2P and direct sums                                                 */
/* ------------------------------------------------------------------ */

/*
 * Near field over (src, tgt) leaf pairs on tree-order points, accumulated in
 * double.  eps = machine epsilon of the working dtype
 * (kernels_cpu.py:140-142).
 */
ORC_API void orc_p2p(const double *pts, const double *q, int64_t n, const int64_t *ranges,
                     const int64_t *pairs, int64_t n_pairs, double eps, double *phi) {
    memset(phi, 0, sizeof(double) * n);
    /* pairs are sorted by tgt: parallelise over targets' contiguous blocks */
    int64_t *blk = malloc(sizeof(int64_t) * (n_pairs + 1));
    int64_t nb = 0;
    for (int64_t k = 0; k < n_pairs; ++k)
        if (k == 0 || pairs[2 * k + 1] != pairs[2 * k - 1]) blk[nb++] = k;
    blk[nb] = n_pairs;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t b = 0; b < nb; ++b) {
        for (int64_t k = blk[b]; k < blk[b + 1]; ++k) {
            int64_t s = pairs[2 * k], g = pairs[2 * k + 1];
            int64_t s0 = ranges[2 * s], s1 = ranges[2 * s + 1];
            int64_t t0 = ranges[2 * g], t1 = ranges[2 * g + 1];
            for (int64_t i = t0; i < t1; ++i) {
                double acc = 0.0;
                for (int64_t j = s0; j < s1; ++j) {
                    if (s == g && i == j) continue;
                    double dx = pts[3 * i] - pts[3 * j], dy = pts[3 * i + 1] - pts[3 * j + 1],
                           dz = pts[3 * i + 2] - pts[3 * j + 2];
                    double r = sqrt(dx * dx + dy * dy + dz * dz);
                    if (r < eps) r = eps;
                    acc += q[j] / r;
                }
                phi[i] += acc;
            }
        }
    }
    free(blk);
}

/* phi(t) = sum_{j != idx(t)} q_j / |x_t - x_j| in double (sanity_suite.py:83-121). */
ORC_API void orc_direct(const double *pts, const double *q, int64_t n, const int64_t *tgt_idx,
                        int64_t n_tgt, double *phi) {
#pragma omp parallel for schedule(static)
    for (int64_t a = 0; a < n_tgt; ++a) {
        int64_t i = tgt_idx[a];
        double x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2], acc = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = x - pts[3 * j], dy = y - pts[3 * j + 1], dz = z - pts[3 * j + 2];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > 0.0) acc += q[j] / sqrt(r2);
        }
        phi[a] = acc;
    }
}

/* Dense single-layer operator restated from core/bem_kernel.py:157-230:
 * V_i = sum_{j != i} K_E * sigma_j * A_j * rsqrt(max(r^2, 1e-24))
 *       + self_integrals[i] * sigma_i * A_i                                  */
ORC_API void orc_dense_matvec(const double *c, const double *sigma, const double *areas,
                              const double *self_int, int64_t n, double ke, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = c[3 * i] - c[3 * j], dy = c[3 * i + 1] - c[3 * j + 1], dz = c[3 * i + 2] - c[3 * j + 2];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < 1e-24) r2 = 1e-24;
            acc += ke / sqrt(r2) * sigma[j] * areas[j];
        }
        double d = self_int ? self_int[i] : 0.0;
        out[i] = acc + d * sigma[i] * areas[i];
    }
}

/* ------------------------------------------------------------------ */
/* Analytic far field (FP64)                                           */
/* ------------------------------------------------------------------ */
/*
 * Complex solid harmonics with Condon-Shortley phase, stored for m >= 0,
 * index (n, m) -> n (n + 1) / 2 + m:
 *   R_n^m(v) = |v|^n P_n^m(cos t) e^{i m phi} / (n + m)!
 *   I_n^m(v) = (n - m)! P_n^m(cos t) e^{i m phi} / |v|^{n + 1}
 * with X_n^{-m} = (-1)^m conj(X_n^m).  Then
 *   1/|x - y| = sum_{n,m} conj(R_n^m(y)) I_n^m(x)           (|y| < |x|)
 *   M2M: M'_n^m = sum_{k,l} conj(R_k^l(c - c')) M_{n-k}^{m-l}
 *   M2L: L_n^m  = (-1)^(n+m) sum_{k,l} M_k^l I_{n+k}^{l-m}(c_L - c_M)
 *   L2L: L'_j^u = sum_{k,l} L_{j+k}^{u+l} R_k^l(c' - c)
 *   L2P: phi(x) = sum_{n,m} L_n^m R_n^m(x - c)
 * Coefficients are stored scaled by the node radius a:
 *   Mhat_n = M_n / a^n, Lhat_n = L_n a^n.
 */
typedef struct {
    double re, im;
} cplx;

#define ORC_PMAX 20
#define TRI(n, m) ((n) * ((n) + 1) / 2 + (m))

static void regular_harmonics(double x, double y, double z, int p, cplx *R) {
    double r2 = x * x + y * y + z * z;
    R[0].re = 1.0;
    R[0].im = 0.0;
    for (int m = 1; m <= p; ++m) {
        cplx a = R[TRI(m - 1, m - 1)];
        double s = -1.0 / (2.0 * m);
        R[TRI(m, m)].re = s * (x * a.re - y * a.im);
        R[TRI(m, m)].im = s * (x * a.im + y * a.re);
    }
    for (int m = 0; m <= p; ++m)
        for (int n = m + 1; n <= p; ++n) {
            cplx a = R[TRI(n - 1, m)];
            cplx b = n - 2 >= m ? R[TRI(n - 2, m)] : (cplx){0, 0};
            double d = 1.0 / ((double)(n + m) * (n - m));
            R[TRI(n, m)].re = ((2 * n - 1) * z * a.re - r2 * b.re) * d;
            R[TRI(n, m)].im = ((2 * n - 1) * z * a.im - r2 * b.im) * d;
        }
}

static void irregular_harmonics(double x, double y, double z, int p, cplx *I) {
    double r2 = x * x + y * y + z * z, ir2 = 1.0 / r2;
    I[0].re = 1.0 / sqrt(r2);
    I[0].im = 0.0;
    for (int m = 1; m <= p; ++m) {
        cplx a = I[TRI(m - 1, m - 1)];
        double s = -(2.0 * m - 1.0) * ir2;
        I[TRI(m, m)].re = s * (x * a.re - y * a.im);
        I[TRI(m, m)].im = s * (x * a.im + y * a.re);
    }
    for (int m = 0; m <= p; ++m)
        for (int n = m + 1; n <= p; ++n) {
            cplx a = I[TRI(n - 1, m)];
            cplx b = n - 2 >= m ? I[TRI(n - 2, m)] : (cplx){0, 0};
            double c2 = (double)(n - 1 + m) * (n - 1 - m);
            I[TRI(n, m)].re = ((2 * n - 1) * z * a.re - c2 * b.re) * ir2;
            I[TRI(n, m)].im = ((2 * n - 1) * z * a.im - c2 * b.im) * ir2;
        }
}

/* X_n^m for any sign of m from m >= 0 storage. */
static inline cplx harm_at(const cplx *X, int n, int m) {
    if (m >= 0) return X[TRI(n, m)];
    cplx v = X[TRI(n, -m)];
    if ((-m) & 1) return (cplx){-v.re, v.im};
    return (cplx){v.re, -v.im};
}

static inline cplx cmul(cplx a, cplx b) { return (cplx){a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline cplx conjc(cplx a) { return (cplx){a.re, -a.im}; }

static inline double node_scale(const orc_tree *t, int64_t i) { return t->radius[i] > 0 ? t->radius[i] : 1.0; }

/*
 * Full FMM matvec in FP64 on an oracle tree + lists.
 *   sigma, areas, self_int: original order (self_int may be NULL)
 *   reference_pair_order != 0 applies each listed (src, tgt) M2L pair as
 *   L[src] += M2L(M[tgt]), which is how the reference unpacks its pairs
 *   (multipole_operators.py:1671).
 *   out: original order.  phi_far_tree / phi_near_tree (tree order, may be NULL).
 */
ORC_API int orc_fmm_matvec(void *th, void *lh, const double *points_orig, const double *sigma,
                           const double *areas, const double *self_int, int p, double ke,
                           int reference_pair_order, double eps, double *out, double *phi_far_tree,
                           double *phi_near_tree) {
    orc_tree *t = th;
    orc_lists *L = lh;
    int64_t n = t->n_points, m = t->n_nodes;
    if (p < 0 || p > ORC_PMAX / 2) return -1;
    if (n == 0) return 0;
    int nc = (p + 1) * (p + 2) / 2;
    double *pts = malloc(sizeof(double) * 3 * n);
    double *q = malloc(sizeof(double) * n);
    for (int64_t i = 0; i < n; ++i) {
        int64_t o = t->index_map[i];
        for (int a = 0; a < 3; ++a) pts[3 * i + a] = points_orig[3 * o + a];
        q[i] = sigma[o] * areas[o];
    }
    cplx *Mc = calloc((size_t)m * nc, sizeof(cplx));
    cplx *Lc = calloc((size_t)m * nc, sizeof(cplx));
    /* P2M */
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < m; ++i) {
        if (!t->is_leaf[i]) continue;
        cplx R[ORC_PMAX * ORC_PMAX];
        double a = node_scale(t, i), ia = 1.0 / a;
        for (int64_t j = t->start[i]; j < t->end[i]; ++j) {
            regular_harmonics((pts[3 * j] - t->center[3 * i]) * ia, (pts[3 * j + 1] - t->center[3 * i + 1]) * ia,
                              (pts[3 * j + 2] - t->center[3 * i + 2]) * ia, p, R);
            for (int c = 0; c < nc; ++c) {
                Mc[i * nc + c].re += q[j] * R[c].re;
                Mc[i * nc + c].im -= q[j] * R[c].im;
            }
        }
    }
    /* M2M, deepest level first */
    int maxlev = 0;
    for (int64_t i = 0; i < m; ++i)
        if (t->level[i] > maxlev) maxlev = t->level[i];
    for (int lev = maxlev - 1; lev >= 0; --lev) {
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t i = 0; i < m; ++i) {
            if (t->level[i] != lev || t->is_leaf[i]) continue;
            double aP = node_scale(t, i);
            cplx R[ORC_PMAX * ORC_PMAX];
            for (int o = 0; o < 8; ++o) {
                int64_t ch = t->children[8 * i + o];
                if (ch < 0) continue;
                double aC = node_scale(t, ch), ratio = aC / aP;
                regular_harmonics((t->center[3 * ch] - t->center[3 * i]) / aP,
                                  (t->center[3 * ch + 1] - t->center[3 * i + 1]) / aP,
                                  (t->center[3 * ch + 2] - t->center[3 * i + 2]) / aP, p, R);
                for (int nn = 0; nn <= p; ++nn)
                    for (int mm = 0; mm <= nn; ++mm) {
                        cplx acc = {0, 0};
                        for (int k = 0; k <= nn; ++k) {
                            double sc = pow(ratio, nn - k);
                            for (int l = -k; l <= k; ++l) {
                                int j = nn - k, u = mm - l;
                                if (u < -j || u > j) continue;
                                cplx v = cmul(conjc(harm_at(R, k, l)), harm_at(Mc + ch * nc, j, u));
                                acc.re += sc * v.re;
                                acc.im += sc * v.im;
                            }
                        }
                        Mc[i * nc + TRI(nn, mm)].re += acc.re;
                        Mc[i * nc + TRI(nn, mm)].im += acc.im;
                    }
            }
        }
    }
    /* M2L: per-target rows of the (tgt, src)-sorted list */
    int64_t np = L->n_m2l;
    int64_t *tg = malloc(sizeof(int64_t) * (np > 0 ? np : 1));
    int64_t *sr = malloc(sizeof(int64_t) * (np > 0 ? np : 1));
    for (int64_t k = 0; k < np; ++k) {
        if (reference_pair_order) {
            tg[k] = L->m2l[2 * k];
            sr[k] = L->m2l[2 * k + 1];
        } else {
            sr[k] = L->m2l[2 * k];
            tg[k] = L->m2l[2 * k + 1];
        }
    }
    /* group by target (rows are contiguous in the sorted list for the
       correct order; for the swapped order use a per-target CSR) */
    int64_t *cnt = calloc(m + 1, sizeof(int64_t));
    for (int64_t k = 0; k < np; ++k) cnt[tg[k] + 1]++;
    for (int64_t i = 0; i < m; ++i) cnt[i + 1] += cnt[i];
    int64_t *rows = malloc(sizeof(int64_t) * (np > 0 ? np : 1));
    int64_t *cur = malloc(sizeof(int64_t) * (m + 1));
    memcpy(cur, cnt, sizeof(int64_t) * (m + 1));
    for (int64_t k = 0; k < np; ++k) rows[cur[tg[k]]++] = sr[k];
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t g = 0; g < m; ++g) {
        cplx I[2 * ORC_PMAX * ORC_PMAX];
        double aL = node_scale(t, g);
        for (int64_t k = cnt[g]; k < cnt[g + 1]; ++k) {
            int64_t s = rows[k];
            double aM = node_scale(t, s);
            double tx = t->center[3 * g] - t->center[3 * s], ty = t->center[3 * g + 1] - t->center[3 * s + 1],
                   tz = t->center[3 * g + 2] - t->center[3 * s + 2];
            double rho = sqrt(tx * tx + ty * ty + tz * tz);
            irregular_harmonics(tx / rho, ty / rho, tz / rho, 2 * p, I);
            double fa[ORC_PMAX + 1], fb[ORC_PMAX + 1];
            fa[0] = fb[0] = 1.0;
            for (int j = 1; j <= p; ++j) {
                fa[j] = fa[j - 1] * (aM / rho);
                fb[j] = fb[j - 1] * (aL / rho);
            }
            for (int nn = 0; nn <= p; ++nn)
                for (int mm = 0; mm <= nn; ++mm) {
                    cplx acc = {0, 0};
                    for (int kk = 0; kk <= p; ++kk)
                        for (int l = -kk; l <= kk; ++l) {
                            cplx v = cmul(harm_at(Mc + s * nc, kk, l), harm_at(I, nn + kk, l - mm));
                            acc.re += fa[kk] * v.re;
                            acc.im += fa[kk] * v.im;
                        }
                    double sg = ((nn + mm) & 1) ? -1.0 : 1.0;
                    double f = sg * fb[nn] / rho;
                    Lc[g * nc + TRI(nn, mm)].re += f * acc.re;
                    Lc[g * nc + TRI(nn, mm)].im += f * acc.im;
                }
        }
    }
    free(tg);
    free(sr);
    free(rows);
    free(cur);
    free(cnt);
    /* L2L, root level first */
    for (int lev = 1; lev <= maxlev; ++lev) {
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t i = 0; i < m; ++i) {
            if (t->level[i] != lev) continue;
            int64_t par = t->parent[i];
            double aP = node_scale(t, par), aC = node_scale(t, i), ratio = aC / aP;
            cplx R[ORC_PMAX * ORC_PMAX];
            regular_harmonics((t->center[3 * i] - t->center[3 * par]) / aP,
                              (t->center[3 * i + 1] - t->center[3 * par + 1]) / aP,
                              (t->center[3 * i + 2] - t->center[3 * par + 2]) / aP, p, R);
            for (int j = 0; j <= p; ++j) {
                double sc = pow(ratio, j);
                for (int u = 0; u <= j; ++u) {
                    cplx acc = {0, 0};
                    for (int k = 0; k + j <= p; ++k)
                        for (int l = -k; l <= k; ++l) {
                            int nn = j + k, mm = u + l;
                            if (mm < -nn || mm > nn) continue;
                            cplx v = cmul(harm_at(Lc + par * nc, nn, mm), harm_at(R, k, l));
                            acc.re += v.re;
                            acc.im += v.im;
                        }
                    Lc[i * nc + TRI(j, u)].re += sc * acc.re;
                    Lc[i * nc + TRI(j, u)].im += sc * acc.im;
                }
            }
        }
    }
    /* L2P + P2P */
    double *far = malloc(sizeof(double) * n);
    double *near = malloc(sizeof(double) * n);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < m; ++i) {
        if (!t->is_leaf[i]) continue;
        cplx R[ORC_PMAX * ORC_PMAX];
        double a = node_scale(t, i), ia = 1.0 / a;
        for (int64_t j = t->start[i]; j < t->end[i]; ++j) {
            regular_harmonics((pts[3 * j] - t->center[3 * i]) * ia, (pts[3 * j + 1] - t->center[3 * i + 1]) * ia,
                              (pts[3 * j + 2] - t->center[3 * i + 2]) * ia, p, R);
            double acc = 0.0;
            for (int nn = 0; nn <= p; ++nn)
                for (int mm = 0; mm <= nn; ++mm) {
                    cplx v = cmul(Lc[i * nc + TRI(nn, mm)], R[TRI(nn, mm)]);
                    acc += (mm == 0 ? 1.0 : 2.0) * v.re;
                }
            far[j] = acc;
        }
    }
    int64_t *ranges = malloc(sizeof(int64_t) * 2 * m);
    for (int64_t i = 0; i < m; ++i) {
        ranges[2 * i] = t->start[i];
        ranges[2 * i + 1] = t->end[i];
    }
    orc_p2p(pts, q, n, ranges, L->p2p, L->n_p2p, eps, near);
    for (int64_t i = 0; i < n; ++i) {
        int64_t o = t->index_map[i];
        double v = (far[i] + near[i]) * ke;
        if (self_int) v += self_int[o] * sigma[o] * areas[o];
        if (!isfinite(v)) v = 0.0;
        out[o] = v;
    }
    if (phi_far_tree) memcpy(phi_far_tree, far, sizeof(double) * n);
    if (phi_near_tree) memcpy(phi_near_tree, near, sizeof(double) * n);
    free(ranges);
    free(far);
    free(near);
    free(Mc);
    free(Lc);
    free(pts);
    free(q);
    return 0;
}

ORC_API int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* Panel quadrature (core/bem_quadrature.py:79-308, core/bem.py:475-734) */
/* ------------------------------------------------------------------ */

typedef struct {
    double x, y, z;
} v3d;

static inline v3d v3_mid(v3d a, v3d b) { return (v3d){0.5 * (a.x + b.x), 0.5 * (a.y + b.y), 0.5 * (a.z + b.z)}; }
static inline double v3_dist(v3d a, v3d b) {
    double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrt((dx * dx + dy * dy) + dz * dz);
}
static inline v3d v3_cent(v3d a, v3d b, v3d c) {
    return (v3d){(a.x + b.x + c.x) / 3.0, (a.y + b.y + c.y) / 3.0, (a.z + b.z + c.z) / 3.0};
}
static double tri_area_d(v3d a, v3d b, v3d c) {
    double e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z, e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
    double cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
    return 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
}
/* standard_triangle_quadrature (order 1 or 2) applied to 1/r */
static double rule_sum_d(v3d a, v3d b, v3d c, v3d t, int order, double ke) {
    double area = tri_area_d(a, b, c);
    if (!(area > 0.0)) return 0.0;
    if (order <= 1) return ke / fmax(v3_dist(t, v3_cent(a, b, c)), 1e-12) * area;
    double p = 2.0 / 3.0, q = 1.0 / 6.0, s = 0.0;
    for (int k = 0; k < 3; ++k) {
        double l0 = k == 0 ? p : q, l1 = k == 1 ? p : q, l2 = k == 2 ? p : q;
        v3d y = {l0 * a.x + l1 * b.x + l2 * c.x, l0 * a.y + l1 * b.y + l2 * c.y, l0 * a.z + l1 * b.z + l2 * c.z};
        s += ke / fmax(v3_dist(t, y), 1e-12) * (area / 3.0);
    }
    return s;
}

/* near_singular_quadrature at target t, summed against K_E / r */
static double adaptive_sum_d(v3d v0, v3d v1, v3d v2, v3d t, int order, int depth, double ke) {
    v3d tri[64][3];
    int n = 1;
    tri[0][0] = v0;
    tri[0][1] = v1;
    tri[0][2] = v2;
    for (int d = 0; d < depth && n + 3 <= 64; ++d) {
        int best = 0;
        double bd = INFINITY;
        for (int i = 0; i < n; ++i) {
            double dd = v3_dist(v3_cent(tri[i][0], tri[i][1], tri[i][2]), t);
            if (dd < bd) {
                bd = dd;
                best = i;
            }
        }
        v3d a = tri[best][0], b = tri[best][1], c = tri[best][2];
        memmove(tri[best], tri[best + 1], sizeof(v3d) * 3 * (n - best - 1));
        n--;
        v3d m01 = v3_mid(a, b), m12 = v3_mid(b, c), m20 = v3_mid(c, a);
        v3d k[4][3] = {{a, m01, m20}, {m01, b, m12}, {m20, m12, c}, {m01, m12, m20}};
        for (int i = 0; i < 4; ++i) {
            memcpy(tri[n], k[i], sizeof(v3d) * 3);
            n++;
        }
    }
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += rule_sum_d(tri[i][0], tri[i][1], tri[i][2], t, order, ke);
    return s;
}

ORC_API void orc_self_integrals(const double *verts, const double *cent, int64_t n, int order, int depth, double ke,
                                double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double *v = verts + 9 * i;
        out[i] = adaptive_sum_d((v3d){v[0], v[1], v[2]}, (v3d){v[3], v[4], v[5]}, (v3d){v[6], v[7], v[8]},
                                (v3d){cent[3 * i], cent[3 * i + 1], cent[3 * i + 2]}, order, depth, ke);
    }
}

/* _build_near_pairs_for_panels: row-major (i ascending, j ascending) */
static const double *g_sort_x;
static int cmp_by_x(const void *a, const void *b) {
    int64_t i = *(const int64_t *)a, j = *(const int64_t *)b;
    double xi = g_sort_x[3 * i], xj = g_sort_x[3 * j];
    if (xi < xj) return -1;
    if (xi > xj) return 1;
    return (i > j) - (i < j);
}

/* The pair test of _build_near_pairs_for_panels (0 < |C_i - C_j| <= f (R_i + R_j),
 * R = sqrt(max(A, 0) / pi)), evaluated for every candidate inside an x-window
 * of half-width 2 f (R_i + R_max) over the points sorted by x; points outside
 * the window fail the test (|C_i - C_j| >= |dx|), so the set and its (i, j)
 * order are those of the all-pairs loop. */
ORC_API int64_t orc_near_pairs(const double *cent, const double *areas, int64_t n, double factor, int64_t *pairs,
                               int64_t cap) {
    if (n <= 0) return 0;
    double *r = (double *)malloc(sizeof(double) * n);
    int64_t *ord = (int64_t *)malloc(sizeof(int64_t) * n);
    int64_t *cnt = (int64_t *)calloc(n + 1, sizeof(int64_t));
    int64_t m = 0;
    double rmax = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        r[i] = sqrt((areas[i] > 0 ? areas[i] : 0.0) / M_PI);
        if (isfinite(r[i]) && r[i] > rmax) rmax = r[i];
        if (isfinite(cent[3 * i]) && isfinite(cent[3 * i + 1]) && isfinite(cent[3 * i + 2])) ord[m++] = i;
    }
    g_sort_x = cent;
    qsort(ord, m, sizeof(int64_t), cmp_by_x);
    double *xs = (double *)malloc(sizeof(double) * (m > 0 ? m : 1));
    for (int64_t k = 0; k < m; ++k) xs[k] = cent[3 * ord[k]];
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            if (!pairs) break;
            int64_t acc = 0;
            for (int64_t i = 0; i < n; ++i) {
                int64_t c = cnt[i];
                cnt[i] = acc;
                acc += c;
            }
            cnt[n] = acc;
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            v3d ci = {cent[3 * i], cent[3 * i + 1], cent[3 * i + 2]};
            if (!(isfinite(ci.x) && isfinite(ci.y) && isfinite(ci.z))) continue;
            double w = 2.0 * factor * (r[i] + rmax);
            if (!isfinite(w)) w = INFINITY;
            int64_t lo = 0, hi = m;
            while (lo < hi) {
                int64_t mid = lo + (hi - lo) / 2;
                if (xs[mid] < ci.x - w) lo = mid + 1;
                else hi = mid;
            }
            int64_t row = pass == 1 ? cnt[i] : 0, k0 = row, c = 0;
            for (int64_t k = lo; k < m && xs[k] <= ci.x + w; ++k) {
                int64_t j = ord[k];
                double d = v3_dist(ci, (v3d){cent[3 * j], cent[3 * j + 1], cent[3 * j + 2]});
                double th = factor * (r[i] + r[j]);
                if (isfinite(d) && isfinite(th) && d > 0.0 && d <= th) {
                    if (pass == 1 && row < cap) {
                        pairs[2 * row] = i;
                        pairs[2 * row + 1] = j;
                    }
                    row++;
                    c++;
                }
            }
            if (pass == 0) {
                cnt[i] = c;
            } else {
                /* order the row by j (insertion sort: rows are short) */
                int64_t e = row < cap ? row : cap;
                for (int64_t a = k0 + 1; a < e; ++a) {
                    int64_t v = pairs[2 * a + 1], b = a - 1;
                    while (b >= k0 && pairs[2 * b + 1] > v) {
                        pairs[2 * (b + 1) + 1] = pairs[2 * b + 1];
                        --b;
                    }
                    pairs[2 * (b + 1) + 1] = v;
                }
            }
        }
    }
    int64_t total = 0;
    if (pairs) total = cnt[n];
    else
        for (int64_t i = 0; i < n; ++i) total += cnt[i];
    free(r);
    free(ord);
    free(cnt);
    free(xs);
    return total;
}

/* _precompute_near_correction_weights with uniform refinement `depth` */
ORC_API void orc_near_weights(const double *cent, const double *areas, const double *verts, const int64_t *pairs,
                              int64_t np, int order, int depth, double ke, double *w) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < np; ++p) {
        int64_t i = pairs[2 * p], j = pairs[2 * p + 1];
        double aj = areas[j];
        if (!(aj > 0.0)) {
            w[p] = 0.0;
            continue;
        }
        v3d ci = {cent[3 * i], cent[3 * i + 1], cent[3 * i + 2]};
        const double *v = verts + 9 * j;
        int leaves = 1 << (2 * depth);
        double s = 0.0;
        for (int leaf = 0; leaf < leaves; ++leaf) {
            v3d a = {v[0], v[1], v[2]}, b = {v[3], v[4], v[5]}, c = {v[6], v[7], v[8]};
            for (int d = depth - 1; d >= 0; --d) {
                int digit = (leaf >> (2 * d)) & 3;
                v3d m01 = v3_mid(a, b), m12 = v3_mid(b, c), m20 = v3_mid(c, a);
                if (digit == 0) {
                    b = m01;
                    c = m20;
                } else if (digit == 1) {
                    a = m01;
                    c = m12;
                } else if (digit == 2) {
                    a = m20;
                    b = m12;
                } else {
                    a = m01;
                    b = m12;
                    c = m20;
                }
            }
            s += rule_sum_d(a, b, c, ci, order, ke);
        }
        double far = ke * aj / fmax(v3_dist(ci, (v3d){cent[3 * j], cent[3 * j + 1], cent[3 * j + 2]}), 1e-12);
        w[p] = s - far;
    }
}
