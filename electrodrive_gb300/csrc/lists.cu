// GPU dual-tree traversal producing the P2P and M2L interaction lists.
//
// The reference walks (src, tgt) node pairs from (root, root) with a LIFO
// stack (electrodrive/fmm3d/interaction_lists.py:419-472).  Every reachable
// pair has a unique parent pair, so the traversal is a tree of pairs and the
// output is a set; here it is expanded breadth first, one frontier of pairs
// per step, with stable scan-based compaction.  The decisions reproduce the
// reference bit for bit:
//   * MAC (interaction_lists.py:273-297): dist = |c_s - c_t| rounded in the
//     tree dtype as sqrt(fma(dz, dz, fma(dy, dy, dx * dx))), d = 2 * radius in
//     the tree dtype, accept iff dist != 0 and max(d_s, d_t) / dist < theta
//     evaluated in double; never for the same node;
//   * leaf-leaf -> P2P (self pairs included);
//   * refinement side (interaction_lists.py:306-337): the non-leaf side,
//     else the side whose diameter exceeds the other's by 1.01x, else the side
//     with more (or equal: src) points.
// The output is stored as CSR rows by target with sources ascending, i.e.
// the reference's (tgt, src) sort order (interaction_lists.py:474-485).
#include <algorithm>
#include <cmath>
#include <vector>

#include "edfmm_internal.cuh"

namespace edfmm {

namespace {

__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rn_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rn_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float rn_sqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double rn_sqrt(double a) { return __dsqrt_rn(a); }

enum : uint8_t { kM2L = 0, kP2P = 1, kRefineSrc = 2, kRefineTgt = 3 };

// s indexes the source tree (sc, sleaf, srange), t the target tree; `same`
// marks the single-tree case, where a node is never paired with itself by M2L.
template <typename T>
__device__ __forceinline__ uint8_t classify(int s, int t, const typename Vec4<T>::type *__restrict__ sc,
                                            const uint8_t *__restrict__ sleaf, const int2 *__restrict__ srange,
                                            const typename Vec4<T>::type *__restrict__ tc,
                                            const uint8_t *__restrict__ tleaf, const int2 *__restrict__ trange,
                                            int same, double theta) {
    typename Vec4<T>::type cs = sc[s], ct = tc[t];
    double ds = (double)rn_mul((T)2, cs.w), dt = (double)rn_mul((T)2, ct.w);
    if (!(same && s == t)) {
        T dx = rn_sub(cs.x, ct.x), dy = rn_sub(cs.y, ct.y), dz = rn_sub(cs.z, ct.z);
        double dist = (double)rn_sqrt(rn_fma(dz, dz, rn_fma(dy, dy, rn_mul(dx, dx))));
        if (dist != 0.0) {
            double mx = ds >= dt ? ds : dt;
            if (__ddiv_rn(mx, dist) < theta) return kM2L;
        }
    }
    bool sl = sleaf[s], tl = tleaf[t];
    if (sl && tl) return kP2P;
    if (sl) return kRefineTgt;
    if (tl) return kRefineSrc;
    if (ds > __dmul_rn(dt, 1.01)) return kRefineSrc;
    if (dt > __dmul_rn(ds, 1.01)) return kRefineTgt;
    int ns = srange[s].y - srange[s].x, nt = trange[t].y - trange[t].x;
    return ns >= nt ? kRefineSrc : kRefineTgt;
}

// the arrays of one tree that the traversal reads
template <typename T> struct TravTree {
    const typename Vec4<T>::type *center;
    const uint8_t *is_leaf;
    const int2 *range;
    const int32_t *children;
};

__device__ __forceinline__ int n_children(const int32_t *children, int node) {
    int c = 0;
#pragma unroll
    for (int o = 0; o < 8; ++o) c += children[8 * node + o] >= 0 ? 1 : 0;
    return c;
}

template <typename T>
__global__ void k_classify(const int2 *__restrict__ front, int64_t nf, TravTree<T> S, TravTree<T> Tt, int same,
                           double theta, uint8_t *code, int32_t *c_m2l, int32_t *c_p2p, int32_t *c_next) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    int2 pr = front[i];
    uint8_t c = classify<T>(pr.x, pr.y, S.center, S.is_leaf, S.range, Tt.center, Tt.is_leaf, Tt.range, same, theta);
    code[i] = c;
    c_m2l[i] = c == kM2L;
    c_p2p[i] = c == kP2P;
    c_next[i] = c == kRefineSrc ? n_children(S.children, pr.x) : (c == kRefineTgt ? n_children(Tt.children, pr.y) : 0);
}

__global__ void k_emit(const int2 *__restrict__ front, int64_t nf, const uint8_t *code, const int32_t *s_children,
                       const int32_t *t_children, const int32_t *o_m2l, const int32_t *o_p2p, const int32_t *o_next,
                       int2 *m2l, int64_t m2l_base, int2 *p2p, int64_t p2p_base, int2 *next) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    int2 pr = front[i];
    uint8_t c = code[i];
    if (c == kM2L) {
        m2l[m2l_base + o_m2l[i]] = pr;
    } else if (c == kP2P) {
        p2p[p2p_base + o_p2p[i]] = pr;
    } else {
        const int32_t *children = c == kRefineSrc ? s_children : t_children;
        int node = c == kRefineSrc ? pr.x : pr.y;
        int j = o_next[i];
        for (int o = 0; o < 8; ++o) {
            int ch = children[8 * node + o];
            if (ch < 0) continue;
            next[j++] = c == kRefineSrc ? make_int2(ch, pr.y) : make_int2(pr.x, ch);
        }
    }
}

// CSR helpers: rows keyed by .y (target) or .x (swapped)
__global__ void k_row_counts(const int2 *pairs, int64_t np, int key_x, int32_t *cnt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    int r = key_x ? pairs[i].x : pairs[i].y;
    atomicAdd(&cnt[r], 1);
}
__global__ void k_row_fill(const int2 *pairs, int64_t np, int key_x, int32_t *cursor, int32_t *vals) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    int2 p = pairs[i];
    int r = key_x ? p.x : p.y;
    int v = key_x ? p.y : p.x;
    vals[atomicAdd(&cursor[r], 1)] = v;
}
__global__ void k_set_last(int32_t *off, int64_t rows, const int64_t *total) { off[rows] = (int32_t)*total; }
__global__ void k_max_count(const int32_t *cnt, int64_t rows, int *mx) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int v = i < rows ? cnt[i] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, v);
}
// sum over P2P pairs of n_s * n_t
__global__ void k_interactions(const int2 *pairs, int64_t np, const int2 *srange, const int2 *trange,
                               unsigned long long *acc) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long v = 0;
    if (i < np) {
        int2 p = pairs[i];
        v = (unsigned long long)(srange[p.x].y - srange[p.x].x) * (unsigned long long)(trange[p.y].y - trange[p.y].x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, v);
}
// transposed CSR from a CSR: pairs (row -> val) become (val -> row)
__global__ void k_csr_to_pairs(const int32_t *off, const int32_t *vals, int64_t rows, int2 *pairs) {
    int64_t r = (int64_t)blockIdx.x * blockDim.y + threadIdx.y;
    if (r >= rows) return;
    for (int k = off[r] + threadIdx.x; k < off[r + 1]; k += blockDim.x) pairs[k] = make_int2(vals[k], (int)r);
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// growable pair buffer
struct PairBuf {
    DevBuf buf;
    int64_t n = 0, cap = 0;
    int ensure(int64_t want, cudaStream_t s) {
        if (want <= cap) return EDFMM_OK;
        int64_t nc = std::max<int64_t>(want, std::max<int64_t>(cap * 2, 1 << 16));
        DevBuf nb;
        int rc = nb.reserve(sizeof(int2) * nc);
        if (rc) return rc;
        if (n > 0) EDFMM_CUDA_TRY(cudaMemcpyAsync(nb.p, buf.p, sizeof(int2) * n, cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
        buf = std::move(nb);
        cap = nc;
        return EDFMM_OK;
    }
};

// Build CSR (rows 0..rows-1) from a pair array keyed on .y (or .x).
int build_csr(const int2 *pairs, int64_t np, int64_t rows, int key_x, DevBuf &off, DevBuf &vals, int64_t &max_row,
              cudaStream_t s) {
    int rc;
    DevBuf cnt, tmp, total, mx;
    if ((rc = off.reserve(sizeof(int32_t) * (rows + 1))) || (rc = vals.reserve(sizeof(int32_t) * std::max<int64_t>(np, 1))) ||
        (rc = cnt.reserve(sizeof(int32_t) * rows)) || (rc = tmp.reserve(scan_tmp_bytes(rows))) ||
        (rc = total.reserve(sizeof(int64_t))) || (rc = mx.reserve(sizeof(int))))
        return rc;
    EDFMM_CUDA_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * rows, s));
    EDFMM_CUDA_TRY(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
    if (np > 0) {
        k_row_counts<<<nblk(np, 256), 256, 0, s>>>(pairs, np, key_x, dptr<int32_t>(cnt));
        EDFMM_LAUNCH_CHECK("k_row_counts");
    }
    if ((rc = scan_exclusive(dptr<int32_t>(cnt), dptr<int32_t>(off), rows, dptr<int64_t>(total), tmp.p, s))) return rc;
    k_set_last<<<1, 1, 0, s>>>(dptr<int32_t>(off), rows, dptr<int64_t>(total));
    EDFMM_LAUNCH_CHECK("k_set_last");
    k_max_count<<<nblk(rows, 256), 256, 0, s>>>(dptr<int32_t>(cnt), rows, dptr<int>(mx));
    EDFMM_LAUNCH_CHECK("k_max_count");
    if (np > 0) {
        EDFMM_CUDA_TRY(cudaMemcpyAsync(cnt.p, off.p, sizeof(int32_t) * rows, cudaMemcpyDeviceToDevice, s));
        k_row_fill<<<nblk(np, 256), 256, 0, s>>>(pairs, np, key_x, dptr<int32_t>(cnt), dptr<int32_t>(vals));
        EDFMM_LAUNCH_CHECK("k_row_fill");
    }
    int hmx = 0;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&hmx, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    max_row = hmx;
    return sort_csr_rows(dptr<int32_t>(off), dptr<int32_t>(vals), rows, max_row, s);
}

// the first front of a forest's traversal: (root, root) for every root
// (level 0 of the tree; a single tree has one root, DFS id 0)
__global__ void k_root_pairs(const int32_t *level_nodes, int K, int2 *front) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < K) front[k] = make_int2(level_nodes[k], level_nodes[k]);
}

// near-field work of each target leaf: (sum of its P2P sources' points) x its
// points, plus one for the epilogue of a leaf without sources
__global__ void k_leaf_work(const int32_t *__restrict__ leaves, int64_t nl, const int32_t *__restrict__ off,
                            const int32_t *__restrict__ src, const int2 *__restrict__ trange,
                            const int2 *__restrict__ srange, int64_t *__restrict__ work) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nl) return;
    const int t = leaves[i];
    int64_t w = 0;
    for (int k = off[t]; k < off[t + 1]; ++k) {
        const int2 r = srange[src[k]];
        w += r.y - r.x;
    }
    work[i] = w * (int64_t)(trange[t].y - trange[t].x) + 1;
}

// L.p2p_leaves: the target tree's leaves by decreasing work, in 64 buckets of
// log2(work) in quarter steps (a counting sort; leaves keep their tree order
// within a bucket, so the order is deterministic)
int order_p2p_leaves(const DevTree &tree, const DevTree &stree, DevLists &L, cudaStream_t s) {
    const int64_t nl = tree.n_leaves;
    if (nl <= 0) return EDFMM_OK;
    int rc;
    DevBuf work;
    if ((rc = work.reserve(sizeof(int64_t) * nl)) || (rc = L.p2p_leaves.reserve(sizeof(int32_t) * nl))) return rc;
    k_leaf_work<<<nblk(nl, 256), 256, 0, s>>>(dptr<int32_t>(tree.leaves), nl, dptr<int32_t>(L.p2p_off),
                                              dptr<int32_t>(L.p2p_src), dptr<int2>(tree.range), dptr<int2>(stree.range),
                                              dptr<int64_t>(work));
    EDFMM_LAUNCH_CHECK("k_leaf_work");
    std::vector<int64_t> w(nl);
    std::vector<int32_t> leaves(nl), order(nl);
    EDFMM_CUDA_TRY(cudaMemcpyAsync(w.data(), work.p, sizeof(int64_t) * nl, cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaMemcpyAsync(leaves.data(), tree.leaves.p, sizeof(int32_t) * nl, cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    constexpr int kBuckets = 256;
    auto bucket = [](int64_t v) {
        const int b = (int)std::floor(4.0 * std::log2((double)v));
        return kBuckets - 1 - std::min(std::max(b, 0), kBuckets - 1);  // decreasing work
    };
    std::vector<int64_t> start(kBuckets + 1, 0);
    for (int64_t i = 0; i < nl; ++i) ++start[bucket(w[i]) + 1];
    for (int b = 0; b < kBuckets; ++b) start[b + 1] += start[b];
    for (int64_t i = 0; i < nl; ++i) order[start[bucket(w[i])]++] = leaves[i];
    EDFMM_CUDA_TRY(cudaMemcpyAsync(L.p2p_leaves.p, order.data(), sizeof(int32_t) * nl, cudaMemcpyHostToDevice, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    return EDFMM_OK;
}

// L.m2l_rows: the target tree's nodes by decreasing M2L pair count (a
// counting sort on the count; nodes keep their DFS order within a count)
int order_m2l_rows(const DevTree &tree, DevLists &L, cudaStream_t s) {
    const int64_t M = tree.n_nodes;
    if (M <= 0) return EDFMM_OK;
    int rc;
    if ((rc = L.m2l_rows.reserve(sizeof(int32_t) * M))) return rc;
    std::vector<int32_t> off(M + 1), order(M);
    EDFMM_CUDA_TRY(cudaMemcpyAsync(off.data(), L.m2l_off.p, sizeof(int32_t) * (M + 1), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t top = 0;
    for (int64_t t = 0; t < M; ++t) top = std::max<int64_t>(top, off[t + 1] - off[t]);
    std::vector<int64_t> start(top + 2, 0);  // bucket b = top - count
    for (int64_t t = 0; t < M; ++t) ++start[top - (off[t + 1] - off[t]) + 1];
    for (int64_t b = 0; b <= top; ++b) start[b + 1] += start[b];
    for (int64_t t = 0; t < M; ++t) order[start[top - (off[t + 1] - off[t])]++] = (int32_t)t;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(L.m2l_rows.p, order.data(), sizeof(int32_t) * M, cudaMemcpyHostToDevice, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    return EDFMM_OK;
}

template <typename T>
int lists_impl(const DevTree &stree, const DevTree &tree, double theta, DevLists &L, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    int rc;
    const int64_t M = tree.n_nodes;  // rows: target-tree nodes
    const int same = &stree == &tree ? 1 : 0;
    const TravTree<T> S{dptr<T4>(stree.center), dptr<uint8_t>(stree.is_leaf), dptr<int2>(stree.range),
                        dptr<int32_t>(stree.children)};
    const TravTree<T> Tt{dptr<T4>(tree.center), dptr<uint8_t>(tree.is_leaf), dptr<int2>(tree.range),
                         dptr<int32_t>(tree.children)};
    L = DevLists();
    if (M == 0 || stree.n_nodes == 0) {
        if ((rc = L.p2p_off.reserve(sizeof(int32_t))) || (rc = L.m2l_off.reserve(sizeof(int32_t))) ||
            (rc = L.p2p_src.reserve(4)) || (rc = L.m2l_src.reserve(4)))
            return rc;
        EDFMM_CUDA_TRY(cudaMemsetAsync(L.p2p_off.p, 0, sizeof(int32_t), s));
        EDFMM_CUDA_TRY(cudaMemsetAsync(L.m2l_off.p, 0, sizeof(int32_t), s));
        return EDFMM_OK;
    }
    PairBuf m2l, p2p;
    DevBuf front, next, code, cm, cp, cn, om, op, on, tmp, tot;
    // a same-tree forest (batched plan) starts from every (root, root) pair;
    // no pair ever joins two trees, so each tree gets its own lists
    const int n_roots = same && tree.level_offsets.size() > 1 ? tree.level_offsets[1] - tree.level_offsets[0] : 1;
    if ((rc = tot.reserve(sizeof(int64_t) * 3)) || (rc = front.reserve(sizeof(int2) * n_roots))) return rc;
    if (n_roots > 1) {
        k_root_pairs<<<nblk(n_roots, 256), 256, 0, s>>>(dptr<int32_t>(tree.level_nodes), n_roots, dptr<int2>(front));
        EDFMM_LAUNCH_CHECK("k_root_pairs");
    } else {
        int2 root = make_int2(0, 0);
        EDFMM_CUDA_TRY(cudaMemcpyAsync(front.p, &root, sizeof(int2), cudaMemcpyHostToDevice, s));
    }
    int64_t nf = n_roots;
    while (nf > 0) {
        if ((rc = code.reserve(nf)) || (rc = cm.reserve(4 * nf)) || (rc = cp.reserve(4 * nf)) || (rc = cn.reserve(4 * nf)) ||
            (rc = om.reserve(4 * nf)) || (rc = op.reserve(4 * nf)) || (rc = on.reserve(4 * nf)) ||
            (rc = tmp.reserve(scan_tmp_bytes(nf))))
            return rc;
        k_classify<T><<<nblk(nf, 256), 256, 0, s>>>(dptr<int2>(front), nf, S, Tt, same, theta, dptr<uint8_t>(code),
                                                     dptr<int32_t>(cm), dptr<int32_t>(cp), dptr<int32_t>(cn));
        EDFMM_LAUNCH_CHECK("k_classify");
        int64_t *t3 = dptr<int64_t>(tot);
        if ((rc = scan_exclusive(dptr<int32_t>(cm), dptr<int32_t>(om), nf, t3, tmp.p, s)) ||
            (rc = scan_exclusive(dptr<int32_t>(cp), dptr<int32_t>(op), nf, t3 + 1, tmp.p, s)) ||
            (rc = scan_exclusive(dptr<int32_t>(cn), dptr<int32_t>(on), nf, t3 + 2, tmp.p, s)))
            return rc;
        int64_t h[3];
        EDFMM_CUDA_TRY(cudaMemcpyAsync(h, t3, sizeof(h), cudaMemcpyDeviceToHost, s));
        EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
        if (h[0] + m2l.n >= INT32_MAX || h[1] + p2p.n >= INT32_MAX || h[2] >= INT32_MAX)
            return fail(EDFMM_ERR_ARG, "interaction lists exceed 2^31 pairs");
        if ((rc = m2l.ensure(m2l.n + h[0], s)) || (rc = p2p.ensure(p2p.n + h[1], s)) ||
            (rc = next.reserve(sizeof(int2) * std::max<int64_t>(h[2], 1))))
            return rc;
        k_emit<<<nblk(nf, 256), 256, 0, s>>>(dptr<int2>(front), nf, dptr<uint8_t>(code), S.children, Tt.children,
                                              dptr<int32_t>(om), dptr<int32_t>(op), dptr<int32_t>(on), dptr<int2>(m2l.buf),
                                              m2l.n, dptr<int2>(p2p.buf), p2p.n, dptr<int2>(next));
        EDFMM_LAUNCH_CHECK("k_emit");
        m2l.n += h[0];
        p2p.n += h[1];
        nf = h[2];
        std::swap(front, next);
    }
    L.n_m2l = m2l.n;
    L.n_p2p = p2p.n;
    if ((rc = build_csr(dptr<int2>(p2p.buf), p2p.n, M, 0, L.p2p_off, L.p2p_src, L.max_p2p_row, s)) ||
        (rc = build_csr(dptr<int2>(m2l.buf), m2l.n, M, 0, L.m2l_off, L.m2l_src, L.max_m2l_row, s)))
        return rc;
    DevBuf acc;
    if ((rc = acc.reserve(sizeof(unsigned long long)))) return rc;
    EDFMM_CUDA_TRY(cudaMemsetAsync(acc.p, 0, sizeof(unsigned long long), s));
    if (p2p.n > 0) {
        k_interactions<<<nblk(p2p.n, 256), 256, 0, s>>>(dptr<int2>(p2p.buf), p2p.n, dptr<int2>(stree.range),
                                                         dptr<int2>(tree.range), dptr<unsigned long long>(acc));
        EDFMM_LAUNCH_CHECK("k_interactions");
    }
    unsigned long long hi = 0;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&hi, acc.p, sizeof(hi), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    L.p2p_interactions = (int64_t)hi;
    if ((rc = order_p2p_leaves(tree, stree, L, s))) return rc;
    return order_m2l_rows(tree, L, s);
}

}  // namespace

int lists_build(const DevTree &tree, double theta, DevLists &lists, cudaStream_t s) {
    if (tree.dtype == EDFMM_F64) return lists_impl<double>(tree, tree, theta, lists, s);
    return lists_impl<float>(tree, tree, theta, lists, s);
}

int lists_build_two(const DevTree &src_tree, const DevTree &tgt_tree, double theta, DevLists &lists, cudaStream_t s) {
    if (src_tree.dtype != tgt_tree.dtype) return fail(EDFMM_ERR_ARG, "source and target trees differ in dtype");
    if (src_tree.dtype == EDFMM_F64) return lists_impl<double>(src_tree, tgt_tree, theta, lists, s);
    return lists_impl<float>(src_tree, tgt_tree, theta, lists, s);
}

int lists_build_swapped(const DevTree &tree, DevLists &L, cudaStream_t s) {
    if (L.have_m2l_swapped) return EDFMM_OK;
    int rc;
    const int64_t M = tree.n_nodes;
    DevBuf pairs;
    if ((rc = pairs.reserve(sizeof(int2) * std::max<int64_t>(L.n_m2l, 1)))) return rc;
    if (M > 0) {
        dim3 blk(32, 8);
        k_csr_to_pairs<<<nblk(M, 8), blk, 0, s>>>(dptr<int32_t>(L.m2l_off), dptr<int32_t>(L.m2l_src), M, dptr<int2>(pairs));
        EDFMM_LAUNCH_CHECK("k_csr_to_pairs");
    }
    // pairs are (src, tgt); the swapped rows are keyed on src
    int64_t mx = 0;
    if ((rc = build_csr(dptr<int2>(pairs), L.n_m2l, std::max<int64_t>(M, 1), 1, L.m2l_swapped_off, L.m2l_swapped_src, mx, s)))
        return rc;
    L.have_m2l_swapped = true;
    return EDFMM_OK;
}

}  // namespace edfmm
