// GPU construction of the adaptive tight-bbox octree.
//
// The reference builds the tree with a depth-first Python recursion
// (electrodrive/fmm3d/tree.py:801-960).  Here the same tree is built one
// level at a time:
//   * every node of a level reduces the tight bounding box of its point range
//     (exact min/max via order-preserving integer atomics, so the result does
//     not depend on the reduction order);
//   * centre = 0.5 * (min + max), half = max(0.5 * (max - min), 0) and the
//     radius = sqrt(fma(hz, hz, fma(hy, hy, hx * hx))) * (1 + 1e-12) are
//     formed with the same roundings as the reference's torch ops;
//   * a node splits unless n <= leaf_size, level >= max_depth or
//     max(half) < 1e-7 (tree.py:895-897);
//   * points are partitioned stably by octant (x > cx) + 2 (y > cy) + 4 (z > cz)
//     with chunked counting (per-chunk octant counts, per-node prefix over its
//     chunks, ballot ranks inside a chunk), which reproduces the reference's
//     stable counting sort (tree.py:921-939);
//   * the final DFS pre-order numbering (tree.py:878-889) equals the rank of
//     each node by (range start, level): nodes sharing a start form a chain
//     of first children, so dfs = #nodes with smaller start + depth inside
//     the chain.
#include <algorithm>
#include <cfloat>

#include "edfmm_internal.cuh"

namespace edfmm {

namespace {

constexpr int kChunk = 1024;  // points per chunk, one thread per point

// order-preserving float <-> int maps for exact atomic min / max
__device__ __forceinline__ int ord_of(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float from_ord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }
__device__ __forceinline__ long long ord_of(double f) {
    long long i = __double_as_longlong(f);
    return i >= 0 ? i : i ^ 0x7fffffffffffffffLL;
}
__device__ __forceinline__ double from_ord(long long i) {
    return __longlong_as_double(i >= 0 ? i : i ^ 0x7fffffffffffffffLL);
}

template <typename T> struct OrdT {};
template <> struct OrdT<float> {
    using type = int;
    static constexpr int hi = 0x7fffffff;
    static constexpr int lo = (int)0x80000000;
};
template <> struct OrdT<double> {
    using type = long long;
    static constexpr long long hi = 0x7fffffffffffffffLL;
    static constexpr long long lo = (long long)0x8000000000000000ULL;
};

// exact-rounding helpers (no contraction across these)
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rn_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rn_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float rn_sqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double rn_sqrt(double a) { return __dsqrt_rn(a); }

// radius = ||h|| * (1 + 1e-12) rounded in T (tree.py:331)
__device__ __forceinline__ float radius_of(float hx, float hy, float hz) {
    float r = rn_sqrt(rn_fma(hz, hz, rn_fma(hy, hy, rn_mul(hx, hx))));
    return rn_mul(r, (float)(1.0 + 1e-12));
}
__device__ __forceinline__ double radius_of(double hx, double hy, double hz) {
    double r = rn_sqrt(rn_fma(hz, hz, rn_fma(hy, hy, rn_mul(hx, hx))));
    return rn_mul(r, 1.0 + 1e-12);
}

template <typename T> struct LevelNode {
    int32_t start, end;
};

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

template <typename T>
__global__ void k_init_points(const T *__restrict__ pts, int64_t n, typename Vec4<T>::type *xyz, int32_t *perm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    typename Vec4<T>::type v;
    v.x = pts[3 * i];
    v.y = pts[3 * i + 1];
    v.z = pts[3 * i + 2];
    v.w = 0;
    xyz[i] = v;
    perm[i] = (int32_t)i;
}

// chunk counts per node of the level
__global__ void k_chunk_counts(const int2 *rng, int K, int32_t *cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K) return;
    int n = rng[i].y - rng[i].x;
    cnt[i] = (n + kChunk - 1) / kChunk;
}

__global__ void k_chunk_fill(const int2 *rng, int K, const int32_t *chunk_off, int32_t *chunk_node) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K) return;
    int n = rng[i].y - rng[i].x;
    int c = (n + kChunk - 1) / kChunk;
    int b = chunk_off[i];
    for (int k = 0; k < c; ++k) chunk_node[b + k] = i;
}

template <typename T>
__global__ void k_bbox_init(typename OrdT<T>::type *bb, int K) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K) return;
    for (int a = 0; a < 3; ++a) {
        bb[6 * i + a] = OrdT<T>::hi;      // min
        bb[6 * i + 3 + a] = OrdT<T>::lo;  // max
    }
}

template <typename T>
__global__ void __launch_bounds__(kChunk) k_bbox(const typename Vec4<T>::type *__restrict__ xyz, const int2 *rng,
                                                 const int32_t *chunk_node, const int32_t *chunk_off,
                                                 typename OrdT<T>::type *bb) {
    using O = typename OrdT<T>::type;
    int q = blockIdx.x;
    int node = chunk_node[q];
    int k = q - chunk_off[node];
    int s = rng[node].x + k * kChunk;
    int e = min(rng[node].y, s + kChunk);
    int i = s + threadIdx.x;
    O mn[3] = {OrdT<T>::hi, OrdT<T>::hi, OrdT<T>::hi}, mx[3] = {OrdT<T>::lo, OrdT<T>::lo, OrdT<T>::lo};
    if (i < e) {
        typename Vec4<T>::type v = xyz[i];
        mn[0] = mx[0] = ord_of(v.x);
        mn[1] = mx[1] = ord_of(v.y);
        mn[2] = mx[2] = ord_of(v.z);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            O y = __shfl_xor_sync(0xffffffffu, mn[a], o);
            mn[a] = y < mn[a] ? y : mn[a];
            O z = __shfl_xor_sync(0xffffffffu, mx[a], o);
            mx[a] = z > mx[a] ? z : mx[a];
        }
    }
    __shared__ O smn[32][3], smx[32][3];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) {
            smn[w][a] = mn[a];
            smx[w][a] = mx[a];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        int a = threadIdx.x;
        O m0 = smn[0][a], m1 = smx[0][a];
        for (int ww = 1; ww < (int)(blockDim.x >> 5); ++ww) {
            m0 = smn[ww][a] < m0 ? smn[ww][a] : m0;
            m1 = smx[ww][a] > m1 ? smx[ww][a] : m1;
        }
        atomicMin(&bb[6 * node + a], m0);
        atomicMax(&bb[6 * node + 3 + a], m1);
    }
}

// centre / half / radius / leaf decision for every node of the level
template <typename T>
__global__ void k_finalize(const typename OrdT<T>::type *bb, const int2 *rng, int K, int level, int leaf_size,
                           int max_depth, typename Vec4<T>::type *center, typename Vec4<T>::type *half,
                           uint8_t *is_leaf, int *warn) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K) return;
    T c[3], h[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T mn = from_ord(bb[6 * i + a]);
        T mx = from_ord(bb[6 * i + 3 + a]);
        c[a] = rn_mul((T)0.5, rn_add(mn, mx));
        T hh = rn_mul((T)0.5, rn_sub(mx, mn));
        h[a] = hh < (T)0 ? (T)0 : hh;
    }
    T r = radius_of(h[0], h[1], h[2]);
    typename Vec4<T>::type cv, hv;
    cv.x = c[0];
    cv.y = c[1];
    cv.z = c[2];
    cv.w = r;
    hv.x = h[0];
    hv.y = h[1];
    hv.z = h[2];
    hv.w = 0;  // expansion scale, filled after the root radius is known
    center[i] = cv;
    half[i] = hv;
    int n = rng[i].y - rng[i].x;
    T hmax = h[0] > h[1] ? h[0] : h[1];
    hmax = hmax > h[2] ? hmax : h[2];
    bool degenerate = (double)hmax < 1e-7;
    bool leaf = n <= leaf_size || level >= max_depth || degenerate;
    is_leaf[i] = leaf ? 1 : 0;
    if (level >= max_depth && n > leaf_size && !degenerate) atomicAdd(warn, 1);
}

template <typename T>
__device__ __forceinline__ int octant_of(const typename Vec4<T>::type &p, const typename Vec4<T>::type &c) {
    return (p.x > c.x ? 1 : 0) + (p.y > c.y ? 2 : 0) + (p.z > c.z ? 4 : 0);
}

// per-chunk octant counts (chunks of split nodes only)
template <typename T>
__global__ void __launch_bounds__(kChunk) k_octant_counts(const typename Vec4<T>::type *__restrict__ xyz,
                                                          const int2 *rng, const int32_t *chunk_node,
                                                          const int32_t *chunk_off,
                                                          const typename Vec4<T>::type *center,
                                                          const uint8_t *is_leaf, int32_t *ccnt) {
    int q = blockIdx.x;
    int node = chunk_node[q];
    if (is_leaf[node]) return;
    __shared__ int cnt[8];
    if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
    __syncthreads();
    int k = q - chunk_off[node];
    int s = rng[node].x + k * kChunk;
    int e = min(rng[node].y, s + kChunk);
    int i = s + threadIdx.x;
    if (i < e) atomicAdd(&cnt[octant_of<T>(xyz[i], center[node])], 1);
    __syncthreads();
    if (threadIdx.x < 8) ccnt[8 * q + threadIdx.x] = cnt[threadIdx.x];
}

// per split node: exclusive prefix of octant counts over its chunks, totals
__global__ void k_node_octants(const int2 *rng, int K, const int32_t *chunk_off, const uint8_t *is_leaf,
                               int32_t *ccnt, int32_t *oct_start, int32_t *oct_cnt, int32_t *n_children) {
    // all 32 lanes stay to the end: the shuffles below use the full mask
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int i = t >> 3, o = t & 7;
    bool active = i < K && !is_leaf[i];
    int run = 0;
    if (active) {
        int n = rng[i].y - rng[i].x;
        int c = (n + kChunk - 1) / kChunk;
        int b = chunk_off[i];
        for (int k = 0; k < c; ++k) {
            int v = ccnt[8 * (b + k) + o];
            ccnt[8 * (b + k) + o] = run;
            run += v;
        }
    }
    // octant start = node start + counts of lower octants (the 8 lanes of one
    // node are consecutive lanes of one warp)
    int base = 0, nz = 0;
    for (int oo = 0; oo < 8; ++oo) {
        int v = __shfl_sync(0xffffffffu, run, (threadIdx.x & 31 & ~7) + oo);
        if (oo < o) base += v;
        nz += v > 0 ? 1 : 0;
    }
    if (i >= K) return;
    oct_cnt[8 * i + o] = run;
    oct_start[8 * i + o] = rng[i].x + base;
    if (o == 0) n_children[i] = nz;
}

// stable scatter of the chunk's points into their octant slots
template <typename T>
__global__ void __launch_bounds__(kChunk) k_scatter(const typename Vec4<T>::type *__restrict__ xyz,
                                                    const int32_t *__restrict__ perm, const int2 *rng,
                                                    const int32_t *chunk_node, const int32_t *chunk_off,
                                                    const typename Vec4<T>::type *center, const uint8_t *is_leaf,
                                                    const int32_t *ccnt, const int32_t *oct_start,
                                                    typename Vec4<T>::type *xyz_out, int32_t *perm_out) {
    int q = blockIdx.x;
    int node = chunk_node[q];
    if (is_leaf[node]) return;
    __shared__ int wcnt[32][8];
    int k = q - chunk_off[node];
    int s = rng[node].x + k * kChunk;
    int e = min(rng[node].y, s + kChunk);
    int i = s + threadIdx.x;
    bool valid = i < e;
    int o = -1;
    typename Vec4<T>::type v;
    if (valid) {
        v = xyz[i];
        o = octant_of<T>(v, center[node]);
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned lt = (1u << lane) - 1u;
    int my_rank = 0;
#pragma unroll
    for (int oo = 0; oo < 8; ++oo) {
        unsigned m = __ballot_sync(0xffffffffu, o == oo);
        if (o == oo) my_rank = __popc(m & lt);
        if (lane == 0) wcnt[w][oo] = __popc(m);
    }
    __syncthreads();
    // exclusive scan over warps for each octant
    if (threadIdx.x < 8) {
        int run = 0;
        int nw = blockDim.x >> 5;
        for (int ww = 0; ww < nw; ++ww) {
            int c = wcnt[ww][threadIdx.x];
            wcnt[ww][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
    if (valid) {
        int dest = oct_start[8 * node + o] + ccnt[8 * q + o] + wcnt[w][o] + my_rank;
        xyz_out[dest] = v;
        perm_out[dest] = perm[i];
    }
}

template <typename T>
__global__ void __launch_bounds__(kChunk) k_copy_back(const int2 *rng, const int32_t *chunk_node,
                                                      const int32_t *chunk_off, const uint8_t *is_leaf,
                                                      const typename Vec4<T>::type *xyz_tmp, const int32_t *perm_tmp,
                                                      typename Vec4<T>::type *xyz, int32_t *perm) {
    int q = blockIdx.x;
    int node = chunk_node[q];
    if (is_leaf[node]) return;
    int k = q - chunk_off[node];
    int s = rng[node].x + k * kChunk;
    int e = min(rng[node].y, s + kChunk);
    int i = s + threadIdx.x;
    if (i < e) {
        xyz[i] = xyz_tmp[i];
        perm[i] = perm_tmp[i];
    }
}

// children of split nodes -> next level
__global__ void k_make_children(int K, const uint8_t *is_leaf, const int32_t *oct_start, const int32_t *oct_cnt,
                                const int32_t *child_off, int level_base, int next_base, int2 *next_rng,
                                int32_t *next_parent, int32_t *children_bfs, const int32_t *root,
                                int32_t *next_root) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K) return;
    int j = child_off[i];
    for (int o = 0; o < 8; ++o) {
        int c = oct_cnt[8 * i + o];
        if (!is_leaf[i] && c > 0) {
            next_rng[j] = make_int2(oct_start[8 * i + o], oct_start[8 * i + o] + c);
            next_parent[j] = level_base + i;
            next_root[j] = root[i];
            children_bfs[8 * i + o] = next_base + j;
            ++j;
        } else {
            children_bfs[8 * i + o] = -1;
        }
    }
}

// DFS numbering
__global__ void k_dfs_marks(const int2 *rng, const int32_t *lev, int64_t M, int32_t *cnt_at, int32_t *minlev_at) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= M) return;
    int s = rng[b].x;
    atomicAdd(&cnt_at[s], 1);
    atomicMin(&minlev_at[s], lev[b]);
}

__global__ void k_dfs_ids(const int2 *rng, const int32_t *lev, int64_t M, const int32_t *base_at,
                          const int32_t *minlev_at, int32_t *dfs) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= M) return;
    int s = rng[b].x;
    dfs[b] = base_at[s] + lev[b] - minlev_at[s];
}

// Floor of the expansion scale of each tree of the forest: 2^-40 of its
// root's radius (1 for a root of radius 0); level 0 holds the roots.
template <typename T>
__global__ void k_root_floors(const typename Vec4<T>::type *root_cen, int K, T *floors) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const T r = root_cen[k].w;
    floors[k] = r > (T)0 ? (T)(r * (T)9.094947017729282e-13) : (T)1;
}

template <typename T>
__global__ void k_permute_nodes(int64_t M, const int32_t *dfs, const int2 *rng, const int32_t *lev,
                                const int32_t *par_bfs, const int32_t *ch_bfs,
                                const typename Vec4<T>::type *cen, const typename Vec4<T>::type *hal,
                                const uint8_t *leaf, const int32_t *root, const T *floors, int2 *o_rng,
                                int32_t *o_lev, int32_t *o_par,
                                int32_t *o_ch, typename Vec4<T>::type *o_cen, typename Vec4<T>::type *o_hal,
                                uint8_t *o_leaf, int32_t *level_nodes) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= M) return;
    int d = dfs[b];
    o_rng[d] = rng[b];
    o_lev[d] = lev[b];
    o_par[d] = par_bfs[b] >= 0 ? dfs[par_bfs[b]] : -1;
    for (int o = 0; o < 8; ++o) {
        int c = ch_bfs[8 * b + o];
        o_ch[8 * d + o] = c >= 0 ? dfs[c] : -1;
    }
    o_cen[d] = cen[b];
    typename Vec4<T>::type h = hal[b];
    const T r = cen[b].w, scale_floor = floors[root[b]];
    h.w = r > scale_floor ? r : scale_floor;
    o_hal[d] = h;
    o_leaf[d] = leaf[b];
    level_nodes[b] = d;
}

// Expansion scale of one level's nodes: at least 1/8 of the parent's scale.
// A node whose points coincide (radius 0, e.g. a single-point leaf) would
// otherwise get the global floor, and every M2L pair into it would have a
// source/target scale ratio far above the fast kernel's range.  Any positive
// scale is exact algebra; this one keeps the ratios O(10).
template <typename T>
__global__ void k_scale_from_parent(const int32_t *__restrict__ nodes, int count, const int32_t *__restrict__ parent,
                                    typename Vec4<T>::type *half) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int d = nodes[i];
    const int p = parent[d];
    if (p < 0) return;
    const T lo = half[p].w * (T)0.125;
    if (half[d].w < lo) half[d].w = lo;
}

__global__ void k_leaf_flags(const uint8_t *leaf, int64_t M, int32_t *flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < M) flag[i] = leaf[i];
}
__global__ void k_leaf_compact(const uint8_t *leaf, int64_t M, const int32_t *off, int32_t *leaves) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < M && leaf[i]) leaves[off[i]] = (int32_t)i;
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// One level's working set.
template <typename T> struct Level {
    int K = 0;
    int base = 0;  // BFS id of the level's first node
    DevBuf rng, parent, center, half, leaf, children, root;
};

__global__ void k_inst_node_off(const int32_t *level_nodes, int K, int32_t M, int32_t *off) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < K) off[k] = level_nodes[k];  // DFS id of root k
    if (k == K) off[K] = M;
}

// A forest when inst_off (host, n_inst + 1 point offsets) is given: level 0
// holds one root per instance over its rows, every later level the children
// of all instances' split nodes, so each level is one set of launches for
// the whole batch.  Each tree is the one a single build of its rows gives.
template <typename T>
int build_impl(const void *points_dev, int64_t n, int leaf_size, int max_depth, DevTree &tree, cudaStream_t s,
               const int64_t *inst_off, int n_inst) {
    using T4 = typename Vec4<T>::type;
    using O = typename OrdT<T>::type;
    int rc;
    tree.n_points = n;
    tree.dtype = sizeof(T) == 8 ? EDFMM_F64 : EDFMM_F32;
    tree.depth_warnings = 0;
    if (n == 0) {
        tree.n_nodes = tree.n_leaves = 0;
        tree.max_level = 0;
        tree.level_offsets.assign(1, 0);
        if ((rc = tree.pts.reserve(16)) || (rc = tree.index_map.reserve(16))) return rc;
        return EDFMM_OK;
    }
    if (n >= (int64_t)INT32_MAX) return fail(EDFMM_ERR_ARG, "n_points must be < 2^31");

    DevBuf xyz, xyz_tmp, perm, perm_tmp, warn, scan_tmp, total;
    if ((rc = xyz.reserve(sizeof(T4) * n)) || (rc = xyz_tmp.reserve(sizeof(T4) * n)) ||
        (rc = perm.reserve(sizeof(int32_t) * n)) || (rc = perm_tmp.reserve(sizeof(int32_t) * n)) ||
        (rc = warn.reserve(sizeof(int))) || (rc = total.reserve(sizeof(int64_t))))
        return rc;
    EDFMM_CUDA_TRY(cudaMemsetAsync(warn.p, 0, sizeof(int), s));
    k_init_points<T><<<nblk(n, 256), 256, 0, s>>>(static_cast<const T *>(points_dev), n, dptr<T4>(xyz), dptr<int32_t>(perm));
    EDFMM_LAUNCH_CHECK("k_init_points");

    std::vector<Level<T>> levels;
    levels.emplace_back();
    const int K0 = inst_off ? n_inst : 1;
    std::vector<int2> h_r0(K0);
    std::vector<int32_t> h_p0(K0, -1), h_root0(K0);
    {
        Level<T> &L0 = levels.back();
        L0.K = K0;
        L0.base = 0;
        if ((rc = L0.rng.reserve(sizeof(int2) * K0)) || (rc = L0.parent.reserve(sizeof(int32_t) * K0)) ||
            (rc = L0.root.reserve(sizeof(int32_t) * K0)))
            return rc;
        for (int k = 0; k < K0; ++k) {
            h_r0[k] = inst_off ? make_int2((int)inst_off[k], (int)inst_off[k + 1]) : make_int2(0, (int)n);
            h_root0[k] = k;
        }
        EDFMM_CUDA_TRY(cudaMemcpyAsync(L0.rng.p, h_r0.data(), sizeof(int2) * K0, cudaMemcpyHostToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(L0.parent.p, h_p0.data(), sizeof(int32_t) * K0, cudaMemcpyHostToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(L0.root.p, h_root0.data(), sizeof(int32_t) * K0, cudaMemcpyHostToDevice, s));
    }
    DevBuf cnt, off, chunk_node, bb, ccnt, oct_start, oct_cnt, nchild, child_off;
    int64_t total_nodes = K0;  // the roots
    for (int lev = 0;; ++lev) {
        Level<T> &L = levels[lev];
        const int K = L.K;
        if ((rc = L.center.reserve(sizeof(T4) * K)) || (rc = L.half.reserve(sizeof(T4) * K)) ||
            (rc = L.leaf.reserve(K)) || (rc = L.children.reserve(sizeof(int32_t) * 8 * K)) ||
            (rc = cnt.reserve(sizeof(int32_t) * K)) || (rc = off.reserve(sizeof(int32_t) * K)) ||
            (rc = bb.reserve(sizeof(O) * 6 * K)) || (rc = oct_start.reserve(sizeof(int32_t) * 8 * K)) ||
            (rc = oct_cnt.reserve(sizeof(int32_t) * 8 * K)) || (rc = nchild.reserve(sizeof(int32_t) * K)) ||
            (rc = child_off.reserve(sizeof(int32_t) * K)) || (rc = scan_tmp.reserve(scan_tmp_bytes(K))))
            return rc;
        const int2 *rng = dptr<int2>(L.rng);
        // chunks
        k_chunk_counts<<<nblk(K, 256), 256, 0, s>>>(rng, K, dptr<int32_t>(cnt));
        EDFMM_LAUNCH_CHECK("k_chunk_counts");
        if ((rc = scan_exclusive(dptr<int32_t>(cnt), dptr<int32_t>(off), K, dptr<int64_t>(total), scan_tmp.p, s))) return rc;
        int64_t Q = 0;
        EDFMM_CUDA_TRY(cudaMemcpyAsync(&Q, total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
        if ((rc = chunk_node.reserve(sizeof(int32_t) * Q)) || (rc = ccnt.reserve(sizeof(int32_t) * 8 * Q))) return rc;
        k_chunk_fill<<<nblk(K, 256), 256, 0, s>>>(rng, K, dptr<int32_t>(off), dptr<int32_t>(chunk_node));
        EDFMM_LAUNCH_CHECK("k_chunk_fill");
        // bounding boxes and node geometry
        k_bbox_init<T><<<nblk(K, 256), 256, 0, s>>>(dptr<O>(bb), K);
        EDFMM_LAUNCH_CHECK("k_bbox_init");
        k_bbox<T><<<(unsigned)Q, kChunk, 0, s>>>(dptr<T4>(xyz), rng, dptr<int32_t>(chunk_node), dptr<int32_t>(off), dptr<O>(bb));
        EDFMM_LAUNCH_CHECK("k_bbox");
        k_finalize<T><<<nblk(K, 256), 256, 0, s>>>(dptr<O>(bb), rng, K, lev, leaf_size, max_depth, dptr<T4>(L.center),
                                                     dptr<T4>(L.half), dptr<uint8_t>(L.leaf), dptr<int>(warn));
        EDFMM_LAUNCH_CHECK("k_finalize");
        // partition the points of split nodes
        k_octant_counts<T><<<(unsigned)Q, kChunk, 0, s>>>(dptr<T4>(xyz), rng, dptr<int32_t>(chunk_node), dptr<int32_t>(off),
                                                          dptr<T4>(L.center), dptr<uint8_t>(L.leaf), dptr<int32_t>(ccnt));
        EDFMM_LAUNCH_CHECK("k_octant_counts");
        k_node_octants<<<nblk((int64_t)K * 8, 256), 256, 0, s>>>(rng, K, dptr<int32_t>(off), dptr<uint8_t>(L.leaf),
                                                                 dptr<int32_t>(ccnt), dptr<int32_t>(oct_start),
                                                                 dptr<int32_t>(oct_cnt), dptr<int32_t>(nchild));
        EDFMM_LAUNCH_CHECK("k_node_octants");
        k_scatter<T><<<(unsigned)Q, kChunk, 0, s>>>(dptr<T4>(xyz), dptr<int32_t>(perm), rng, dptr<int32_t>(chunk_node),
                                                    dptr<int32_t>(off), dptr<T4>(L.center), dptr<uint8_t>(L.leaf),
                                                    dptr<int32_t>(ccnt), dptr<int32_t>(oct_start), dptr<T4>(xyz_tmp),
                                                    dptr<int32_t>(perm_tmp));
        EDFMM_LAUNCH_CHECK("k_scatter");
        k_copy_back<T><<<(unsigned)Q, kChunk, 0, s>>>(rng, dptr<int32_t>(chunk_node), dptr<int32_t>(off),
                                                      dptr<uint8_t>(L.leaf), dptr<T4>(xyz_tmp), dptr<int32_t>(perm_tmp),
                                                      dptr<T4>(xyz), dptr<int32_t>(perm));
        EDFMM_LAUNCH_CHECK("k_copy_back");
        // next level
        if ((rc = scan_exclusive(dptr<int32_t>(nchild), dptr<int32_t>(child_off), K, dptr<int64_t>(total), scan_tmp.p, s)))
            return rc;
        int64_t Kn = 0;
        EDFMM_CUDA_TRY(cudaMemcpyAsync(&Kn, total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
        int next_base = L.base + K;
        Level<T> next;
        next.K = (int)Kn;
        next.base = next_base;
        if (Kn > 0) {
            if ((rc = next.rng.reserve(sizeof(int2) * Kn)) || (rc = next.parent.reserve(sizeof(int32_t) * Kn)) ||
                (rc = next.root.reserve(sizeof(int32_t) * Kn)))
                return rc;
        }
        k_make_children<<<nblk(K, 256), 256, 0, s>>>(K, dptr<uint8_t>(L.leaf), dptr<int32_t>(oct_start),
                                                     dptr<int32_t>(oct_cnt), dptr<int32_t>(child_off), L.base, next_base,
                                                     dptr<int2>(next.rng), dptr<int32_t>(next.parent),
                                                     dptr<int32_t>(L.children), dptr<int32_t>(L.root),
                                                     dptr<int32_t>(next.root));
        EDFMM_LAUNCH_CHECK("k_make_children");
        if (Kn == 0) break;
        total_nodes += Kn;
        if (total_nodes >= (int64_t)INT32_MAX / 8) return fail(EDFMM_ERR_ARG, "octree too large");
        levels.push_back(std::move(next));
    }
    const int64_t M = total_nodes;
    const int nlev = (int)levels.size();
    // concatenate the levels (BFS order)
    DevBuf b_rng, b_lev, b_par, b_ch, b_cen, b_hal, b_leaf, b_root;
    if ((rc = b_rng.reserve(sizeof(int2) * M)) || (rc = b_lev.reserve(sizeof(int32_t) * M)) ||
        (rc = b_par.reserve(sizeof(int32_t) * M)) || (rc = b_ch.reserve(sizeof(int32_t) * 8 * M)) ||
        (rc = b_cen.reserve(sizeof(T4) * M)) || (rc = b_hal.reserve(sizeof(T4) * M)) || (rc = b_leaf.reserve(M)) ||
        (rc = b_root.reserve(sizeof(int32_t) * M)))
        return rc;
    std::vector<int32_t> hlev(M);
    tree.level_offsets.assign(nlev + 1, 0);
    for (int l = 0; l < nlev; ++l) {
        Level<T> &L = levels[l];
        size_t b = L.base;
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<int2>(b_rng) + b, L.rng.p, sizeof(int2) * L.K, cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<int32_t>(b_par) + b, L.parent.p, sizeof(int32_t) * L.K, cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<int32_t>(b_ch) + 8 * b, L.children.p, sizeof(int32_t) * 8 * L.K,
                                       cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<T4>(b_cen) + b, L.center.p, sizeof(T4) * L.K, cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<T4>(b_hal) + b, L.half.p, sizeof(T4) * L.K, cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<uint8_t>(b_leaf) + b, L.leaf.p, L.K, cudaMemcpyDeviceToDevice, s));
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<int32_t>(b_root) + b, L.root.p, sizeof(int32_t) * L.K,
                                       cudaMemcpyDeviceToDevice, s));
        for (int i = 0; i < L.K; ++i) hlev[b + i] = l;
        tree.level_offsets[l + 1] = L.base + L.K;
    }
    EDFMM_CUDA_TRY(cudaMemcpyAsync(b_lev.p, hlev.data(), sizeof(int32_t) * M, cudaMemcpyHostToDevice, s));
    // DFS numbering
    DevBuf cnt_at, minlev_at, base_at, dfs;
    if ((rc = cnt_at.reserve(sizeof(int32_t) * n)) || (rc = minlev_at.reserve(sizeof(int32_t) * n)) ||
        (rc = base_at.reserve(sizeof(int32_t) * n)) || (rc = dfs.reserve(sizeof(int32_t) * M)) ||
        (rc = scan_tmp.reserve(scan_tmp_bytes(std::max<int64_t>(n, M)))))
        return rc;
    EDFMM_CUDA_TRY(cudaMemsetAsync(cnt_at.p, 0, sizeof(int32_t) * n, s));
    EDFMM_CUDA_TRY(cudaMemsetAsync(minlev_at.p, 0x7f, sizeof(int32_t) * n, s));
    k_dfs_marks<<<nblk(M, 256), 256, 0, s>>>(dptr<int2>(b_rng), dptr<int32_t>(b_lev), M, dptr<int32_t>(cnt_at),
                                             dptr<int32_t>(minlev_at));
    EDFMM_LAUNCH_CHECK("k_dfs_marks");
    if ((rc = scan_exclusive(dptr<int32_t>(cnt_at), dptr<int32_t>(base_at), n, nullptr, scan_tmp.p, s))) return rc;
    k_dfs_ids<<<nblk(M, 256), 256, 0, s>>>(dptr<int2>(b_rng), dptr<int32_t>(b_lev), M, dptr<int32_t>(base_at),
                                           dptr<int32_t>(minlev_at), dptr<int32_t>(dfs));
    EDFMM_LAUNCH_CHECK("k_dfs_ids");
    // each root's radius sets the floor of its tree's expansion scales
    DevBuf floors;
    if ((rc = floors.reserve(sizeof(T) * K0))) return rc;
    k_root_floors<T><<<nblk(K0, 256), 256, 0, s>>>(dptr<T4>(b_cen), K0, dptr<T>(floors));
    EDFMM_LAUNCH_CHECK("k_root_floors");
    if ((rc = tree.range.reserve(sizeof(int2) * M)) || (rc = tree.level.reserve(sizeof(int32_t) * M)) ||
        (rc = tree.parent.reserve(sizeof(int32_t) * M)) || (rc = tree.children.reserve(sizeof(int32_t) * 8 * M)) ||
        (rc = tree.center.reserve(sizeof(T4) * M)) || (rc = tree.half.reserve(sizeof(T4) * M)) ||
        (rc = tree.is_leaf.reserve(M)) || (rc = tree.level_nodes.reserve(sizeof(int32_t) * M)))
        return rc;
    k_permute_nodes<T><<<nblk(M, 256), 256, 0, s>>>(
        M, dptr<int32_t>(dfs), dptr<int2>(b_rng), dptr<int32_t>(b_lev), dptr<int32_t>(b_par), dptr<int32_t>(b_ch),
        dptr<T4>(b_cen), dptr<T4>(b_hal), dptr<uint8_t>(b_leaf), dptr<int32_t>(b_root), dptr<T>(floors),
        dptr<int2>(tree.range), dptr<int32_t>(tree.level),
        dptr<int32_t>(tree.parent), dptr<int32_t>(tree.children), dptr<T4>(tree.center), dptr<T4>(tree.half),
        dptr<uint8_t>(tree.is_leaf), dptr<int32_t>(tree.level_nodes));
    EDFMM_LAUNCH_CHECK("k_permute_nodes");
    for (size_t l = 1; l + 1 < tree.level_offsets.size(); ++l) {
        const int a = tree.level_offsets[l], b = tree.level_offsets[l + 1];
        if (b <= a) continue;
        k_scale_from_parent<T><<<nblk(b - a, 256), 256, 0, s>>>(dptr<int32_t>(tree.level_nodes) + a, b - a,
                                                                 dptr<int32_t>(tree.parent), dptr<T4>(tree.half));
        EDFMM_LAUNCH_CHECK("k_scale_from_parent");
    }
    // leaves
    DevBuf flag, loff;
    if ((rc = flag.reserve(sizeof(int32_t) * M)) || (rc = loff.reserve(sizeof(int32_t) * M))) return rc;
    k_leaf_flags<<<nblk(M, 256), 256, 0, s>>>(dptr<uint8_t>(tree.is_leaf), M, dptr<int32_t>(flag));
    EDFMM_LAUNCH_CHECK("k_leaf_flags");
    if ((rc = scan_exclusive(dptr<int32_t>(flag), dptr<int32_t>(loff), M, dptr<int64_t>(total), scan_tmp.p, s))) return rc;
    int64_t nleaves = 0;
    int hwarn = 0;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&nleaves, total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&hwarn, warn.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    if ((rc = tree.leaves.reserve(sizeof(int32_t) * nleaves))) return rc;
    k_leaf_compact<<<nblk(M, 256), 256, 0, s>>>(dptr<uint8_t>(tree.is_leaf), M, dptr<int32_t>(loff), dptr<int32_t>(tree.leaves));
    EDFMM_LAUNCH_CHECK("k_leaf_compact");
    // points in tree order: keep xyz (charges filled per matvec), permutation
    if ((rc = tree.pts.reserve(sizeof(T4) * n)) || (rc = tree.index_map.reserve(sizeof(int32_t) * n))) return rc;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(tree.pts.p, xyz.p, sizeof(T4) * n, cudaMemcpyDeviceToDevice, s));
    EDFMM_CUDA_TRY(cudaMemcpyAsync(tree.index_map.p, perm.p, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    tree.n_nodes = M;
    tree.n_leaves = nleaves;
    tree.max_level = nlev - 1;
    tree.depth_warnings = hwarn;
    tree.n_inst = 0;
    if (inst_off) {
        // instance k owns the DFS range [root_k, root_{k+1}) (roots are BFS 0..K0-1)
        tree.n_inst = K0;
        if ((rc = tree.inst_node_off.reserve(sizeof(int32_t) * (K0 + 1)))) return rc;
        k_inst_node_off<<<nblk(K0 + 1, 256), 256, 0, s>>>(dptr<int32_t>(tree.level_nodes), K0, (int32_t)M,
                                                           dptr<int32_t>(tree.inst_node_off));
        EDFMM_LAUNCH_CHECK("k_inst_node_off");
    }
    return EDFMM_OK;
}

}  // namespace

int tree_build(const void *points_dev, int64_t n, int dtype, int leaf_size, int max_depth, DevTree &tree,
               cudaStream_t s) {
    if (dtype == EDFMM_F64) return build_impl<double>(points_dev, n, leaf_size, max_depth, tree, s, nullptr, 1);
    return build_impl<float>(points_dev, n, leaf_size, max_depth, tree, s, nullptr, 1);
}

int tree_build_forest(const void *points_dev, const int64_t *inst_off, int n_inst, int dtype, int leaf_size,
                      int max_depth, DevTree &tree, cudaStream_t s) {
    const int64_t n = inst_off[n_inst];
    if (dtype == EDFMM_F64) return build_impl<double>(points_dev, n, leaf_size, max_depth, tree, s, inst_off, n_inst);
    return build_impl<float>(points_dev, n, leaf_size, max_depth, tree, s, inst_off, n_inst);
}

}  // namespace edfmm
