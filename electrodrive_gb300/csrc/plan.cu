// C ABI of libedfmm: plan life cycle, exports and the matvec pipeline.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

#include "edfmm_internal.cuh"
#include "harmonics.cuh"

namespace edfmm {

namespace {
thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};

inline cudaStream_t S(void *s) { return static_cast<cudaStream_t>(s); }
inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <typename T>
__global__ void k_export_tree(int64_t M, int64_t N, const int32_t *idx, const typename Vec4<T>::type *center,
                              const typename Vec4<T>::type *half, const int2 *range, const int32_t *parent,
                              const int32_t *children, const int32_t *level, const uint8_t *leaf, int64_t *o_idx,
                              T *o_c, T *o_h, T *o_r, int32_t *o_lev, int64_t *o_par, int64_t *o_ch, int64_t *o_rng,
                              uint8_t *o_leaf) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o_idx && i < N) o_idx[i] = idx[i];
    if (i >= M) return;
    typename Vec4<T>::type c = center[i], h = half[i];
    if (o_c) {
        o_c[3 * i] = c.x;
        o_c[3 * i + 1] = c.y;
        o_c[3 * i + 2] = c.z;
    }
    if (o_h) {
        o_h[3 * i] = h.x;
        o_h[3 * i + 1] = h.y;
        o_h[3 * i + 2] = h.z;
    }
    if (o_r) o_r[i] = c.w;
    if (o_lev) o_lev[i] = level[i];
    if (o_par) o_par[i] = parent[i];
    if (o_ch)
        for (int o = 0; o < 8; ++o) o_ch[8 * i + o] = children[8 * i + o];
    if (o_rng) {
        o_rng[2 * i] = range[i].x;
        o_rng[2 * i + 1] = range[i].y;
    }
    if (o_leaf) o_leaf[i] = leaf[i];
}

__global__ void k_export_pairs(int64_t rows, const int32_t *off, const int32_t *src, int64_t *out) {
    int64_t r = (int64_t)blockIdx.x * blockDim.y + threadIdx.y;
    if (r >= rows) return;
    for (int k = off[r] + threadIdx.x; k < off[r + 1]; k += blockDim.x) {
        out[2 * (int64_t)k] = src[k];
        out[2 * (int64_t)k + 1] = r;
    }
}

template <typename T>
__global__ void k_export_coeffs(int64_t M, int nc, int nc_pad, const Cplx<T> *in, Cplx<T> *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * nc) return;
    int64_t node = i / nc;
    int c = (int)(i % nc);
    out[i] = in[node * nc_pad + c];
}

template <typename Tin, typename Tout>
__global__ void k_cast_vals(const Tin *in, Tout *out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (Tout)in[i];
}

// whole-buffer device copy
int clone_buf(const DevBuf &src, DevBuf &dst, cudaStream_t s) {
    if (!src.p) return EDFMM_OK;
    if (int rc = dst.reserve(src.bytes)) return rc;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(dst.p, src.p, src.bytes, cudaMemcpyDeviceToDevice, s));
    return EDFMM_OK;
}

// n values of the source dtype into a new buffer of the target dtype
int cast_buf(const DevBuf &src, int sdt, DevBuf &dst, int ddt, int64_t n, cudaStream_t s) {
    if (int rc = dst.reserve((ddt == EDFMM_F64 ? 8 : 4) * (size_t)std::max<int64_t>(n, 1))) return rc;
    if (n <= 0) return EDFMM_OK;
    const unsigned g = (unsigned)((n + 255) / 256);
    if (sdt == ddt) {
        EDFMM_CUDA_TRY(cudaMemcpyAsync(dst.p, src.p, (sdt == EDFMM_F64 ? 8 : 4) * (size_t)n,
                                       cudaMemcpyDeviceToDevice, s));
    } else if (sdt == EDFMM_F64) {
        k_cast_vals<double, float><<<g, 256, 0, s>>>(dptr<double>(src), dptr<float>(dst), n);
        EDFMM_LAUNCH_CHECK("k_cast_vals");
    } else {
        k_cast_vals<float, double><<<g, 256, 0, s>>>(dptr<float>(src), dptr<double>(dst), n);
        EDFMM_LAUNCH_CHECK("k_cast_vals");
    }
    return EDFMM_OK;
}

int alloc_expansions(edfmm_plan *p, int dtype, int expansion_order, cudaStream_t s) {
    p->fmm.p = expansion_order;
    p->fmm.nc = num_coeffs(expansion_order);
    p->fmm.nc_pad = (p->fmm.nc + 1) & ~1;
    size_t esz = (dtype == EDFMM_F64 ? 16 : 8) * (size_t)p->fmm.nc_pad * (size_t)std::max<int64_t>(p->tree.n_nodes, 1);
    int rc = p->fmm.multipoles.reserve(esz);
    if (!rc) rc = p->fmm.locals.reserve(esz);
    if (!rc) rc = p->fmm.translated.reserve(esz);
    if (!rc) {
        cudaError_t e = cudaMemsetAsync(p->fmm.multipoles.p, 0, esz, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(p->fmm.locals.p, 0, esz, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("plan set-up: ") + cudaGetErrorString(e));
    }
    return rc;
}

// Plan buffers built inside a BlockCacheScope may sit in cached blocks larger
// than they need; move those to exact-size blocks before the plan is handed out.
int shrink_tree_lists(DevTree &t, DevLists &l, cudaStream_t s) {
    DevBuf *bufs[] = {&t.pts,      &t.index_map,     &t.center,      &t.half,    &t.range,
                      &t.parent,   &t.children,      &t.level,       &t.is_leaf, &t.leaves,
                      &t.level_nodes, &t.inst_node_off, &l.p2p_off,  &l.p2p_src, &l.m2l_off,
                      &l.m2l_src,  &l.m2l_swapped_off, &l.m2l_swapped_src, &l.p2p_leaves, &l.m2l_rows};
    for (DevBuf *b : bufs)
        if (int rc = b->shrink_to_fit(s)) return rc;
    return EDFMM_OK;
}

int check_plan(const edfmm_plan *p) {
    if (!p) return fail(EDFMM_ERR_ARG, "plan is NULL");
    return EDFMM_OK;
}

}  // namespace

struct BlockCache {
    std::multimap<size_t, void *> free_blocks;  // by size
};

namespace {
thread_local BlockCache *g_block_cache = nullptr;
}

BlockCache *block_cache() { return g_block_cache; }

void *block_cache_take(BlockCache *c, size_t nbytes, size_t *got) {
    // the smallest held block that fits, unless it is more than twice the request
    auto it = c->free_blocks.lower_bound(nbytes);
    if (it == c->free_blocks.end() || it->first > 2 * nbytes + 256) return nullptr;
    void *p = it->second;
    *got = it->first;
    c->free_blocks.erase(it);
    return p;
}

void block_cache_put(BlockCache *c, void *p, size_t nbytes) { c->free_blocks.emplace(nbytes, p); }

void block_cache_trim(BlockCache *c) {
    for (auto &kv : c->free_blocks) cudaFree(kv.second);
    c->free_blocks.clear();
}

cudaError_t malloc_or_trim(void **p, size_t nbytes) {
    cudaError_t e = cudaMalloc(p, nbytes);
    BlockCache *c = block_cache();
    if (e == cudaErrorMemoryAllocation && c && !c->free_blocks.empty()) {
        (void)cudaGetLastError();  // clear the failed allocation's error state
        block_cache_trim(c);
        e = cudaMalloc(p, nbytes);
    }
    return e;
}

BlockCacheScope::BlockCacheScope() : prev(g_block_cache), cache(new BlockCache()) { g_block_cache = cache; }

BlockCacheScope::~BlockCacheScope() {
    g_block_cache = prev;
    for (auto &kv : cache->free_blocks) cudaFree(kv.second);  // cudaFree waits for the device
    delete cache;
}

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace edfmm

using namespace edfmm;

extern "C" {

const char *edfmm_last_error(void) { return g_last_error.c_str(); }

const char *edfmm_version(void) { return "edfmm 0.1 (sm_103a)"; }

int64_t edfmm_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int edfmm_plan_create(const void *points_dev, int64_t n, int dtype, int leaf_size, int max_depth, double mac_theta,
                      int expansion_order, void *stream, edfmm_plan **plan_out) {
    if (!plan_out) return fail(EDFMM_ERR_ARG, "plan_out is NULL");
    *plan_out = nullptr;
    if (n < 0) return fail(EDFMM_ERR_ARG, "n must be >= 0");
    if (n > 0 && !points_dev) return fail(EDFMM_ERR_ARG, "points_dev is NULL");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (leaf_size <= 0) return fail(EDFMM_ERR_ARG, "leaf_size must be positive");
    if (max_depth <= 0 || max_depth > 64) return fail(EDFMM_ERR_ARG, "max_depth must be in [1, 64]");
    if (!(mac_theta > 0.0 && mac_theta < 1.0)) return fail(EDFMM_ERR_ARG, "mac_theta must be in (0, 1)");
    if (expansion_order < 1 || expansion_order > 10)
        return fail(EDFMM_ERR_UNSUPPORTED, "expansion_order must be in [1, 10]");
    int rc = upload_tables();
    if (rc) return rc;
    edfmm_plan *p = new edfmm_plan();
    cudaGetDevice(&p->device);
    p->mac_theta = mac_theta;
    p->leaf_size = leaf_size;
    p->max_depth = max_depth;
    cudaStream_t s = S(stream);
    BlockCacheScope cache_scope;  // the build runs on `s` alone
    rc = tree_build(points_dev, n, dtype, leaf_size, max_depth, p->tree, s);
    if (!rc) rc = lists_build(p->tree, mac_theta, p->lists, s);
    if (!rc) rc = shrink_tree_lists(p->tree, p->lists, s);
    if (!rc) {
        p->fmm.p = expansion_order;
        p->fmm.nc = num_coeffs(expansion_order);
        p->fmm.nc_pad = (p->fmm.nc + 1) & ~1;
        size_t esz = (dtype == EDFMM_F64 ? 16 : 8) * (size_t)p->fmm.nc_pad * (size_t)std::max<int64_t>(p->tree.n_nodes, 1);
        rc = p->fmm.multipoles.reserve(esz);
        if (!rc) rc = p->fmm.locals.reserve(esz);
        if (!rc) rc = p->fmm.translated.reserve(esz);
        if (!rc) rc = p->fmm.multipoles.shrink_to_fit(s);
        if (!rc) rc = p->fmm.locals.shrink_to_fit(s);
        if (!rc) rc = p->fmm.translated.shrink_to_fit(s);
        if (!rc) {
            cudaError_t e = cudaMemsetAsync(p->fmm.multipoles.p, 0, esz, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(p->fmm.locals.p, 0, esz, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("plan set-up: ") + cudaGetErrorString(e));
        }
    }
    if (rc) {
        delete p;
        return rc;
    }
    *plan_out = p;
    return EDFMM_OK;
}

int edfmm_plan_create_batch(const void *points_dev, const int64_t *offsets, int n_instances, int dtype, int leaf_size,
                            int max_depth, double mac_theta, int expansion_order, void *stream, edfmm_plan **plan_out) {
    if (!plan_out) return fail(EDFMM_ERR_ARG, "plan_out is NULL");
    *plan_out = nullptr;
    if (n_instances <= 0 || !offsets || !points_dev) return fail(EDFMM_ERR_ARG, "need points, offsets and >= 1 instance");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (leaf_size <= 0) return fail(EDFMM_ERR_ARG, "leaf_size must be positive");
    if (max_depth <= 0 || max_depth > 64) return fail(EDFMM_ERR_ARG, "max_depth must be in [1, 64]");
    if (!(mac_theta > 0.0 && mac_theta < 1.0)) return fail(EDFMM_ERR_ARG, "mac_theta must be in (0, 1)");
    if (expansion_order < 1 || expansion_order > 10)
        return fail(EDFMM_ERR_UNSUPPORTED, "expansion_order must be in [1, 10]");
    if (offsets[0] != 0) return fail(EDFMM_ERR_ARG, "offsets[0] must be 0");
    for (int i = 0; i < n_instances; ++i)
        if (offsets[i + 1] <= offsets[i]) return fail(EDFMM_ERR_ARG, "every instance needs at least one point");
    int rc = upload_tables();
    if (rc) return rc;
    cudaStream_t s = S(stream);
    // every build below runs on `s`: temporaries are recycled in stream order
    BlockCacheScope cache_scope;
    // one forest over all instances, level by level (each instance's tree and
    // lists equal what edfmm_plan_create builds for it alone)
    edfmm_plan *p = new edfmm_plan();
    cudaGetDevice(&p->device);
    p->mac_theta = mac_theta;
    p->leaf_size = leaf_size;
    p->max_depth = max_depth;
    if (offsets[n_instances] >= (int64_t)INT32_MAX) {
        delete p;
        return fail(EDFMM_ERR_UNSUPPORTED, "batched plan exceeds 32-bit point indices");
    }
    rc = tree_build_forest(points_dev, offsets, n_instances, dtype, leaf_size, max_depth, p->tree, s);
    if (!rc) rc = lists_build(p->tree, mac_theta, p->lists, s);
    if (!rc) rc = shrink_tree_lists(p->tree, p->lists, s);
    if (!rc) {
        p->fmm.p = expansion_order;
        p->fmm.nc = num_coeffs(expansion_order);
        p->fmm.nc_pad = (p->fmm.nc + 1) & ~1;
        size_t esz = (dtype == EDFMM_F64 ? 16 : 8) * (size_t)p->fmm.nc_pad * (size_t)std::max<int64_t>(p->tree.n_nodes, 1);
        rc = p->fmm.multipoles.reserve(esz);
        if (!rc) rc = p->fmm.locals.reserve(esz);
        if (!rc) rc = p->fmm.translated.reserve(esz);
        if (!rc) rc = p->fmm.multipoles.shrink_to_fit(s);
        if (!rc) rc = p->fmm.locals.shrink_to_fit(s);
        if (!rc) rc = p->fmm.translated.shrink_to_fit(s);
        if (!rc) {
            cudaError_t e = cudaMemsetAsync(p->fmm.multipoles.p, 0, esz, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(p->fmm.locals.p, 0, esz, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("plan set-up: ") + cudaGetErrorString(e));
        }
    }
    if (rc) {
        delete p;
        return rc;
    }
    *plan_out = p;
    return EDFMM_OK;
}

int edfmm_plan_convert(const edfmm_plan *src, int dtype, int expansion_order, void *stream, edfmm_plan **plan_out) {
    if (!plan_out) return fail(EDFMM_ERR_ARG, "plan_out is NULL");
    *plan_out = nullptr;
    if (int rc = check_plan(src)) return rc;
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (expansion_order < 1 || expansion_order > 10)
        return fail(EDFMM_ERR_UNSUPPORTED, "expansion_order must be in [1, 10]");
    cudaStream_t s = S(stream);
    edfmm_plan *p = new edfmm_plan();
    cudaGetDevice(&p->device);
    p->mac_theta = src->mac_theta;
    p->leaf_size = src->leaf_size;
    p->max_depth = src->max_depth;
    const DevTree &a = src->tree;
    DevTree &t = p->tree;
    t.dtype = dtype;
    t.n_points = a.n_points;
    t.n_nodes = a.n_nodes;
    t.n_leaves = a.n_leaves;
    t.max_level = a.max_level;
    t.depth_warnings = a.depth_warnings;
    t.level_offsets = a.level_offsets;
    t.n_inst = a.n_inst;
    const DevLists &la = src->lists;
    DevLists &l = p->lists;
    l.n_p2p = la.n_p2p;
    l.n_m2l = la.n_m2l;
    l.p2p_interactions = la.p2p_interactions;
    l.max_p2p_row = la.max_p2p_row;
    l.max_m2l_row = la.max_m2l_row;
    l.have_m2l_swapped = la.have_m2l_swapped;
    int rc = EDFMM_OK;
    if (!rc) rc = cast_buf(a.pts, a.dtype, t.pts, dtype, 4 * a.n_points, s);
    if (!rc) rc = cast_buf(a.center, a.dtype, t.center, dtype, 4 * a.n_nodes, s);
    if (!rc) rc = cast_buf(a.half, a.dtype, t.half, dtype, 4 * a.n_nodes, s);
    const DevBuf *from[] = {&a.index_map, &a.range, &a.parent, &a.children, &a.level, &a.is_leaf, &a.leaves,
                            &a.level_nodes, &a.inst_node_off, &la.p2p_off, &la.p2p_src, &la.m2l_off, &la.m2l_src,
                            &la.m2l_swapped_off, &la.m2l_swapped_src, &la.p2p_leaves, &la.m2l_rows};
    DevBuf *to[] = {&t.index_map, &t.range, &t.parent, &t.children, &t.level, &t.is_leaf, &t.leaves,
                    &t.level_nodes, &t.inst_node_off, &l.p2p_off, &l.p2p_src, &l.m2l_off, &l.m2l_src,
                    &l.m2l_swapped_off, &l.m2l_swapped_src, &l.p2p_leaves, &l.m2l_rows};
    for (size_t i = 0; !rc && i < sizeof(from) / sizeof(from[0]); ++i) rc = clone_buf(*from[i], *to[i], s);
    if (!rc) rc = alloc_expansions(p, dtype, expansion_order, s);  // synchronises the stream
    if (rc) {
        delete p;
        return rc;
    }
    *plan_out = p;
    return EDFMM_OK;
}

int edfmm_block_cache_selfcheck(int64_t *results_host) {
    if (!results_host) return fail(EDFMM_ERR_ARG, "results_host is NULL");
    for (int i = 0; i < 4; ++i) results_host[i] = 0;
    BlockCacheScope scope;
    void *small_block = nullptr;
    {
        DevBuf a, b;
        if (int rc = a.reserve(1 << 20)) return rc;
        if (int rc = b.reserve(3 << 20)) return rc;
        small_block = a.p;
    }  // both blocks now held by the cache
    // larger than anything cached: a fresh allocation
    DevBuf big;
    if (int rc = big.reserve(16 << 20)) return rc;
    results_host[0] = (big.p != nullptr && big.bytes == (16u << 20)) ? 1 : 0;
    // within 2x of a cached block: the 1 MiB block is reused
    DevBuf reuse;
    if (int rc = reuse.reserve(700 << 10)) return rc;
    results_host[1] = (reuse.p == small_block && reuse.bytes == (1u << 20)) ? 1 : 0;
    // a persistent buffer that took the 3 MiB block for 2 MiB moves to 2 MiB
    DevBuf keep;
    if (int rc = keep.reserve(2 << 20)) return rc;
    results_host[2] = keep.bytes == (3u << 20) ? 1 : 0;
    if (int rc = keep.shrink_to_fit(nullptr)) return rc;
    results_host[3] = (keep.bytes == (2u << 20) && keep.used == (2u << 20)) ? 1 : 0;
    EDFMM_CUDA_TRY(cudaDeviceSynchronize());
    return EDFMM_OK;
}

int edfmm_plan_destroy(edfmm_plan *plan) {
    delete plan;
    return EDFMM_OK;
}

int edfmm_plan_set_arithmetic(edfmm_plan *p, int mode, void *stream) {
    if (int rc = check_plan(p)) return rc;
    if (mode != EDFMM_ARITH_NATIVE && mode != EDFMM_ARITH_TWO_FLOAT)
        return fail(EDFMM_ERR_ARG, "mode must be EDFMM_ARITH_NATIVE or EDFMM_ARITH_TWO_FLOAT");
    cudaStream_t s = S(stream);
    if (mode == EDFMM_ARITH_NATIVE) {
        p->tree.pts_tf.release();
        p->tree.nodes_tf.release();
        p->fmm.mult_tf.release();
        p->fmm.arith = EDFMM_ARITH_NATIVE;
        return EDFMM_OK;
    }
    if (p->tree.dtype != EDFMM_F64) return fail(EDFMM_ERR_UNSUPPORTED, "two-float arithmetic applies to FP64 plans");
    if (p->tree.n_points > 0) {
        if (int rc = p->tree.pts_tf.reserve(sizeof(float) * 8 * (size_t)p->tree.n_points)) return rc;
        if (int rc = set_charges(p->tree, nullptr, nullptr, s)) return rc;  // splits the points and charges
    }
    if (int rc = prepare_two_float(p->tree, p->fmm, s)) return rc;  // split nodes, split-multipole buffer
    // the pairs the two-float M2L leaves to the FP64 kernel, built now (it
    // synchronises the stream) rather than inside a later matvec
    if (int rc = prepare_extreme_rows(p->tree, p->lists, p->fmm, s)) return rc;
    p->fmm.arith = EDFMM_ARITH_TWO_FLOAT;
    return EDFMM_OK;
}

int edfmm_plan_set_launch(edfmm_plan *p, int knob, int value) {
    if (int rc = check_plan(p)) return rc;
    switch (knob) {
    case EDFMM_LAUNCH_M2L_TF_BLOCK:
        if (value != 128 && value != 256) return fail(EDFMM_ERR_ARG, "two-float M2L block must be 128 or 256");
        p->fmm.m2l_tf_block = value;
        return EDFMM_OK;
    case EDFMM_LAUNCH_NEAR_OVERLAP:
        if (value != 0 && value != 1) return fail(EDFMM_ERR_ARG, "near-field overlap must be 0 or 1");
        p->fmm.near_overlap = value;
        return EDFMM_OK;
    case EDFMM_LAUNCH_M2L_PACKED:
        if (value != 0 && value != 1) return fail(EDFMM_ERR_ARG, "packed M2L must be 0 or 1");
        p->fmm.m2l_packed = value;
        return EDFMM_OK;
    default:
        return fail(EDFMM_ERR_ARG, "unknown launch knob");
    }
}

int edfmm_plan_get_launch(const edfmm_plan *p, int knob, int *value) {
    if (int rc = check_plan(p)) return rc;
    if (!value) return fail(EDFMM_ERR_ARG, "value is NULL");
    switch (knob) {
    case EDFMM_LAUNCH_M2L_TF_BLOCK: *value = p->fmm.m2l_tf_block; return EDFMM_OK;
    case EDFMM_LAUNCH_NEAR_OVERLAP: *value = p->fmm.near_overlap; return EDFMM_OK;
    case EDFMM_LAUNCH_M2L_PACKED: *value = p->fmm.m2l_packed; return EDFMM_OK;
    default: return fail(EDFMM_ERR_ARG, "unknown launch knob");
    }
}

int edfmm_plan_rebuild_lists(edfmm_plan *p, double mac_theta, void *stream) {
    if (int rc = check_plan(p)) return rc;
    if (!(mac_theta > 0.0 && mac_theta < 1.0)) return fail(EDFMM_ERR_ARG, "mac_theta must be in (0, 1)");
    if (mac_theta == p->mac_theta) return EDFMM_OK;
    if (int rc = lists_build(p->tree, mac_theta, p->lists, S(stream))) return rc;
    p->mac_theta = mac_theta;
    p->fmm.extreme = ExtremeRows();
    p->fmm.extreme_swapped = ExtremeRows();
    if (p->fmm.arith == EDFMM_ARITH_TWO_FLOAT) {
        if (int rc = prepare_extreme_rows(p->tree, p->lists, p->fmm, S(stream))) return rc;
    }
    return EDFMM_OK;
}

int edfmm_plan_set_instance_mask(edfmm_plan *p, const double *flags_dev, int stride) {
    if (int rc = check_plan(p)) return rc;
    if (!flags_dev) {
        p->fmm.mask = InstMask{};
        return EDFMM_OK;
    }
    if (p->tree.n_inst <= 0) return fail(EDFMM_ERR_ARG, "the instance mask needs a batched plan");
    if (stride < 1) return fail(EDFMM_ERR_ARG, "stride must be >= 1");
    InstMask m;
    m.node_off = dptr<int32_t>(p->tree.inst_node_off);
    m.n_inst = p->tree.n_inst;
    m.flags = flags_dev;
    m.stride = stride;
    p->fmm.mask = m;
    return EDFMM_OK;
}

int edfmm_plan_set_order(edfmm_plan *p, int expansion_order, void *stream) {
    if (int rc = check_plan(p)) return rc;
    if (expansion_order < 1 || expansion_order > 10)
        return fail(EDFMM_ERR_UNSUPPORTED, "expansion_order must be in [1, 10]");
    if (expansion_order == p->fmm.p) return EDFMM_OK;
    cudaStream_t s = S(stream);
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    p->fmm.p = expansion_order;
    p->fmm.nc = num_coeffs(expansion_order);
    p->fmm.nc_pad = (p->fmm.nc + 1) & ~1;
    size_t esz = (p->tree.dtype == EDFMM_F64 ? 16 : 8) * (size_t)p->fmm.nc_pad *
                 (size_t)std::max<int64_t>(p->tree.n_nodes, 1);
    p->fmm.multipoles.release();
    p->fmm.locals.release();
    p->fmm.translated.release();
    int rc = p->fmm.multipoles.reserve(esz);
    if (!rc) rc = p->fmm.locals.reserve(esz);
    if (!rc) rc = p->fmm.translated.reserve(esz);
    if (rc) return rc;
    EDFMM_CUDA_TRY(cudaMemsetAsync(p->fmm.multipoles.p, 0, esz, s));
    EDFMM_CUDA_TRY(cudaMemsetAsync(p->fmm.locals.p, 0, esz, s));
    if (p->fmm.arith == EDFMM_ARITH_TWO_FLOAT) {
        if ((rc = prepare_two_float(p->tree, p->fmm, s))) return rc;  // split-multipole buffer at the new order
    }
    return EDFMM_OK;
}

int edfmm_plan_get_info(const edfmm_plan *p, edfmm_plan_info *info) {
    if (int rc = check_plan(p)) return rc;
    if (!info) return fail(EDFMM_ERR_ARG, "info is NULL");
    std::memset(info, 0, sizeof(*info));
    info->n_points = p->tree.n_points;
    info->n_nodes = p->tree.n_nodes;
    info->n_leaves = p->tree.n_leaves;
    info->n_p2p_pairs = p->lists.n_p2p;
    info->n_m2l_pairs = p->lists.n_m2l;
    info->p2p_interactions = p->lists.p2p_interactions;
    info->max_level = p->tree.max_level;
    info->depth_warnings = p->tree.depth_warnings;
    info->dtype = p->tree.dtype;
    info->expansion_order = p->fmm.p;
    info->leaf_size = p->leaf_size;
    info->max_depth = p->max_depth;
    info->mac_theta = p->mac_theta;
    return EDFMM_OK;
}

int edfmm_plan_export_tree(const edfmm_plan *p, int64_t *index_map, void *centers, void *half_extents, void *radii,
                           int32_t *levels, int64_t *parents, int64_t *children, int64_t *ranges, uint8_t *is_leaf,
                           void *stream) {
    if (int rc = check_plan(p)) return rc;
    const DevTree &t = p->tree;
    int64_t n = std::max(t.n_nodes, t.n_points);
    if (n == 0) return EDFMM_OK;
    if (t.dtype == EDFMM_F64)
        k_export_tree<double><<<nblk(n, 256), 256, 0, S(stream)>>>(
            t.n_nodes, t.n_points, dptr<int32_t>(t.index_map), dptr<double4>(t.center), dptr<double4>(t.half),
            dptr<int2>(t.range), dptr<int32_t>(t.parent), dptr<int32_t>(t.children), dptr<int32_t>(t.level),
            dptr<uint8_t>(t.is_leaf), index_map, static_cast<double *>(centers), static_cast<double *>(half_extents),
            static_cast<double *>(radii), levels, parents, children, ranges, is_leaf);
    else
        k_export_tree<float><<<nblk(n, 256), 256, 0, S(stream)>>>(
            t.n_nodes, t.n_points, dptr<int32_t>(t.index_map), dptr<float4>(t.center), dptr<float4>(t.half),
            dptr<int2>(t.range), dptr<int32_t>(t.parent), dptr<int32_t>(t.children), dptr<int32_t>(t.level),
            dptr<uint8_t>(t.is_leaf), index_map, static_cast<float *>(centers), static_cast<float *>(half_extents),
            static_cast<float *>(radii), levels, parents, children, ranges, is_leaf);
    EDFMM_LAUNCH_CHECK("k_export_tree");
    return EDFMM_OK;
}

int edfmm_plan_export_lists(const edfmm_plan *p, int64_t *p2p_pairs, int64_t *m2l_pairs, void *stream) {
    if (int rc = check_plan(p)) return rc;
    const int64_t M = p->tree.n_nodes;
    if (M == 0) return EDFMM_OK;
    dim3 blk(32, 8);
    if (p2p_pairs && p->lists.n_p2p > 0) {
        k_export_pairs<<<nblk(M, 8), blk, 0, S(stream)>>>(M, dptr<int32_t>(p->lists.p2p_off),
                                                           dptr<int32_t>(p->lists.p2p_src), p2p_pairs);
        EDFMM_LAUNCH_CHECK("k_export_pairs");
    }
    if (m2l_pairs && p->lists.n_m2l > 0) {
        k_export_pairs<<<nblk(M, 8), blk, 0, S(stream)>>>(M, dptr<int32_t>(p->lists.m2l_off),
                                                           dptr<int32_t>(p->lists.m2l_src), m2l_pairs);
        EDFMM_LAUNCH_CHECK("k_export_pairs");
    }
    return EDFMM_OK;
}

int edfmm_plan_get_expansions(const edfmm_plan *p, void *multipoles, void *locals, void *stream) {
    if (int rc = check_plan(p)) return rc;
    const int64_t M = p->tree.n_nodes;
    const int nc = p->fmm.nc;
    if (M == 0) return EDFMM_OK;
    for (int k = 0; k < 2; ++k) {
        void *dst = k == 0 ? multipoles : locals;
        if (!dst) continue;
        const DevBuf &src = k == 0 ? p->fmm.multipoles : p->fmm.locals;
        if (p->tree.dtype == EDFMM_F64)
            k_export_coeffs<double><<<nblk(M * nc, 256), 256, 0, S(stream)>>>(M, nc, p->fmm.nc_pad, dptr<Cplx<double>>(src),
                                                                              static_cast<Cplx<double> *>(dst));
        else
            k_export_coeffs<float><<<nblk(M * nc, 256), 256, 0, S(stream)>>>(M, nc, p->fmm.nc_pad, dptr<Cplx<float>>(src),
                                                                             static_cast<Cplx<float> *>(dst));
        EDFMM_LAUNCH_CHECK("k_export_coeffs");
    }
    return EDFMM_OK;
}

int edfmm_plan_set_charges(edfmm_plan *p, const void *charges, void *stream) {
    if (int rc = check_plan(p)) return rc;
    if (p->tree.n_points > 0 && !charges) return fail(EDFMM_ERR_ARG, "charges is NULL");
    return set_charges(p->tree, charges, nullptr, S(stream));
}

int edfmm_plan_p2m(edfmm_plan *p, void *stream) {
    if (int rc = check_plan(p)) return rc;
    return run_p2m(p->tree, p->fmm, S(stream));
}

int edfmm_plan_m2m(edfmm_plan *p, void *stream) {
    if (int rc = check_plan(p)) return rc;
    return run_m2m(p->tree, p->fmm, S(stream));
}

int edfmm_plan_m2l(edfmm_plan *p, int flags, void *stream) {
    if (int rc = check_plan(p)) return rc;
    const bool swapped = (flags & EDFMM_REFERENCE_PAIR_ORDER) != 0;
    if (swapped) {
        if (int rc = lists_build_swapped(p->tree, p->lists, S(stream))) return rc;
    }
    return run_m2l(p->tree, p->lists, p->fmm, swapped, S(stream));
}

int edfmm_plan_l2l(edfmm_plan *p, void *stream) {
    if (int rc = check_plan(p)) return rc;
    return run_l2l(p->tree, p->fmm, S(stream));
}

int edfmm_plan_l2p(edfmm_plan *p, void *phi_far_tree, void *stream) {
    if (int rc = check_plan(p)) return rc;
    if (p->tree.n_points > 0 && !phi_far_tree) return fail(EDFMM_ERR_ARG, "output is NULL");
    NearArgs a;
    a.out = phi_far_tree;
    a.near = false;
    a.far = true;
    return run_p2p_l2p(p->tree, p->lists, p->fmm, a, S(stream));
}

int edfmm_plan_p2p(edfmm_plan *p, void *phi_near_tree, void *stream) {
    if (int rc = check_plan(p)) return rc;
    if (p->tree.n_points > 0 && !phi_near_tree) return fail(EDFMM_ERR_ARG, "output is NULL");
    NearArgs a;
    a.out = phi_near_tree;
    a.near = true;
    a.far = false;
    return run_p2p_l2p(p->tree, p->lists, p->fmm, a, S(stream));
}

int edfmm_plan_matvec(edfmm_plan *p, const void *sigma, const void *areas, const void *self_integrals, double k_e,
                      void *out, int flags, void *stream) {
    if (int rc = check_plan(p)) return rc;
    if (p->tree.n_points == 0) return EDFMM_OK;
    if (!sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "sigma, areas and out must be non-NULL");
    cudaStream_t s = S(stream);
    const bool far = (flags & EDFMM_NO_FARFIELD) == 0;
    const bool near = (flags & EDFMM_NO_NEARFIELD) == 0;
    const bool swapped = (flags & EDFMM_REFERENCE_PAIR_ORDER) != 0;
    int rc;
    if (swapped && (rc = lists_build_swapped(p->tree, p->lists, s))) return rc;
    if ((rc = set_charges(p->tree, sigma, areas, s))) return rc;
    if (far && near && p->fmm.near_overlap) {
        // The near field depends only on the charges: it runs on a second
        // stream beside P2M -> M2M -> M2L -> L2L, into tree-order sums that
        // the final pass (L2P + epilogue) adds.  Fork and join through
        // events, so the pattern is also valid inside a stream capture.
        if (!p->side) {
            EDFMM_CUDA_TRY(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
            EDFMM_CUDA_TRY(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
            EDFMM_CUDA_TRY(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
        }
        const size_t elt = p->tree.dtype == EDFMM_F64 ? sizeof(double) : sizeof(float);
        if ((rc = p->near_sum.reserve(elt * (size_t)p->tree.n_points))) return rc;
        EDFMM_CUDA_TRY(cudaEventRecord(p->ev_fork, s));
        EDFMM_CUDA_TRY(cudaStreamWaitEvent(p->side, p->ev_fork, 0));
        NearArgs an;
        an.out = p->near_sum.p;
        an.scatter = false;
        an.near = true;
        an.far = false;
        if ((rc = run_p2p_l2p(p->tree, p->lists, p->fmm, an, p->side))) return rc;
        EDFMM_CUDA_TRY(cudaEventRecord(p->ev_join, p->side));
        if ((rc = run_p2m(p->tree, p->fmm, s)) || (rc = run_m2m(p->tree, p->fmm, s)) ||
            (rc = run_m2l(p->tree, p->lists, p->fmm, swapped, s)) || (rc = run_l2l(p->tree, p->fmm, s)))
            return rc;
        EDFMM_CUDA_TRY(cudaStreamWaitEvent(s, p->ev_join, 0));
        NearArgs a;
        a.sigma = sigma;
        a.areas = areas;
        a.self_int = self_integrals;
        a.k_e = k_e;
        a.out = out;
        a.scatter = true;
        a.near = false;
        a.far = true;
        a.add_in = p->near_sum.p;
        return run_p2p_l2p(p->tree, p->lists, p->fmm, a, s);
    }
    if (far) {
        if ((rc = run_p2m(p->tree, p->fmm, s)) || (rc = run_m2m(p->tree, p->fmm, s)) ||
            (rc = run_m2l(p->tree, p->lists, p->fmm, swapped, s)) || (rc = run_l2l(p->tree, p->fmm, s)))
            return rc;
    }
    NearArgs a;
    a.sigma = sigma;
    a.areas = areas;
    a.self_int = self_integrals;
    a.k_e = k_e;
    a.out = out;
    a.scatter = true;
    a.near = near;
    a.far = far;
    return run_p2p_l2p(p->tree, p->lists, p->fmm, a, s);
}

struct edfmm_targets {
    edfmm_plan *plan = nullptr;  // source plan (not owned)
    DevTree tree;                // tree of the target points
    DevLists lists;              // rows: target nodes; sources: source-plan nodes
    FmmBuffers buf;              // target locals
};

int edfmm_targets_create(edfmm_plan *p, const void *targets_dev, int64_t m, void *stream, edfmm_targets **out) {
    if (!out) return fail(EDFMM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (int rc = check_plan(p)) return rc;
    if (m < 0 || (m > 0 && !targets_dev)) return fail(EDFMM_ERR_ARG, "need m >= 0 target points");
    if (p->tree.n_inst > 0) return fail(EDFMM_ERR_UNSUPPORTED, "batched plans have no two-tree lists");
    cudaStream_t s = S(stream);
    edfmm_targets *t = new edfmm_targets();
    t->plan = p;
    int rc = tree_build(targets_dev, m, p->tree.dtype, p->leaf_size, p->max_depth, t->tree, s);
    if (!rc) rc = lists_build_two(p->tree, t->tree, p->mac_theta, t->lists, s);
    if (!rc) {
        t->buf.p = p->fmm.p;
        t->buf.nc = p->fmm.nc;
        t->buf.nc_pad = p->fmm.nc_pad;
        const size_t esz = (p->tree.dtype == EDFMM_F64 ? 16 : 8) * (size_t)t->buf.nc_pad *
                           (size_t)std::max<int64_t>(t->tree.n_nodes, 1);
        rc = t->buf.locals.reserve(esz);
        if (!rc) {
            cudaError_t e = cudaMemsetAsync(t->buf.locals.p, 0, esz, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("target set-up: ") + cudaGetErrorString(e));
        }
    }
    if (rc) {
        delete t;
        return rc;
    }
    *out = t;
    return EDFMM_OK;
}

int edfmm_targets_create_from_plan(edfmm_plan *p, const edfmm_plan *tp, double mac_theta, void *stream,
                                   edfmm_targets **out) {
    if (!out) return fail(EDFMM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (int rc = check_plan(p)) return rc;
    if (int rc = check_plan(tp)) return rc;
    if (tp->tree.dtype != p->tree.dtype) return fail(EDFMM_ERR_ARG, "source and target plans must share a dtype");
    if (p->tree.n_inst > 0 || tp->tree.n_inst > 0)
        return fail(EDFMM_ERR_UNSUPPORTED, "batched plans have no two-tree lists");
    if (!(mac_theta > 0.0 && mac_theta < 1.0)) return fail(EDFMM_ERR_ARG, "mac_theta must be in (0, 1)");
    cudaStream_t s = S(stream);
    std::unique_ptr<edfmm_targets> t(new edfmm_targets());
    t->plan = p;
    const DevTree &a = tp->tree;
    DevTree &tt = t->tree;
    tt.dtype = a.dtype;
    tt.n_points = a.n_points;
    tt.n_nodes = a.n_nodes;
    tt.n_leaves = a.n_leaves;
    tt.max_level = a.max_level;
    tt.depth_warnings = a.depth_warnings;
    tt.level_offsets = a.level_offsets;
    const DevBuf *from[] = {&a.pts,     &a.index_map, &a.center, &a.half,   &a.range,
                            &a.parent,  &a.children,  &a.level,  &a.is_leaf, &a.leaves, &a.level_nodes};
    DevBuf *to[] = {&tt.pts,    &tt.index_map, &tt.center, &tt.half,    &tt.range,
                    &tt.parent, &tt.children,  &tt.level,  &tt.is_leaf, &tt.leaves, &tt.level_nodes};
    int rc = EDFMM_OK;
    for (size_t i = 0; !rc && i < sizeof(from) / sizeof(from[0]); ++i) rc = clone_buf(*from[i], *to[i], s);
    if (!rc) rc = lists_build_two(p->tree, tt, mac_theta, t->lists, s);
    if (!rc) {
        t->buf.p = p->fmm.p;
        t->buf.nc = p->fmm.nc;
        t->buf.nc_pad = p->fmm.nc_pad;
        const size_t esz = (tt.dtype == EDFMM_F64 ? 16 : 8) * (size_t)t->buf.nc_pad *
                           (size_t)std::max<int64_t>(tt.n_nodes, 1);
        rc = t->buf.locals.reserve(esz);
        if (!rc) {
            cudaError_t e = cudaMemsetAsync(t->buf.locals.p, 0, esz, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("target set-up: ") + cudaGetErrorString(e));
        }
    }
    if (rc) return rc;
    *out = t.release();
    return EDFMM_OK;
}

int edfmm_targets_stage(edfmm_targets *t, int stage, void *out_dev, void *stream) {
    if (!t) return fail(EDFMM_ERR_ARG, "targets is NULL");
    edfmm_plan *p = t->plan;
    if (int rc = check_plan(p)) return rc;
    if (t->buf.p != p->fmm.p)
        return fail(EDFMM_ERR_STATE, "the source plan's expansion order changed after the targets were created");
    cudaStream_t s = S(stream);
    const int64_t M = t->tree.n_nodes;
    switch (stage) {
    case EDFMM_TARGETS_M2L:
        return run_m2l_two(t->tree, p->tree, t->lists, p->fmm, t->buf, s);
    case EDFMM_TARGETS_L2L:
        return run_l2l(t->tree, t->buf, s);
    case EDFMM_TARGETS_L2P:
    case EDFMM_TARGETS_P2P: {
        if (t->tree.n_points == 0) return EDFMM_OK;
        if (!out_dev) return fail(EDFMM_ERR_ARG, "output is NULL");
        NearArgs a;
        a.out = out_dev;
        a.near = stage == EDFMM_TARGETS_P2P;
        a.far = stage == EDFMM_TARGETS_L2P;
        a.src_tree = &p->tree;
        return run_p2p_l2p(t->tree, t->lists, t->buf, a, s);
    }
    case EDFMM_TARGETS_LOCALS: {
        if (M == 0) return EDFMM_OK;
        if (!out_dev) return fail(EDFMM_ERR_ARG, "output is NULL");
        const int nc = t->buf.nc;
        if (t->tree.dtype == EDFMM_F64)
            k_export_coeffs<double><<<nblk(M * nc, 256), 256, 0, s>>>(M, nc, t->buf.nc_pad,
                                                                      dptr<Cplx<double>>(t->buf.locals),
                                                                      static_cast<Cplx<double> *>(out_dev));
        else
            k_export_coeffs<float><<<nblk(M * nc, 256), 256, 0, s>>>(M, nc, t->buf.nc_pad,
                                                                     dptr<Cplx<float>>(t->buf.locals),
                                                                     static_cast<Cplx<float> *>(out_dev));
        EDFMM_LAUNCH_CHECK("k_export_coeffs");
        return EDFMM_OK;
    }
    default:
        return fail(EDFMM_ERR_ARG, "unknown targets stage");
    }
}

int edfmm_targets_destroy(edfmm_targets *t) {
    delete t;
    return EDFMM_OK;
}

int edfmm_targets_info(const edfmm_targets *t, int64_t *n_nodes, int64_t *n_p2p_pairs, int64_t *n_m2l_pairs,
                       int64_t *p2p_interactions) {
    if (!t) return fail(EDFMM_ERR_ARG, "targets is NULL");
    if (n_nodes) *n_nodes = t->tree.n_nodes;
    if (n_p2p_pairs) *n_p2p_pairs = t->lists.n_p2p;
    if (n_m2l_pairs) *n_m2l_pairs = t->lists.n_m2l;
    if (p2p_interactions) *p2p_interactions = t->lists.p2p_interactions;
    return EDFMM_OK;
}

int edfmm_targets_export_lists(const edfmm_targets *t, int64_t *p2p_pairs, int64_t *m2l_pairs, void *stream) {
    if (!t) return fail(EDFMM_ERR_ARG, "targets is NULL");
    const int64_t M = t->tree.n_nodes;
    if (M == 0) return EDFMM_OK;
    dim3 blk(32, 8);
    if (p2p_pairs && t->lists.n_p2p > 0) {
        k_export_pairs<<<nblk(M, 8), blk, 0, S(stream)>>>(M, dptr<int32_t>(t->lists.p2p_off),
                                                           dptr<int32_t>(t->lists.p2p_src), p2p_pairs);
        EDFMM_LAUNCH_CHECK("k_export_pairs");
    }
    if (m2l_pairs && t->lists.n_m2l > 0) {
        k_export_pairs<<<nblk(M, 8), blk, 0, S(stream)>>>(M, dptr<int32_t>(t->lists.m2l_off),
                                                           dptr<int32_t>(t->lists.m2l_src), m2l_pairs);
        EDFMM_LAUNCH_CHECK("k_export_pairs");
    }
    return EDFMM_OK;
}

int edfmm_targets_potential(edfmm_targets *t, const void *sigma, const void *areas, double k_e, void *out, int flags,
                            void *stream) {
    if (!t) return fail(EDFMM_ERR_ARG, "targets is NULL");
    edfmm_plan *p = t->plan;
    if (int rc = check_plan(p)) return rc;
    if (t->tree.n_points == 0) return EDFMM_OK;
    if (!sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "sigma, areas and out must be non-NULL");
    cudaStream_t s = S(stream);
    const bool far = (flags & EDFMM_NO_FARFIELD) == 0;
    const bool near = (flags & EDFMM_NO_NEARFIELD) == 0;
    int rc;
    if ((rc = set_charges(p->tree, sigma, areas, s))) return rc;
    if (far) {
        if ((rc = run_p2m(p->tree, p->fmm, s)) || (rc = run_m2m(p->tree, p->fmm, s)) ||
            (rc = run_m2l_two(t->tree, p->tree, t->lists, p->fmm, t->buf, s)) || (rc = run_l2l(t->tree, t->buf, s)))
            return rc;
    }
    NearArgs a;
    a.k_e = k_e;
    a.out = out;
    a.scatter = true;
    a.near = near;
    a.far = far;
    a.src_tree = &p->tree;
    return run_p2p_l2p(t->tree, t->lists, t->buf, a, s);
}

int edfmm_targets_field(edfmm_targets *t, const void *sigma, const void *areas, double k_e, void *out, int flags,
                        void *stream) {
    if (!t) return fail(EDFMM_ERR_ARG, "targets is NULL");
    edfmm_plan *p = t->plan;
    if (int rc = check_plan(p)) return rc;
    if (t->tree.n_points == 0) return EDFMM_OK;
    if (!sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "sigma, areas and out must be non-NULL");
    cudaStream_t s = S(stream);
    const bool far = (flags & EDFMM_NO_FARFIELD) == 0;
    const bool near = (flags & EDFMM_NO_NEARFIELD) == 0;
    int rc;
    if ((rc = set_charges(p->tree, sigma, areas, s))) return rc;
    if (far) {
        if ((rc = run_p2m(p->tree, p->fmm, s)) || (rc = run_m2m(p->tree, p->fmm, s)) ||
            (rc = run_m2l_two(t->tree, p->tree, t->lists, p->fmm, t->buf, s)) || (rc = run_l2l(t->tree, t->buf, s)))
            return rc;
    }
    return run_targets_field(t->tree, t->lists, t->buf, p->tree, k_e, near, far, out, s);
}

}  // extern "C"
