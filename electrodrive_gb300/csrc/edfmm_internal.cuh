// Internal declarations shared by the libedfmm translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/edfmm.h"

namespace edfmm {

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
void count_launch(int n = 1);

#define EDFMM_CUDA_TRY(expr)                                                                  \
    do {                                                                                      \
        cudaError_t _e = (expr);                                                              \
        if (_e != cudaSuccess)                                                                \
            return ::edfmm::fail(EDFMM_ERR_CUDA, std::string(#expr " failed: ") +             \
                                                     cudaGetErrorString(_e));                 \
    } while (0)

#define EDFMM_LAUNCH_CHECK(name)                                                              \
    do {                                                                                      \
        ::edfmm::count_launch();                                                              \
        cudaError_t _e = cudaGetLastError();                                                  \
        if (_e != cudaSuccess)                                                                \
            return ::edfmm::fail(EDFMM_ERR_CUDA, std::string("launch of " name " failed: ") + \
                                                     cudaGetErrorString(_e));                 \
    } while (0)

// ---------------------------------------------------------------------------
// device buffer (owning)
// ---------------------------------------------------------------------------
// Blocks released while a BlockCacheScope is active on this thread are kept
// for the scope's later reserves instead of being freed: a build that runs on
// ONE stream then reuses its temporaries in stream order without a
// cudaMalloc / cudaFree (which synchronises the device) per temporary.  The
// scope frees what it still holds when it ends.
struct BlockCache;
BlockCache *block_cache();  // this thread's active cache or NULL
void *block_cache_take(BlockCache *c, size_t nbytes, size_t *got);
void block_cache_put(BlockCache *c, void *p, size_t nbytes);
// frees every block the cache holds (cudaFree waits for the device)
void block_cache_trim(BlockCache *c);
// cudaMalloc that, when it fails inside a cache scope, frees the cached
// blocks and tries once more (a held block may be what the device lacks)
cudaError_t malloc_or_trim(void **p, size_t nbytes);
struct BlockCacheScope {
    BlockCacheScope();
    ~BlockCacheScope();
    BlockCacheScope(const BlockCacheScope &) = delete;
    BlockCacheScope &operator=(const BlockCacheScope &) = delete;
    BlockCache *prev;
    BlockCache *cache;
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;  // size of the block held
    size_t used = 0;   // size last asked for (a cached block may be larger)
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes), used(o.used) {
        o.p = nullptr;
        o.bytes = 0;
        o.used = 0;
    }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            bytes = o.bytes;
            used = o.used;
            o.p = nullptr;
            o.bytes = 0;
            o.used = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            if (BlockCache *c = block_cache()) block_cache_put(c, p, bytes);
            else cudaFree(p);
        }
        p = nullptr;
        bytes = 0;
        used = 0;
    }
    // grows (never shrinks); contents are not preserved
    int reserve(size_t nbytes) {
        if (nbytes <= bytes && p) {
            used = nbytes;
            return EDFMM_OK;
        }
        release();
        size_t want = nbytes ? nbytes : 16;
        if (BlockCache *c = block_cache()) {
            size_t got = 0;
            if (void *q = block_cache_take(c, want, &got)) {
                p = q;
                bytes = got;
                used = want;
                return EDFMM_OK;
            }
        }
        cudaError_t e = malloc_or_trim(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(EDFMM_ERR_ALLOC, std::string("cudaMalloc of ") + std::to_string(want) +
                                             " bytes failed: " + cudaGetErrorString(e));
        }
        bytes = want;
        used = want;
        return EDFMM_OK;
    }
    // A buffer that outlives its build (a plan's tree, lists, expansions)
    // and received a cached block well above its size moves to a block of
    // its own size (contents copied in stream order), so the plan holds no
    // slack for its lifetime.
    int shrink_to_fit(cudaStream_t s) {
        if (!p || bytes <= used + used / 8 + 4096) return EDFMM_OK;
        void *q = nullptr;
        cudaError_t e = malloc_or_trim(&q, used);
        if (e == cudaSuccess) e = cudaMemcpyAsync(q, p, used, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) {
            if (q) cudaFree(q);
            return fail(EDFMM_ERR_ALLOC, std::string("exact-size copy of a plan buffer failed: ") +
                                             cudaGetErrorString(e));
        }
        const size_t keep = used;
        release();  // the cache frees it only after the device is done with it
        p = q;
        bytes = keep;
        used = keep;
        return EDFMM_OK;
    }
    template <class U> U *as() const { return static_cast<U *>(p); }
};

// typed view of a buffer (a free function, so no `template` keyword is needed
// inside templates)
template <class U> inline U *dptr(const DevBuf &b) { return static_cast<U *>(b.p); }

// ---------------------------------------------------------------------------
// primitives (scan.cu)
// ---------------------------------------------------------------------------
// Exclusive prefix sum of n int32 counts into int32 offsets; the grand total
// is written to *total_dev (int64) if non-null.  tmp must hold scan_tmp_bytes(n).
size_t scan_tmp_bytes(int64_t n);
int scan_exclusive(const int32_t *in, int32_t *out, int64_t n, int64_t *total_dev, void *tmp,
                   cudaStream_t s);

// Sort every CSR row of `vals` ascending (rows given by offsets[0..rows]).
// tmp must hold sort_rows_tmp_bytes(...) for the longest rows.
int sort_csr_rows(const int32_t *offsets, int32_t *vals, int64_t rows, int64_t max_row_len,
                  cudaStream_t s);

// ---------------------------------------------------------------------------
// tree + lists (tree.cu, lists.cu)
// ---------------------------------------------------------------------------
template <typename T> struct Vec4 {};
template <> struct Vec4<float> {
    using type = float4;
};
template <> struct Vec4<double> {
    using type = double4;
};

#ifdef __CUDACC__
// 1/sqrt(x) for a normal x > 0 (PTX rsqrt.approx.ftz.f32, relative error
// below 2^-22.9).  Callers clamp the argument well above the subnormal range,
// so flushing subnormals changes nothing and no range handling is needed.
__device__ __forceinline__ float rsqrt_normal(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
#endif

// Device-resident tree in DFS pre-order (the reference's node numbering).
struct DevTree {
    int dtype = EDFMM_F32;
    int64_t n_points = 0;
    int64_t n_nodes = 0;
    int64_t n_leaves = 0;
    int max_level = 0;
    int depth_warnings = 0;
    DevBuf pts;        // T4 per point, tree order: (x, y, z, charge)
    DevBuf index_map;  // int32, tree position -> original index
    DevBuf center;     // T4 per node: (cx, cy, cz, radius)
    DevBuf half;       // T4 per node: (hx, hy, hz, expansion scale a)
    DevBuf range;      // int2 per node: [start, end)
    DevBuf parent;     // int32
    DevBuf children;   // int32 x 8
    DevBuf level;      // int32
    DevBuf is_leaf;    // uint8
    DevBuf leaves;     // int32 ids of leaf nodes (ascending)
    std::vector<int32_t> level_offsets;  // host: level l nodes = level_nodes[off[l], off[l+1])
    DevBuf level_nodes;                  // int32 node ids grouped by level
    // FP64 trees in two-float mode: per point (x, y, z, charge) split into
    // FP32 (hi, lo) pairs, 8 floats, refreshed with the charges; per node
    // (cx, cy, cz, expansion scale a) split the same way
    DevBuf pts_tf;
    DevBuf nodes_tf;
    // batched plans: instance k owns nodes inst_node_off[k] .. inst_node_off[k+1]-1
    int n_inst = 0;
    DevBuf inst_node_off;  // int32 x (n_inst + 1)
};

// Per-instance activity of a batched plan's matvec: instance k is active
// when flags[k * stride] != 0 (a column of the batched GMRES state).  M2L
// rows and near-field leaves of inactive instances are skipped; their
// outputs are left unspecified (the batched solver does not read them).
struct InstMask {
    const int32_t *node_off = nullptr;  // NULL: no mask
    int n_inst = 0;
    const double *flags = nullptr;
    int stride = 0;
};
#ifdef __CUDACC__
__device__ __forceinline__ bool inst_active(const InstMask &m, int node) {
    if (!m.node_off) return true;
    int lo = 0, hi = m.n_inst - 1;  // last instance whose first node <= node
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (m.node_off[mid] <= node) lo = mid; else hi = mid - 1;
    }
    return m.flags[(int64_t)lo * m.stride] != 0.0;
}
#endif

int tree_build(const void *points_dev, int64_t n, int dtype, int leaf_size, int max_depth,
               DevTree &tree, cudaStream_t s);
// One tree per instance (rows inst_off[k] .. inst_off[k+1]-1, host offsets),
// built together level by level as one forest: nodes of instance k are the
// DFS range [inst_node_off[k], inst_node_off[k+1]), each tree equal to
// tree_build of its rows alone; nodes grouped by level across instances.
int tree_build_forest(const void *points_dev, const int64_t *inst_off, int n_inst, int dtype, int leaf_size,
                      int max_depth, DevTree &tree, cudaStream_t s);

struct DevLists {
    int64_t n_p2p = 0, n_m2l = 0;
    int64_t p2p_interactions = 0;
    int64_t max_p2p_row = 0, max_m2l_row = 0;
    DevBuf p2p_off, p2p_src;  // CSR by target, sources ascending
    DevBuf m2l_off, m2l_src;
    // the target tree's leaves in decreasing near-field work (sum over the
    // leaf's P2P sources of n_source * n_target): the near-field kernel takes
    // them in this order, so that its last wave holds the short leaves
    DevBuf p2p_leaves;
    // the target tree's nodes by decreasing M2L pair count: the M2L kernels
    // give warp w row m2l_rows[w], so that a block's warps (which run their
    // rounds of pairs together) hold rows of similar length
    DevBuf m2l_rows;
    // transposed M2L CSR (rows = listed sources), built on demand for the
    // reference's swapped pair order
    bool have_m2l_swapped = false;
    DevBuf m2l_swapped_off, m2l_swapped_src;
};

int lists_build(const DevTree &tree, double theta, DevLists &lists, cudaStream_t s);
int lists_build_swapped(const DevTree &tree, DevLists &lists, cudaStream_t s);
// lists between two trees: rows = target-tree nodes, sources = source-tree nodes
// (the reference's build_interaction_lists(source_tree, target_tree))
int lists_build_two(const DevTree &src_tree, const DevTree &tgt_tree, double theta, DevLists &lists, cudaStream_t s);

// ---------------------------------------------------------------------------
// FMM stages (farfield.cu, nearfield.cu)
// ---------------------------------------------------------------------------
inline int num_coeffs(int p) { return (p + 1) * (p + 2) / 2; }

// M2L pairs whose source radius exceeds 256x the target radius, as CSR rows
// by target (FP32 plans only; empty for uniform trees).
struct ExtremeRows {
    bool built = false;
    int64_t n_pairs = 0, n_rows = 0;
    DevBuf off, src, rows;
};

struct FmmBuffers {
    int p = 8;
    int nc = 45;
    int nc_pad = 46;  // per-node stride in complex numbers (even: 16-byte rows for float)
    DevBuf multipoles;  // complex T, n_nodes x nc_pad
    DevBuf locals;      // complex T, n_nodes x nc_pad
    DevBuf translated;  // complex T, n_nodes x nc_pad: each node's multipole moved to its parent's centre
    ExtremeRows extreme, extreme_swapped;
    InstMask mask;  // set around the steps of a batched solve
    // FP64 plans: EDFMM_ARITH_TWO_FLOAT runs M2L and the near field in
    // two-float arithmetic on the FP32 pipe (twofloat.cuh); mult_tf holds
    // the multipoles split into (hi, lo) pairs for the two-float M2L
    int arith = EDFMM_ARITH_NATIVE;
    DevBuf mult_tf;
    // launch shapes the autotuner may change (edfmm_plan_set_launch)
    int m2l_tf_block = 128;  // two-float M2L threads per block (128 or 256, p = 8)
    int near_overlap = 1;    // full matvec: near field on a second stream beside the far field
    int m2l_packed = 1;      // two-float M2L: matrices on packed FP32x2 instructions
};

int set_charges(const DevTree &tree, const void *sigma, const void *areas, cudaStream_t s);
int run_p2m(const DevTree &tree, FmmBuffers &buf, cudaStream_t s);
int run_m2m(const DevTree &tree, FmmBuffers &buf, cudaStream_t s);
int run_m2l(const DevTree &tree, const DevLists &lists, FmmBuffers &buf, bool swapped, cudaStream_t s);
// rotation-based M2L (m2l_rot.cu, kernels in m2l_rot.cuh), orders 1..8, FP32 and FP64
int launch_m2l_rot(int dtype, int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows,
                   const void *tcen,
                   const void *thal, const void *cen, const void *hal, const void *Mx, void *Lx, int nc_pad,
                   const InstMask &mask, cudaStream_t s);
// the same in two-float arithmetic for FP64 plans, orders 6..8
// (EDFMM_ERR_UNSUPPORTED for other orders, launching nothing): node geometry
// and multipoles split into (hi, lo) FP32 pairs (tnodes / snodes: 2 float4
// per node; Mx: one float4 per complex coefficient), locals written as FP64
int launch_m2l_rot_tf(int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows,
                      const void *tnodes, const void *thal,
                      const void *snodes, const void *hal, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                      int block, bool packed, cudaStream_t s);
int run_m2l_two(const DevTree &tgt_tree, const DevTree &src_tree, const DevLists &lists, const FmmBuffers &src_buf,
                FmmBuffers &tgt_buf, cudaStream_t s);
int run_l2l(const DevTree &tree, FmmBuffers &buf, cudaStream_t s);
// the same-tree extreme-pair rows of buf (built once; synchronises s)
int prepare_extreme_rows(const DevTree &tree, const DevLists &lists, FmmBuffers &buf, cudaStream_t s);
// two-float mode of an FP64 plan: split node geometry and the multipole
// buffer (sized for the current order); called when the mode is set and
// when the order changes
int prepare_two_float(DevTree &tree, FmmBuffers &buf, cudaStream_t s);

struct NearArgs {
    const void *sigma = nullptr;      // original order (nullable)
    const void *areas = nullptr;      // original order (nullable)
    const void *self_int = nullptr;   // original order (nullable)
    double k_e = 1.0;
    void *out = nullptr;              // original order if scatter, else tree order
    bool scatter = false;             // write out[index_map[i]] with k_e, self term, clamp
    bool near = true;                 // include P2P
    bool far = true;                  // include L2P
    const void *add_in = nullptr;     // tree-order sums added before the epilogue (nullable)
    // sources of the P2P when they are another tree's points (targets
    // evaluated against a source plan): no self exclusion then
    const struct DevTree *src_tree = nullptr;
};
// field at the points of a target tree (evaluation from a source plan)
int run_targets_field(const DevTree &tree, const DevLists &lists, const FmmBuffers &buf, const DevTree &stree,
                      double k_e, bool near, bool far, void *out, cudaStream_t s);
int run_p2p_l2p(const DevTree &tree, const DevLists &lists, const FmmBuffers &buf,
                const NearArgs &args, cudaStream_t s);
int upload_tables();

}  // namespace edfmm

struct edfmm_plan {
    edfmm::DevTree tree;
    edfmm::DevLists lists;
    edfmm::FmmBuffers fmm;
    double mac_theta = 0.5;
    int leaf_size = 64;
    int max_depth = 32;
    int device = 0;
    // matvec: the near field runs on a second stream beside the far-field
    // chain (fork / join events) into tree-order sums, created on first use
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    edfmm::DevBuf near_sum;
    edfmm_plan() = default;
    edfmm_plan(const edfmm_plan &) = delete;
    edfmm_plan &operator=(const edfmm_plan &) = delete;
    ~edfmm_plan() {
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
    }
};
