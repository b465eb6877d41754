// Batched plans: many independent point sets (BEM instances) in one plan.
//
// Each instance gets its own octree and interaction lists, built exactly as
// a single plan builds them (so each is the reference's tree and lists for
// that instance alone).  They are then packed into one DevTree / DevLists
// with node, point and edge offsets.  No list entry crosses an instance, so
// every FMM stage (P2M over all leaves, M2M / L2L level by level across all
// instances, M2L and P2P over all rows) runs as one launch over the whole
// batch.  The operator is block diagonal: one matvec applies every
// instance's operator to its own slice of sigma.
#include <algorithm>

#include "edfmm_internal.cuh"

namespace edfmm {
namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

__global__ void k_add_i32(const int32_t *__restrict__ src, int64_t n, int32_t add, int keep_negative,
                          int32_t *__restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t v = src[i];
    dst[i] = (keep_negative && v < 0) ? v : v + add;
}

__global__ void k_add_int2(const int2 *__restrict__ src, int64_t n, int32_t add, int2 *__restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 v = src[i];
    dst[i] = make_int2(v.x + add, v.y + add);
}

int add_i32(const DevBuf &src, int64_t n, int32_t add, bool keep_negative, int32_t *dst, cudaStream_t s) {
    if (n <= 0) return EDFMM_OK;
    k_add_i32<<<nblk(n, 256), 256, 0, s>>>(dptr<int32_t>(src), n, add, keep_negative ? 1 : 0, dst);
    EDFMM_LAUNCH_CHECK("k_add_i32");
    return EDFMM_OK;
}

int copy_bytes(void *dst, const DevBuf &src, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return EDFMM_OK;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(dst, src.p, bytes, cudaMemcpyDeviceToDevice, s));
    return EDFMM_OK;
}

}  // namespace

int pack_batch(std::vector<DevTree> &trees, std::vector<DevLists> &lists, int dtype, DevTree &T, DevLists &Lout,
               cudaStream_t s) {
    const size_t t4 = dtype == EDFMM_F64 ? sizeof(double4) : sizeof(float4);
    const int K = (int)trees.size();
    std::vector<int64_t> P(K + 1, 0), N(K + 1, 0), Lf(K + 1, 0), E2(K + 1, 0), EM(K + 1, 0);
    int max_level = 0;
    for (int i = 0; i < K; ++i) {
        P[i + 1] = P[i] + trees[i].n_points;
        N[i + 1] = N[i] + trees[i].n_nodes;
        Lf[i + 1] = Lf[i] + trees[i].n_leaves;
        E2[i + 1] = E2[i] + lists[i].n_p2p;
        EM[i + 1] = EM[i] + lists[i].n_m2l;
        max_level = std::max(max_level, trees[i].max_level);
    }
    if (N[K] >= (int64_t)1 << 31 || P[K] >= (int64_t)1 << 31 || E2[K] >= (int64_t)1 << 31 || EM[K] >= (int64_t)1 << 31)
        return fail(EDFMM_ERR_UNSUPPORTED, "batched plan exceeds 32-bit node, point or list indices");
    T.dtype = dtype;
    T.n_points = P[K];
    T.n_nodes = N[K];
    T.n_inst = K;
    T.n_leaves = Lf[K];
    T.max_level = max_level;
    T.depth_warnings = 0;
    const int64_t M = T.n_nodes, n = T.n_points;
    int rc;
    if ((rc = T.pts.reserve(t4 * std::max<int64_t>(n, 1))) || (rc = T.index_map.reserve(4 * std::max<int64_t>(n, 1))) ||
        (rc = T.center.reserve(t4 * M)) || (rc = T.half.reserve(t4 * M)) || (rc = T.range.reserve(sizeof(int2) * M)) ||
        (rc = T.parent.reserve(4 * M)) || (rc = T.children.reserve(32 * M)) || (rc = T.level.reserve(4 * M)) ||
        (rc = T.is_leaf.reserve(M)) || (rc = T.leaves.reserve(4 * std::max<int64_t>(T.n_leaves, 1))) ||
        (rc = T.level_nodes.reserve(4 * M)))
        return rc;
    {
        std::vector<int32_t> no(N.begin(), N.end());
        if ((rc = T.inst_node_off.reserve(sizeof(int32_t) * (K + 1)))) return rc;
        EDFMM_CUDA_TRY(cudaMemcpyAsync(T.inst_node_off.p, no.data(), sizeof(int32_t) * (K + 1), cudaMemcpyHostToDevice, s));
        EDFMM_CUDA_TRY(cudaStreamSynchronize(s));  // the host vector goes out of scope
    }
    for (int i = 0; i < K; ++i) {
        DevTree &t = trees[i];
        T.depth_warnings += t.depth_warnings;
        const int64_t m = t.n_nodes, np = t.n_points;
        char *pts = static_cast<char *>(T.pts.p) + t4 * P[i];
        if ((rc = copy_bytes(pts, t.pts, t4 * np, s))) return rc;
        if ((rc = add_i32(t.index_map, np, (int32_t)P[i], false, dptr<int32_t>(T.index_map) + P[i], s))) return rc;
        if ((rc = copy_bytes(static_cast<char *>(T.center.p) + t4 * N[i], t.center, t4 * m, s))) return rc;
        if ((rc = copy_bytes(static_cast<char *>(T.half.p) + t4 * N[i], t.half, t4 * m, s))) return rc;
        if (m > 0) {
            k_add_int2<<<nblk(m, 256), 256, 0, s>>>(dptr<int2>(t.range), m, (int32_t)P[i], dptr<int2>(T.range) + N[i]);
            EDFMM_LAUNCH_CHECK("k_add_int2");
        }
        if ((rc = add_i32(t.parent, m, (int32_t)N[i], true, dptr<int32_t>(T.parent) + N[i], s))) return rc;
        if ((rc = add_i32(t.children, 8 * m, (int32_t)N[i], true, dptr<int32_t>(T.children) + 8 * N[i], s))) return rc;
        if ((rc = copy_bytes(dptr<int32_t>(T.level) + N[i], t.level, 4 * m, s))) return rc;
        if ((rc = copy_bytes(dptr<uint8_t>(T.is_leaf) + N[i], t.is_leaf, m, s))) return rc;
        if ((rc = add_i32(t.leaves, t.n_leaves, (int32_t)N[i], false, dptr<int32_t>(T.leaves) + Lf[i], s))) return rc;
    }
    // nodes grouped by level across the batch
    T.level_offsets.assign(max_level + 2, 0);
    int64_t at = 0;
    for (int l = 0; l <= max_level; ++l) {
        T.level_offsets[l] = (int32_t)at;
        for (int i = 0; i < K; ++i) {
            DevTree &t = trees[i];
            if (l + 1 >= (int)t.level_offsets.size()) continue;
            const int a = t.level_offsets[l], b = t.level_offsets[l + 1];
            if (b <= a) continue;
            k_add_i32<<<nblk(b - a, 256), 256, 0, s>>>(dptr<int32_t>(t.level_nodes) + a, b - a, (int32_t)N[i], 0,
                                                        dptr<int32_t>(T.level_nodes) + at);
            EDFMM_LAUNCH_CHECK("k_add_i32");
            at += b - a;
        }
    }
    T.level_offsets[max_level + 1] = (int32_t)at;
    if (at != M) return fail(EDFMM_ERR_STATE, "batched plan: level lists do not cover every node");
    // interaction lists: CSR rows by target node, offsets shifted by the edges before
    Lout = DevLists();
    Lout.n_p2p = E2[K];
    Lout.n_m2l = EM[K];
    if ((rc = Lout.p2p_off.reserve(4 * (M + 1))) || (rc = Lout.m2l_off.reserve(4 * (M + 1))) ||
        (rc = Lout.p2p_src.reserve(4 * std::max<int64_t>(E2[K], 1))) ||
        (rc = Lout.m2l_src.reserve(4 * std::max<int64_t>(EM[K], 1))))
        return rc;
    for (int i = 0; i < K; ++i) {
        DevLists &li = lists[i];
        const int64_t m = trees[i].n_nodes;
        Lout.p2p_interactions += li.p2p_interactions;
        Lout.max_p2p_row = std::max(Lout.max_p2p_row, li.max_p2p_row);
        Lout.max_m2l_row = std::max(Lout.max_m2l_row, li.max_m2l_row);
        if ((rc = add_i32(li.p2p_off, m, (int32_t)E2[i], false, dptr<int32_t>(Lout.p2p_off) + N[i], s))) return rc;
        if ((rc = add_i32(li.m2l_off, m, (int32_t)EM[i], false, dptr<int32_t>(Lout.m2l_off) + N[i], s))) return rc;
        if ((rc = add_i32(li.p2p_src, li.n_p2p, (int32_t)N[i], false, dptr<int32_t>(Lout.p2p_src) + E2[i], s))) return rc;
        if ((rc = add_i32(li.m2l_src, li.n_m2l, (int32_t)N[i], false, dptr<int32_t>(Lout.m2l_src) + EM[i], s))) return rc;
    }
    const int32_t e2 = (int32_t)E2[K], em = (int32_t)EM[K];
    EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<int32_t>(Lout.p2p_off) + M, &e2, 4, cudaMemcpyHostToDevice, s));
    EDFMM_CUDA_TRY(cudaMemcpyAsync(dptr<int32_t>(Lout.m2l_off) + M, &em, 4, cudaMemcpyHostToDevice, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));  // the host values above must outlive the copies
    return EDFMM_OK;
}

}  // namespace edfmm
