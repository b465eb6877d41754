/*
 * edfmm.h -- C ABI of the GB300-native FMM-accelerated Laplace single-layer
 * BEM operator (libedfmm.so).
 *
 * Conventions
 *   - Every pointer argument named *_dev is a device pointer on the current
 *     CUDA device; host pointers are named *_host.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *     All work is stream-ordered; functions that must size device buffers from
 *     device results (plan creation) synchronise `stream` internally.
 *   - `dtype` is EDFMM_F32 or EDFMM_F64 and applies to every floating-point
 *     array of the call.
 *   - Return value: EDFMM_OK (0), a negative code for argument / CUDA /
 *     allocation errors, or a positive code for a numerical condition.
 *     edfmm_last_error() returns a human-readable message for the calling
 *     thread's most recent failure.
 *
 * Each entry point cites the reference interface it replaces (paths inside
 * the reference project).
 */
#ifndef EDFMM_H
#define EDFMM_H

#include <stdint.h>

#if defined(__GNUC__)
#define EDFMM_API __attribute__((visibility("default")))
#else
#define EDFMM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define EDFMM_OK 0
#define EDFMM_ERR_ARG (-1)
#define EDFMM_ERR_CUDA (-2)
#define EDFMM_ERR_ALLOC (-3)
#define EDFMM_ERR_UNSUPPORTED (-4)
#define EDFMM_ERR_STATE (-5)

#define EDFMM_F32 0
#define EDFMM_F64 1

/* matvec flags */
#define EDFMM_REFERENCE_PAIR_ORDER 1 /* apply listed (src, tgt) M2L pairs as L[src] += T M[tgt],
                                        the reference's unpacking (multipole_operators.py:1671) */
#define EDFMM_NO_FARFIELD 2          /* near field only (P2P) */
#define EDFMM_NO_NEARFIELD 4         /* far field only (P2M..L2P) */

/* arithmetic of an FP64 plan's M2L and near field (edfmm_plan_set_arithmetic) */
#define EDFMM_ARITH_NATIVE 0         /* IEEE FP64 */
#define EDFMM_ARITH_TWO_FLOAT 1      /* two-float (hi + lo FP32 pairs, about 48 bits) on the FP32 pipe */

typedef struct edfmm_plan edfmm_plan;

typedef struct {
    int64_t n_points;
    int64_t n_nodes;
    int64_t n_leaves;
    int64_t n_p2p_pairs;
    int64_t n_m2l_pairs;
    int64_t p2p_interactions;  /* sum over P2P pairs of n_src * n_tgt */
    int32_t max_level;
    int32_t depth_warnings;    /* leaves cut by max_depth above leaf_size (tree.py:899-908) */
    int32_t dtype;
    int32_t expansion_order;
    int32_t leaf_size;
    int32_t max_depth;
    double mac_theta;
} edfmm_plan_info;

/*
 * Self-check of the library's build-time block cache (no counterpart in the
 * reference): inside one cache scope it reserves and releases two blocks,
 * reserves a block larger than any cached one, a block that reuses a cached
 * one, and shrinks a buffer that received an oversized cached block to its
 * exact size.  results_host[0..3] are set to 1 for each step that behaved.
 * Allocates about 22 MiB of device memory for the duration of the call.
 */
EDFMM_API int edfmm_block_cache_selfcheck(int64_t *results_host);

/* Thread-local description of the most recent failure. */
EDFMM_API const char *edfmm_last_error(void);

/* Library version string. */
EDFMM_API const char *edfmm_version(void);

/*
 * Build the adaptive octree and the dual-tree interaction lists on the GPU
 * and allocate every buffer a matvec needs.  Replaces the geometry set-up of
 * LaplaceFmm3D.__init__ (electrodrive/fmm3d/bem_fmm.py:127-302), i.e.
 * build_fmm_tree (electrodrive/fmm3d/tree.py:968-1050) followed by
 * build_interaction_lists (electrodrive/fmm3d/interaction_lists.py:531-577).
 * points_dev: (n, 3) row-major in `dtype`.  Tree and lists are bit-identical
 * to the reference's for the same inputs.
 */
EDFMM_API int edfmm_plan_create(const void *points_dev, int64_t n, int dtype, int leaf_size, int max_depth,
                      double mac_theta, int expansion_order, void *stream, edfmm_plan **plan_out);

/*
 * Batched plan (no counterpart in the reference, which solves one geometry at
 * a time): points_dev holds n_instances independent point sets back to back,
 * instance k at rows [offsets[k], offsets[k+1]) (offsets: host array of
 * n_instances + 1 values, offsets[0] = 0, every instance non-empty).  Each
 * instance gets the tree and lists edfmm_plan_create would build for it
 * alone, built for all instances together level by level (one forest, one
 * set of launches per tree level and per list front); the plan's matvec is
 * the block-diagonal operator (no interaction between instances), one launch
 * per stage for the whole batch.
 */
EDFMM_API int edfmm_plan_create_batch(const void *points_dev, const int64_t *offsets, int n_instances, int dtype,
                                      int leaf_size, int max_depth, double mac_theta, int expansion_order,
                                      void *stream, edfmm_plan **plan_out);
/*
 * A plan in another dtype and expansion order over the same partition: the
 * source plan's tree, lists and instance layout are copied and its point and
 * node geometry cast to `dtype` (no new tree or list build).  The source plan
 * is not modified; charges are set on the new plan as on any other.
 */
EDFMM_API int edfmm_plan_convert(const edfmm_plan *plan, int dtype, int expansion_order, void *stream,
                                 edfmm_plan **plan_out);
EDFMM_API int edfmm_plan_destroy(edfmm_plan *plan);

/*
 * Rebuild the interaction lists of an existing plan for another MAC
 * parameter (build_interaction_lists(tree, tree, mac_theta=...),
 * electrodrive/fmm3d/interaction_lists.py:531-577).
 */
EDFMM_API int edfmm_plan_rebuild_lists(edfmm_plan *plan, double mac_theta, void *stream);

/*
 * Arithmetic of an FP64 plan's M2L (orders 6..8) and near field (no
 * counterpart in the reference, whose FP64 path is IEEE FP64 throughout):
 * EDFMM_ARITH_TWO_FLOAT evaluates them on the FP32 pipe in two-float
 * arithmetic (each value an unevaluated sum of two floats, about 48
 * significant bits; within about 1e-13 of the FP64 result, far inside the
 * expansion's truncation error), which on this GPU runs several times faster
 * than FP64; the expansions, P2M, M2M, L2L and every input and output stay
 * FP64.  EDFMM_ARITH_NATIVE (the default) restores IEEE FP64.  Two-float mode
 * keeps a split copy of the points (32 bytes per point) and synchronises
 * `stream` once while it prepares.  FP32 plans accept only EDFMM_ARITH_NATIVE.
 */
EDFMM_API int edfmm_plan_set_arithmetic(edfmm_plan *plan, int mode, void *stream);

/*
 * Launch shapes of a plan's matvec that the autotuner chooses by timing (no
 * counterpart in the reference): EDFMM_LAUNCH_M2L_TF_BLOCK, threads per block
 * of the two-float M2L at p = 8 (128: two blocks per SM; 256: one block of
 * eight warps per SM, one instruction stream for the long pair code);
 * EDFMM_LAUNCH_NEAR_OVERLAP, 1 to run the near field on a second stream beside
 * the far-field chain, 0 for one fused pass after it.  Results are the same
 * either way (bit for bit).  EDFMM_LAUNCH_M2L_PACKED (FP64 plans in two-float
 * mode), 1 (the default) to run the two-float M2L's rotation matrices on
 * packed FP32x2 instructions, two matrix rows per instruction, 0 for the
 * scalar form; the results are the same bit for bit.
 */
#define EDFMM_LAUNCH_M2L_TF_BLOCK 1
#define EDFMM_LAUNCH_NEAR_OVERLAP 2
#define EDFMM_LAUNCH_M2L_PACKED 3
EDFMM_API int edfmm_plan_set_launch(edfmm_plan *plan, int knob, int value);
EDFMM_API int edfmm_plan_get_launch(const edfmm_plan *plan, int knob, int *value);

/*
 * Change the expansion order p (FmmConfig.expansion_order,
 * electrodrive/fmm3d/config.py:90-106); reallocates the expansion buffers.
 */
EDFMM_API int edfmm_plan_set_order(edfmm_plan *plan, int expansion_order, void *stream);
/* Batched plans: from now on a matvec skips the M2L rows and near-field
 * leaves of every instance k with flags_dev[k * stride] == 0.0 (FP64 device
 * array, read when the kernels run, so a captured graph follows its changes);
 * those instances' outputs are left unspecified.  NULL removes the mask.
 * Used by the batched GMRES while instances sit out the rest of a cycle. */
EDFMM_API int edfmm_plan_set_instance_mask(edfmm_plan *plan, const double *flags_dev, int stride);

EDFMM_API int edfmm_plan_get_info(const edfmm_plan *plan, edfmm_plan_info *info_out);

/*
 * Copy the tree into caller buffers in the reference's SoA layout
 * (FmmTree._build_soa, electrodrive/fmm3d/tree.py:286-348).  Any pointer may
 * be NULL.  Float arrays are in the plan dtype; centers/half_extents (M,3),
 * children (M,8) with -1 for a missing child, ranges (M,2) [start, end).
 */
EDFMM_API int edfmm_plan_export_tree(const edfmm_plan *plan, int64_t *index_map_dev, void *centers_dev,
                           void *half_extents_dev, void *radii_dev, int32_t *levels_dev,
                           int64_t *parents_dev, int64_t *children_dev, int64_t *ranges_dev,
                           uint8_t *is_leaf_dev, void *stream);

/*
 * Copy the interaction lists as (src, tgt) pairs sorted by (tgt, src), the
 * InteractionLists.p2p_pairs / m2l_pairs order
 * (electrodrive/fmm3d/interaction_lists.py:474-485).  Either pointer may be NULL.
 */
EDFMM_API int edfmm_plan_export_lists(const edfmm_plan *plan, int64_t *p2p_pairs_dev, int64_t *m2l_pairs_dev,
                            void *stream);

/*
 * The single-layer operator, LaplaceFmm3D.matvec
 * (electrodrive/fmm3d/bem_fmm.py:760-885, GPU body :596-754):
 *   q = sigma * areas; V = k_e * (phi_far + phi_near) in original order;
 *   V += self_integrals * sigma * areas when self_integrals_dev != NULL;
 *   non-finite entries of V -> 0.
 * sigma/areas/self_integrals/out: (n,) original order, plan dtype.
 * Allocates nothing; safe to call repeatedly on the same stream.
 */
EDFMM_API int edfmm_plan_matvec(edfmm_plan *plan, const void *sigma_dev, const void *areas_dev,
                      const void *self_integrals_dev, double k_e, void *out_dev, int flags,
                      void *stream);

/*
 * Stage entry points on the plan's own expansion buffers, mirroring the
 * tree-level operators p2m / m2m / m2l / l2l / l2p
 * (electrodrive/fmm3d/multipole_operators.py:1520-1765) and the near field
 * apply_p2p_gpu (electrodrive/fmm3d/kernels_gpu.py:242-274).
 * charges_dev: (n,) in ORIGINAL order.  phi_*_tree_dev: (n,) in TREE order,
 * pure 1/r kernel (no k_e).
 */
EDFMM_API int edfmm_plan_set_charges(edfmm_plan *plan, const void *charges_dev, void *stream);
EDFMM_API int edfmm_plan_p2m(edfmm_plan *plan, void *stream);
EDFMM_API int edfmm_plan_m2m(edfmm_plan *plan, void *stream);
EDFMM_API int edfmm_plan_m2l(edfmm_plan *plan, int flags, void *stream);
EDFMM_API int edfmm_plan_l2l(edfmm_plan *plan, void *stream);
EDFMM_API int edfmm_plan_l2p(edfmm_plan *plan, void *phi_far_tree_dev, void *stream);
EDFMM_API int edfmm_plan_p2p(edfmm_plan *plan, void *phi_near_tree_dev, void *stream);

/*
 * Expansion coefficients, packed (n_nodes, (p+1)(p+2)/2) complex (re, im
 * interleaved, plan dtype), m >= 0 only, index (n, m) -> n(n+1)/2 + m.
 * Coefficients use complex solid harmonics with the Condon-Shortley phase,
 * scaled by the node radius a: Mhat_n^m = M_n^m / a^n, Lhat_n^m = L_n^m a^n.
 */
EDFMM_API int edfmm_plan_get_expansions(const edfmm_plan *plan, void *multipoles_dev, void *locals_dev,
                              void *stream);

/*
 * Dense single-layer operator, the reference's torch-tiled A(x)
 * (electrodrive/core/bem_kernel.py:157-230, wrapper :341-381):
 *   out_i = k_e sum_{j != i} sigma_j areas_j / sqrt(max(|c_i - c_j|^2, 1e-24))
 *           + self_integrals_i sigma_i areas_i   (self term only if non-NULL);
 *   non-finite entries -> 0.  centroids (n, 3) row-major, vectors (n,).
 * Partial sums live in stream-ordered scratch (cudaMallocAsync/cudaFreeAsync
 * on `stream`).
 */
EDFMM_API int edfmm_dense_matvec(const void *centroids_dev, const void *sigma_dev, const void *areas_dev,
                                 const void *self_integrals_dev, int64_t n, int dtype, double k_e, void *out_dev,
                                 void *stream);

/*
 * The same dense operator for callers that cannot allocate device memory:
 * for example an application whose framework allocator already holds the
 * GPU's free memory, or a host-language binding that has no CUDA allocator
 * and cannot free device memory it did not create.  No counterpart in the
 * reference (it has no device code for this operator).
 *
 * Allocates nothing: the partial sums live in a fixed 8 MiB file-scope
 * device array that every GPU loading the library keeps until exit.
 * Limit: n <= 262144 panels; larger n returns EDFMM_ERR_ARG with a message
 * (use edfmm_dense_matvec).  The caller still provides all inputs and `out`.
 * The first call on each device looks up the array's device address with
 * cudaGetSymbolAddress; make that first call before any stream capture.
 * The address is kept for the life of the process, so do not call this
 * entry point after cudaDeviceReset (or anything else that recreates the
 * device's primary context) in the same process.
 * All calls share the array, so calls whose work overlaps on the GPU (on
 * different streams, or on different host threads without ordering) race;
 * order them on one stream.  Each call rewrites every scratch slot it reads,
 * so no clearing is needed between calls.
 */
EDFMM_API int edfmm_dense_matvec_noalloc(const void *centroids_dev, const void *sigma_dev, const void *areas_dev,
                                         const void *self_integrals_dev, int64_t n, int dtype, double k_e,
                                         void *out_dev, void *stream);

/*
 * Induced potential at separate targets (bem_potential_targets,
 * electrodrive/core/bem_kernel.py:233-270):
 *   out_t = k_e sum_j sigma_j areas_j / sqrt(max(|x_t - c_j|^2, 1e-24)).
 * targets (m, 3); stream-ordered scratch.
 */
EDFMM_API int edfmm_dense_potential_targets(const void *targets_dev, int64_t m, const void *centroids_dev,
                                            const void *sigma_dev, const void *areas_dev, int64_t n, int dtype,
                                            double k_e, void *out_dev, void *stream);
/* Induced field at m separate targets (bem_E_field_targets, the Laplace fast
 * path of electrodrive/core/bem_kernel.py:280-335):
 *   E_i = sum_j (k_e / max(|x_i - r_j|^2, 1e-24)^(3/2)) (sigma_j A_j) (x_i - r_j),
 * non-finite components set to zero as the reference does; targets (m, 3) and
 * centroids (n, 3) row-major, out (m, 3). */
EDFMM_API int edfmm_dense_field_targets(const void *targets_dev, int64_t m, const void *centroids_dev,
                                        const void *sigma_dev, const void *areas_dev, int64_t n, int dtype,
                                        double k_e, void *out_dev, void *stream);

/*
 * Dense operator with a caller-provided workspace of
 * edfmm_dense_workspace_bytes(n, dtype) bytes (may be 0): allocates nothing,
 * so it can be captured in a CUDA graph.  Same math as edfmm_dense_matvec.
 */
EDFMM_API size_t edfmm_dense_workspace_bytes(int64_t n, int dtype);
EDFMM_API int edfmm_dense_matvec_ws(const void *centroids_dev, const void *sigma_dev, const void *areas_dev,
                                    const void *self_integrals_dev, int64_t n, int dtype, double k_e, void *out_dev,
                                    void *workspace_dev, size_t workspace_bytes, void *stream);

/*
 * Device Krylov arithmetic of restarted left-preconditioned GMRES
 * (gmres_restart, electrodrive/core/bem_solver.py:125-920).  Vectors in
 * `dtype`; inner products, H (restart+1, restart) row-major, g, cs, sn and
 * scal are FP64.  pinv (n,) is the diagonal left preconditioner or NULL.
 * scal (5 + restart doubles): [0] |b - Ax| at cycle start, [1] beta = |M(b - Ax)|,
 * [2] first breakdown step or -1, [3] non-finite flag, [4 + j] |g_{j+1}| after
 * step j.  work: edfmm_gmres_work_bytes(n, restart) bytes, zeroed once.
 *   start:   V0 = M(b - ax) / beta, g = beta e1                (bem_solver.py:399-450)
 *   arnoldi: w = M av, CGS2 against V0..Vj, H[:, j], Givens,
 *            g, V_{j+1} = w / H[j+1, j]                          (bem_solver.py:536-616)
 *   update:  y = R^{-1} g[0:m], x += V[0:m]^T y                  (bem_solver.py:762-772)
 * All stream-ordered, no host synchronisation, no allocation.
 */
EDFMM_API size_t edfmm_gmres_work_bytes(int64_t n, int restart);
EDFMM_API int edfmm_gmres_start(int64_t n, int dtype, int restart, const void *b_dev, const void *ax_dev,
                                const void *pinv_dev, void *v0_dev, void *g_dev, void *scal_dev, void *work_dev,
                                void *stream);
EDFMM_API int edfmm_gmres_arnoldi(int64_t n, int dtype, int restart, int j, void *V_dev, const void *av_dev,
                                  const void *pinv_dev, void *H_dev, void *g_dev, void *cs_dev, void *sn_dev,
                                  void *scal_dev, void *w_dev, void *work_dev, void *stream);
EDFMM_API int edfmm_gmres_update(int64_t n, int dtype, int restart, int m, const void *V_dev, const void *H_dev,
                                 const void *g_dev, void *x_dev, void *work_dev, void *stream);

/*
 * Batched GMRES: K independent systems back to back in one vector (instance k
 * owns rows soff[k] .. soff[k+1]-1; soff_dev holds K+1 int64 offsets and
 * max_seg is the longest instance).  Each instance runs the algorithm above
 * (gmres_restart, electrodrive/core/bem_solver.py:125-920, with the cycle
 * ending at the step where the instance's residual estimate meets
 * tol_k * beta_first_k) in its own Krylov space and Hessenberg matrix, while
 * every step shares one operator application over the whole vector (a block
 * diagonal operator, e.g. a batched plan).  V (restart+1, n) and w (n,) are
 * in `dtype`.  state: K rows of edfmm_bgmres_state_cols(restart) doubles:
 * [0] |b - Ax| at cycle start, [1] beta, [2] first breakdown step or -1,
 * [3] non-finite flag, [4] last subdiagonal, [5] estimate threshold,
 * [6] true-residual threshold, [7] steps this cycle, [8] active flag,
 * [9] steps in all cycles, [10 + j] |g_{j+1}| after step j.
 * work: edfmm_bgmres_work_bytes(K, max_seg, restart) bytes.
 *   start:   per instance r = b - ax, V0 = M r / beta, thresholds on the first
 *            call (tol_dev: K doubles, a negative value leaves the instance
 *            out), active = |r| above its threshold
 *   arnoldi: step j for every active instance (av = A V_j for all rows)
 *   update:  per instance y = R^{-1} g, x += V^T y (m = steps of the longest)
 */
EDFMM_API size_t edfmm_bgmres_state_cols(int restart);
EDFMM_API size_t edfmm_bgmres_work_bytes(int K, int max_seg, int restart);
EDFMM_API int edfmm_bgmres_start(int64_t n, int dtype, int K, const int64_t *soff_dev, int max_seg, int restart,
                                 const void *b_dev, const void *ax_dev, const void *pinv_dev, void *v0_dev,
                                 const double *tol_dev, int first, void *state_dev, void *work_dev, void *stream);
EDFMM_API int edfmm_bgmres_arnoldi(int64_t n, int dtype, int K, const int64_t *soff_dev, int max_seg, int restart,
                                   int j, void *V_dev, const void *av_dev, const void *pinv_dev, void *w_dev,
                                   void *state_dev, void *work_dev, void *stream);
EDFMM_API int edfmm_bgmres_update(int64_t n, int dtype, int K, const int64_t *soff_dev, int max_seg, int restart,
                                  int m, const void *V_dev, void *x_dev, void *state_dev, void *work_dev,
                                  void *stream);

/*
 * Singular and near-singular panel quadrature (FP64 geometry).
 * panel_vertices (n, 3, 3), centroids (n, 3), areas (n,): FP64 device arrays.
 *
 * edfmm_self_integrals: I_i = sum_k k_e w_k / max(|C_i - y_k|, 1e-12) with the
 *   adaptive rule near_singular_quadrature(C_i, panel_i, order, max_depth=depth)
 *   (electrodrive/core/bem_quadrature.py:217-308, used at core/bem.py:1781-1805).
 */
EDFMM_API int edfmm_self_integrals(const void *panel_vertices_dev, const void *centroids_dev, int64_t n,
                                   int quad_order, int depth, double k_e, void *out_dev, void *stream);
/* Near-field correction of potentials at m arbitrary targets
 * (_apply_near_quadrature_potentials, electrodrive/core/bem.py:940-1046), in
 * place on V (m, FP64): for every panel j with |C_j - x| <= distance_factor *
 * sqrt(A_j / pi), A_j > 0 and sigma_j != 0,
 *   V(x) += sigma_j (I_near - k_e A_j / max(|C_j - x|, 1e-12)),
 * I_near the adaptive rule of edfmm_self_integrals about x.  All arrays FP64:
 * targets (m, 3), centroids (n, 3), areas, sigma (n), panel_vertices (n, 3, 3). */
EDFMM_API int edfmm_near_targets_correct(const void *targets_dev, int64_t m, const void *centroids_dev,
                                         const void *areas_dev, const void *sigma_dev,
                                         const void *panel_vertices_dev, int64_t n, double distance_factor,
                                         int quad_order, int depth, double k_e, void *V_dev, void *stream);

/*
 * Near-pair correction set (core/bem.py:475-734): pairs 0 < |C_i - C_j| <=
 * f (R_i + R_j), R = sqrt(A / pi) (_build_near_pairs_for_panels), weights
 * delta_ij = I_near(C_i, panel_j refined uniformly `depth` times) -
 * k_e A_j / |C_i - C_j| (_precompute_near_correction_weights), stored as CSR
 * rows by target with sources ascending.  edfmm_near_apply computes
 * v_out = v_in + sum_j sigma_j delta_ij (_apply_near_quadrature_matvec_torch)
 * in `dtype` (v_in may be NULL, v_out may alias v_in).
 */
typedef struct edfmm_near edfmm_near;
EDFMM_API int edfmm_near_create(const void *centroids_dev, const void *areas_dev, const void *panel_vertices_dev,
                                int64_t n, double distance_factor, int quad_order, int depth, double k_e, int dtype,
                                void *stream, edfmm_near **near_out);
/* The same pairs and FP64 weights held for another solve dtype (no new pair
 * search or quadrature): the result equals edfmm_near_create with `dtype`. */
EDFMM_API int edfmm_near_convert(const edfmm_near *near_set, int dtype, void *stream, edfmm_near **near_out);
EDFMM_API int edfmm_near_destroy(edfmm_near *near_set);
EDFMM_API int64_t edfmm_near_num_pairs(const edfmm_near *near_set);
/* (P, 2) int64 (i, j) pairs in row order and FP64 weights; either may be NULL */
EDFMM_API int edfmm_near_export(const edfmm_near *near_set, int64_t *pairs_dev, double *weights_dev, void *stream);
EDFMM_API int edfmm_near_apply(const edfmm_near *near_set, const void *sigma_dev, const void *v_in_dev,
                               void *v_out_dev, void *stream);
EDFMM_API int edfmm_near_rows(const edfmm_near *near_set, const int32_t **row_off_dev, const int32_t **cols_dev);

/*
 * The reference CUDA near-field module's operation (pybind
 * near_quadrature_matvec, core/bem_near_cuda.cpp:239-271; kernel
 * core/bem_near_cuda_kernel.cu:110-232): v_out = v_far + correction with the
 * unrefined rule of quad_order (1 or 2) recomputed per call; pairs as CSR
 * (row_off (n+1), cols) by target.  Arrays in `dtype`.
 */
EDFMM_API int edfmm_near_quadrature_matvec(const void *v_far_dev, const void *sigma_dev, const void *centroids_dev,
                                           const void *areas_dev, const void *panel_vertices_dev,
                                           const int32_t *row_off_dev, const int32_t *cols_dev, int64_t n,
                                           double k_e, int quad_order, int dtype, void *v_out_dev, void *stream);

/*
 * Free-space potential of point charges at points (core/bem.py:291-320):
 * out_i = sum_k k_e q_k / max(|x_i - r_k|, 1e-12); charges (n_charges, 4) FP64
 * rows (q, x, y, z) on the device; points / out in `dtype`.
 */
EDFMM_API int edfmm_point_charge_potential(const void *points_dev, int64_t n, const double *charges_dev,
                                           int n_charges, double k_e, int dtype, void *out_dev, void *stream);

/*
 * Number of the library's own kernel launches issued since load (all
 * threads).  Used by benchmarks to report launches inside a timed region.
 */
EDFMM_API int64_t edfmm_launch_count(void);

/*
 * Measured FP32 FMA throughput of the current device in TFLOP/s (an FMA
 * counts as 2 flops): the roofline denominator of the FP32-bound FMM stages.
 * No counterpart in the reference (it has no GPU kernels for the FMM).
 */
EDFMM_API int edfmm_measure_fp32_peak(int iters, void *stream, double *tflops_out);

/*
 * Potential of a plan's panel charges at arbitrary target points by FMM
 * (replaces bem_potential_targets, electrodrive/core/bem_kernel.py:233-270,
 * for large panel and target counts).  edfmm_targets_create builds a tree of
 * the targets (the plan's leaf size and depth) and the interaction lists
 * between the plan's tree and it, as the reference's
 * build_interaction_lists(source_tree, target_tree) does
 * (electrodrive/fmm3d/interaction_lists.py:374-577).
 * edfmm_targets_potential writes out[i] = k_e * sum_j sigma_j A_j / |x_i - c_j|
 * (FMM, p of the plan; distances clamped at the dtype's epsilon) in the
 * targets' original order.  edfmm_targets_field writes the field
 * out[3 i + c] = k_e * E_c(x_i), E = sum_j sigma_j A_j (x_i - c_j) / |x_i - c_j|^3
 * (zero for distances within the dtype's epsilon; far part as minus the
 * gradient of the local expansions), the FMM counterpart of the dense
 * bem_E_field_targets (electrodrive/core/bem_kernel.py:914).  The targets
 * object keeps a pointer to the plan, which must outlive it.  A batched plan
 * (edfmm_plan_create_batch) has no targets: EDFMM_ERR_UNSUPPORTED.
 */
typedef struct edfmm_targets edfmm_targets;
EDFMM_API int edfmm_targets_create(edfmm_plan *plan, const void *targets_dev, int64_t m, void *stream,
                                   edfmm_targets **targets_out);
EDFMM_API int edfmm_targets_destroy(edfmm_targets *targets);
EDFMM_API int edfmm_targets_info(const edfmm_targets *targets, int64_t *n_nodes, int64_t *n_p2p_pairs,
                                 int64_t *n_m2l_pairs, int64_t *p2p_interactions);
/* (src, tgt) node pairs, sorted by (tgt, src), as edfmm_plan_export_lists */
EDFMM_API int edfmm_targets_export_lists(const edfmm_targets *targets, int64_t *p2p_pairs_dev, int64_t *m2l_pairs_dev,
                                         void *stream);
EDFMM_API int edfmm_targets_potential(edfmm_targets *targets, const void *sigma_dev, const void *areas_dev, double k_e,
                                      void *out_dev, int flags, void *stream);
EDFMM_API int edfmm_targets_field(edfmm_targets *targets, const void *sigma_dev, const void *areas_dev, double k_e,
                                  void *out_dev, int flags, void *stream);

/*
 * Two-tree lists over a target tree the caller already built as a plan of its
 * own (build_interaction_lists(source_tree, target_tree, mac_theta),
 * electrodrive/fmm3d/interaction_lists.py:531-577): the target plan's tree is
 * copied (so the target plan may be destroyed afterwards), the lists between
 * the source plan's tree and it are built with `mac_theta`, and the target
 * locals are allocated at the source plan's expansion order.  Both plans must
 * share a dtype and be unbatched.
 */
EDFMM_API int edfmm_targets_create_from_plan(edfmm_plan *source_plan, const edfmm_plan *target_plan, double mac_theta,
                                             void *stream, edfmm_targets **targets_out);
/*
 * The reference's tree-level stages between a source tree and a target tree
 * (electrodrive/fmm3d/multipole_operators.py:1630-1765 and
 * electrodrive/fmm3d/kernels_gpu.py:242-274 with distinct trees), on the
 * source plan's current multipoles and charges:
 *   EDFMM_TARGETS_M2L     target locals = M2L over the two-tree M2L list
 *   EDFMM_TARGETS_L2L     parent-to-child local translation in the target tree
 *   EDFMM_TARGETS_L2P     out[i] = far potential at target point i (tree order, 1/r)
 *   EDFMM_TARGETS_P2P     out[i] = sum over the two-tree P2P list of q_j / max(r, eps)
 *                         (tree order; no self exclusion between distinct trees)
 *   EDFMM_TARGETS_LOCALS  out = the target locals, (n_target_nodes, (p+1)(p+2)/2) complex
 * Returns EDFMM_ERR_STATE when the source plan's expansion order changed since
 * the targets were created.
 */
#define EDFMM_TARGETS_M2L 1
#define EDFMM_TARGETS_L2L 2
#define EDFMM_TARGETS_L2P 3
#define EDFMM_TARGETS_P2P 4
#define EDFMM_TARGETS_LOCALS 5
EDFMM_API int edfmm_targets_stage(edfmm_targets *targets, int stage, void *out_dev, void *stream);

/*
 * Point-cloud warm-start network (no counterpart in the reference: it maps
 * per-panel features to an initial surface charge density for the GMRES
 * start).  Width 128, 16 input features (8 used), BF16 weights/activations on
 * the tensor cores, FP32 accumulation.  Parameters are one FP32 block of
 * edfmm_pcn_num_params() values: W1[128x16] b1[128] W2[128x128] V2[128x128]
 * b2[128] W3[128x128] b3[128] w4[128] b4.  The workspace holds the
 * activations of one forward pass, which edfmm_pcn_backward reuses (call it
 * with the same workspace right after the forward).  All pointers are device
 * pointers; the calls are stream-ordered and deterministic.
 */
#define EDFMM_PCN_WIDTH 128
#define EDFMM_PCN_INPUTS 16
EDFMM_API int64_t edfmm_pcn_num_params(void);
EDFMM_API size_t edfmm_pcn_workspace_bytes(int64_t n);
/* features (n x 16 FP32): centroid relative to the mean centroid over the
 * RMS radius R, unit normal, log(area / R^2), rhs / RMS rhs, zeros */
EDFMM_API int edfmm_pcn_features(const double *centroids_dev, const double *normals_dev, const double *areas_dev,
                                 const double *rhs_dev, int64_t n, float *features_dev, void *ws_dev, size_t ws_bytes,
                                 void *stream);
EDFMM_API int edfmm_pcn_forward(const float *params_dev, const float *features_dev, int64_t n, float *y_dev,
                                void *ws_dev, size_t ws_bytes, void *stream);
EDFMM_API int edfmm_pcn_backward(const float *params_dev, int64_t n, const float *dy_dev, float *grads_dev,
                                 void *ws_dev, size_t ws_bytes, void *stream);
/* L = sum_i A_i (s_i (1 + y_i) - sigma_i)^2 / sum_i A_i sigma_i^2 and dL/dy */
EDFMM_API int edfmm_pcn_loss(const float *y_dev, const double *scale_dev, const double *sigma_dev,
                             const double *areas_dev, int64_t n, float *dy_dev, double *loss_dev, void *stream);
EDFMM_API int edfmm_pcn_adam(float *params_dev, const float *grads_dev, float *m_dev, float *v_dev, int64_t count,
                             float lr, float beta1, float beta2, float eps, int step, void *stream);

/*
 * Tensor-grid conductor meshes on the GPU (the mesh generators of
 * electrodrive/core/bem_mesh.py:27-212: _mesh_sphere, _mesh_torus,
 * _mesh_plane_patch, joined and finished as generate_mesh does).
 * edfmm_mesh_grid writes one grid's na * nb vertices (row-major, at
 * vertices_dev; the caller offsets the pointer) and its raw triangles (two
 * per cell, vertex ids + vertex_offset) with their conductor id.  Tables
 * (device, FP64): EDFMM_MESH_SPHERE ta = (sin, cos) of the polar angles,
 * tb = (sin, cos) of the azimuths, params (cx, cy, cz, radius);
 * EDFMM_MESH_TORUS ta = (sin, cos) of u, tb = (sin, cos) of v, params
 * (cx, cy, cz, R, a); EDFMM_MESH_PLANE ta = x values, tb = y values,
 * params (z).  edfmm_mesh_finish computes every raw panel's area
 * 0.5 |(v1 - v0) x (v2 - v0)|, drops panels with area <= 1e-16 (order kept),
 * and writes the kept panels' triangles, conductor ids, centroids, unit
 * normals cross / (2 area + 1e-30) and areas; *n_out_host receives their
 * count (the call synchronises `stream`).  Every operation follows numpy's
 * evaluation order with correctly rounded arithmetic, so the arrays equal the
 * host generators' bit for bit for the same tables.  Outputs are sized for
 * n_triangles panels.
 */
#define EDFMM_MESH_SPHERE 1
#define EDFMM_MESH_TORUS 2
#define EDFMM_MESH_PLANE 3
EDFMM_API int edfmm_mesh_grid(int kind, const double *params_host, const double *tab_a_dev, int64_t na,
                              const double *tab_b_dev, int64_t nb, int64_t vertex_offset, int32_t conductor_id,
                              double *vertices_dev, int32_t *triangles_dev, int32_t *conductor_ids_dev, void *stream);
EDFMM_API int edfmm_mesh_finish(const double *vertices_dev, int64_t n_vertices, const int32_t *triangles_dev,
                                const int32_t *conductor_ids_dev, int64_t n_triangles, int32_t *triangles_out_dev,
                                int32_t *conductor_ids_out_dev, double *centroids_dev, double *normals_dev,
                                double *areas_dev, int64_t *n_out_host, void *stream);

/*
 * Measured FP64 FMA throughput (TFLOP/s): the roofline denominator of the
 * FP64 dense operator.  No counterpart in the reference.
 */
EDFMM_API int edfmm_measure_fp64_peak(int iters, void *stream, double *tflops_out);

#ifdef __cplusplus
}
#endif

#endif /* EDFMM_H */
