/*
 * qiw -- GB300-native qMC diagram integration for the inchworm algorithm (C ABI).
 *
 * One library call replaces the per-(inch step, topology group) qMC integral that
 * QInchworm.jl evaluates with
 *     contour_integral(t -> eval(td.topologies, t), c, trans; seq, N)
 * at src/inchworm.jl:181-187 (bold step), :281-287 (bare step) and :868-875 (correlator),
 * i.e. the value `res` just before `all_reduce!` (src/inchworm.jl:178-189):
 *     res = rank_weight * (1/N_rank) * sum_{i in rank range} prod(branch_direction) * J * eval(u(x_i)).
 *
 * Conventions
 *   - All pointers are host pointers owned by the caller for the duration of the call;
 *     calls are synchronous (results are in the output buffers on return).
 *   - Complex numbers are interleaved (re, im) doubles, exactly Julia's ComplexF64 layout.
 *   - Matrices are column-major (Julia's Matrix layout); sectors are 0-based.
 *   - Every entry point returns QIW_OK (0) or an error code; qiw_last_error() gives text.
 *     Nothing aborts the process.
 *   - One context per host thread; a context owns its device buffers and CUDA stream.
 */
#ifndef QIW_H
#define QIW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QIW_OK 0
#define QIW_ERR_ARG 1          /* invalid argument / layout */
#define QIW_ERR_CUDA 2         /* CUDA runtime failure */
#define QIW_ERR_UNSUPPORTED 3  /* valid input outside what this build supports */
#define QIW_ERR_OFFDIAG 4      /* block off-diagonal leaf (src/topology_eval.jl:462-464) */
#define QIW_ERR_DEVICE 5       /* kernel error word set (bounds / non-finite result) */
#define QIW_ERR_MEMORY 6       /* plan exceeds the per-sample working-set budget */

/* propagator (Delta) interpolation rules */
#define QIW_PROP_LINEAR 0      /* Keldysh ImaginaryTimeGF call (linear on the grid) */
#define QIW_PROP_CUBIC 1       /* SplineInterpolatedGF: natural cubic spline (src/spline_gf.jl:195-202) */

/* topology group kinds (fixed-node layouts of src/inchworm.jl) */
#define QIW_GROUP_BOLD 0       /* IdentityNode(t_i), InchNode(t_w), IdentityNode(t_f); P bold  (:161-165) */
#define QIW_GROUP_BARE 1       /* IdentityNode(t_i), IdentityNode(t_f); exact atomic P0         (:266-268) */
#define QIW_GROUP_CORRELATOR 2 /* OperatorNode(B,t_i), OperatorNode(A,t_w), IdentityNode(t_f)  (:846-850) */
#define QIW_GROUP_SIGMA 3      /* self-energy: PairNode(t_i), PairNode(t_f), 2k-2 vertices between (:560-566) */

/* arithmetic of the chain products */
#define QIW_PREC_FP64 0        /* plain FP64 throughout */
#define QIW_PREC_FP32 1        /* FP32 chain products, FP64 compensated accumulation of qMC sums */
#define QIW_PREC_FP32_TC 2     /* QIW_PREC_FP32 with the operator multiplies of 9-wide sector blocks on
                                  tensor cores (mma.sync TF32, 3xTF32 split; large-block problems only) */

typedef struct qiw_ctx qiw_ctx;

/* Replaces: nothing in the reference (it has no device state); creates a context on a device. */
int qiw_ctx_create(qiw_ctx **out, int device);
void qiw_ctx_destroy(qiw_ctx *ctx);
/* Last error message of this context (never NULL). */
const char *qiw_last_error(const qiw_ctx *ctx);

/*
 * Problem data of an `Expansion` (src/expansion.jl:107-197).
 * Operators are SectorBlockMatrix objects (src/sector_block_matrix.jl:44): operator o has
 * op_n_blocks[o] blocks; block b of it is (s_i, s_f) = op_blocks[2*k], op_blocks[2*k+1]
 * (k = running block index over all operators) with a d_f x d_i column-major complex
 * matrix at op_values + 2*op_value_offset[k].
 */
typedef struct {
    int32_t n_sectors;
    const int32_t *sector_dims;        /* [n_sectors] */
    double beta;
    int32_t n_tau;                     /* uniform grid tau_j = j*beta/(n_tau-1) */
    const double *atomic_energies;     /* [sum d]: E + lambda of ExactAtomicPPGF (src/exact_atomic_ppgf.jl:134) */
    int32_t n_ops;
    const int32_t *op_n_blocks;        /* [n_ops] */
    const int32_t *op_blocks;          /* [2 * total blocks] */
    const int64_t *op_value_offset;    /* [total blocks], in complex elements */
    const double *op_values;           /* complex */
    int32_t identity_op;               /* index of expansion.identity_mat */
    int32_t n_pairs;                   /* InteractionPair list (src/expansion.jl:79-90) */
    const int32_t *pair_ops;           /* [2*n_pairs]: (operator_i, operator_f) operator indices */
    const int32_t *pair_prop_kind;     /* [n_pairs]: QIW_PROP_* */
    const double *pair_prop_data;      /* [n_pairs][n_tau] complex: propagator(tau_j, 0) */
} qiw_problem_desc;

/* Replaces: the per-call reads of expansion.P0/pairs/operators in TopologyEvaluator
 * (src/topology_eval.jl:249-331).  Invalidates previously created groups. */
int qiw_problem_set(qiw_ctx *ctx, const qiw_problem_desc *desc);

/* Replaces: the bold P read by kd.interpolate! (src/topology_eval.jl:368) after
 * set_ppgf!/normalize! (src/inchworm.jl:487-488).  `P` holds, for each sector s in
 * order, expansion.P[s].mat.data: d_s x d_s x n_tau complex, column-major. */
int qiw_ppgf_set(qiw_ctx *ctx, const double *P);

/* A TopologiesInputData group (src/inchworm.jl:76-87). */
typedef struct {
    int32_t kind;                      /* QIW_GROUP_* */
    int32_t order;
    int32_t n_pts_after;               /* d_after; ignored for QIW_GROUP_BARE */
    int32_t corr_A_op, corr_B_op;      /* QIW_GROUP_CORRELATOR: operator indices of A and B */
    int32_t n_topologies;
    const int32_t *top_pairs;          /* [n_topologies][order][2]: Topology.pairs (1-based vertices) */
    const int32_t *top_parity;         /* [n_topologies]: Topology.parity */
} qiw_group_desc;

/* Replaces: TopologyEvaluator construction (src/topology_eval.jl:249-331).  Plans the
 * group: the configuration tree of every topology and initial sector is enumerated once
 * (it does not depend on the sample times) and configurations that share their future
 * are merged; the result is a sample-independent instruction stream. */
int qiw_group_create(qiw_ctx *ctx, const qiw_group_desc *desc, int32_t *group_id);

typedef struct {
    int64_t n_nodes_dag;       /* merged configuration-DAG states */
    int64_t n_instructions;
    int64_t arena_elements;    /* per-sample working set (matrix elements) */
    double flops_per_sample;   /* algorithmic flops executed per qMC sample */
    double tree_flops_per_sample; /* flops the reference's per-topology tree would need */
    int64_t n_leaves_tree;     /* configurations the reference traverses per sample */
} qiw_group_stats;

int qiw_group_stats_get(qiw_ctx *ctx, int32_t group_id, qiw_group_stats *out);

/* Plan cache of the process.  qiw_group_create (and qiw_batch_add) keep every plan they make,
 * keyed by the operator structure of the problem (sector dimensions, operator blocks and
 * values, pair operators) and the group (kind, order, n_pts_after, correlator operators,
 * topologies, parities).  Plans hold no times or tables, so a solve repeated with a new Delta,
 * beta or grid on the same operators (an outer self-consistency loop around inchworm!) plans
 * no group again, in any context or batch.  Thread-safe.  The cache is emptied when it would
 * exceed 2 GiB of host memory, or by qiw_plan_cache_clear. */
int qiw_plan_cache_info(int64_t *entries, int64_t *hits, int64_t *bytes);
int qiw_plan_cache_clear(void);

/* Domain maps of a bare group (src/qmc_integrate.jl): the default is RootTransform (:198-258);
 * SortTransform (:282-334) maps x to t_i + sort(x, rev=true) (t_f - t_i); ExpModelFunctionTransform
 * (:99-165) maps x to u_1 = t_f + tau log(1 - x_1), u_n = u_{n-1} + tau log(1 - x_n) with the
 * per-sample Jacobian tau^d / exp(-(t_f - u_d) / tau), discarding samples with u_d < 0 as
 * contour_integral does (:597-612); it needs t_i = 0 and takes tau from t_w.  Bold and correlator
 * groups take the default (DoubleSimplexRootTransform, :363-463) only. */
#define QIW_TRANSFORM_DEFAULT 0
#define QIW_TRANSFORM_SORT 1
#define QIW_TRANSFORM_EXPMODEL 2

/* One qMC integral of one group over a contiguous Sobol index range. */
typedef struct {
    int32_t group;
    int32_t transform;                 /* QIW_TRANSFORM_* (bare groups), else 0 */
    double t_i, t_w, t_f;              /* t_w unused for QIW_GROUP_BARE (EXPMODEL: the decay rate) */
    uint64_t first_index;              /* 0-based Sobol point index = first(N_range) - 1 */
    uint64_t n_samples;                /* length(N_range) */
    uint64_t n_total;                  /* td.N_samples (rank_weight = n_samples / n_total) */
    const uint32_t *sobol_m;           /* [2*order][32] direction numbers (ScrambledSobolSeq.m, row d) */
    const uint32_t *sobol_x0;          /* [2*order] initial point (digital shift; zeros if unscrambled) */
} qiw_work_desc;

/* Replaces: contour_integral(...) for each work item (src/qmc_integrate.jl:597-612 with the
 * integrand of src/topology_eval.jl:350-437).  out: for each work item, the result
 * SectorBlockMatrix as sum_s d_s^2 complex values (sector s block, column-major, sectors
 * in order).  All work items run in one launch. */
int qiw_integrate(qiw_ctx *ctx, int32_t n_work, const qiw_work_desc *work, int32_t precision,
                  double *out);

/* No counterpart in the reference.  qiw_integrate for callers that cannot allocate device
 * memory while they run: it allocates nothing.  Its scratch (launch tables, Sobol tables,
 * per-CTA partial sums) is one 16 MiB static device array per GPU, held until the process
 * exits; calls that need more are rejected with QIW_ERR_MEMORY.  `out_device` is a device
 * buffer the caller owns, laid out like qiw_integrate's `out`.  The first call on a device
 * looks the array's address up (make it before any stream capture).  All calls share the
 * array: calls that overlap on the GPU race and must be serialised by the caller. */
int qiw_integrate_noalloc(qiw_ctx *ctx, int32_t n_work, const qiw_work_desc *work, int32_t precision,
                          double *out_device);

/*
 * Learned change of variables (no counterpart in the reference; its closest relative is the
 * hand-made ExpModelFunctionTransform, src/qmc_integrate.jl:99-165).  A warp is a triangular
 * monotone map x = w(y) of [0,1]^D (D = 2*order <= 8): per dimension a 16-bin piecewise-linear
 * CDF whose bin masses come from a masked MLP (3 hidden layers of 64, BF16 weights, FP32
 * accumulation).  qiw_integrate_warped evaluates f(u(w(y))) J / q(w(y)) on the Sobol points
 * y: unbiased for any weights, so plain qMC stays the reference for its variance and error.
 */
int qiw_warp_create(qiw_ctx *ctx, int32_t D, uint64_t seed, int32_t *warp_id);
/* Weight a in (0, 1] of the uniform density in q (default 0.3): 1/q <= a^-D. */
int qiw_warp_set_mix(qiw_ctx *ctx, int32_t warp_id, double uniform_mix);
int qiw_warp_n_params(qiw_ctx *ctx, int32_t warp_id, int64_t *n);
int qiw_warp_get_params(qiw_ctx *ctx, int32_t warp_id, double *params);
int qiw_warp_set_params(qiw_ctx *ctx, int32_t warp_id, const double *params);
/* Gradient of the |f|-weighted negative log-likelihood -sum_i w_i log q(x_i) / sum_i w_i. */
int qiw_warp_grad(qiw_ctx *ctx, int32_t warp_id, const double *x, const double *w, int64_t n, double *grad,
                  double *loss);
/* Adam on minibatches of (x_i in [0,1)^D, w_i = |f(x_i)|) produced by plain qMC. */
int qiw_warp_train(qiw_ctx *ctx, int32_t warp_id, const double *x, const double *w, int64_t n, int32_t steps,
                   int32_t batch, double lr, double *final_loss);
/* qiw_warp_train of n_warps distinct warps at once (warp k on x[k] [n[k]][D_k], w[k] [n[k]]),
 * trained concurrently on the device; final_loss (optional) receives n_warps values.  The
 * results equal n_warps qiw_warp_train calls. */
int qiw_warp_train_batch(qiw_ctx *ctx, int32_t n_warps, const int32_t *warp_ids, const double *const *x,
                         const double *const *w, const int64_t *n, int32_t steps, int32_t batch, double lr,
                         double *final_loss);
/* Warped points of Sobol indices first..first+n-1: [n][D + 1] = (x_1..x_D, 1/q(x)). */
int qiw_warp_map(qiw_ctx *ctx, int32_t warp_id, const uint32_t *sobol_m, const uint32_t *sobol_x0,
                 uint64_t first, uint64_t n, double *points);
/* qiw_integrate with a warp per work item (warp_ids[i] = -1: plain qMC). */
int qiw_integrate_warped(qiw_ctx *ctx, int32_t n_work, const qiw_work_desc *work, const int32_t *warp_ids,
                         int32_t precision, double *out);
/* qiw_integrate of one work item that also returns the per-sample integrand values
 * samples[n_samples][sum d_s^2] (real parts f_i with out = -i * J / N * sum_i f_i). */
int qiw_integrate_samples(qiw_ctx *ctx, const qiw_work_desc *work, int32_t precision, double *out,
                          double *samples);
/* The same for n_work work items in one launch: out as qiw_integrate, samples holds the items'
 * per-sample values one after another (item i: [n_samples_i][sum d_s^2]). */
int qiw_integrate_samples_batch(qiw_ctx *ctx, int32_t n_work, const qiw_work_desc *work, int32_t precision,
                                double *out, double *samples);
/* The same with only the Euclidean norm of each sample's values returned (norms[sum n_samples_i],
 * item after item): the training weights ||f_i|| of a learned warp, without copying the values. */
int qiw_integrate_sample_norms(qiw_ctx *ctx, int32_t n_work, const qiw_work_desc *work, int32_t precision,
                               double *out, double *norms);

/* Kernel time of the most recent qiw_integrate (ms, CUDA events on the context stream). */
double qiw_last_kernel_ms(const qiw_ctx *ctx);

/* The kernels' own Sobol integers (test and debugging interface): points first .. first + n - 1
 * of the D-dimensional sequence with direction numbers m [D][32] and digital shift x0 [D]
 * (unscrambled: x0 = 0), computed on the device by the Gray-code jump the evaluation kernels
 * use, written to out [n][D] (host buffer).  Point k is what the reference's next! returns on
 * its (k+1)-th call, and skip!(seq, first, exact=true) starts the range at `first`
 * (src/scrambled_sobol.jl:158-208).  first + n <= 2^32; n <= 2^26 per call. */
int qiw_sobol_points(qiw_ctx *ctx, int32_t D, const uint32_t *m, const uint32_t *x0, uint64_t first,
                     uint64_t n, uint32_t *out);

/* No counterpart in the reference: measures this device's CUDA-core FMA throughput
 * (QIW_PREC_FP64: DFMA, QIW_PREC_FP32: FFMA) in TFLOP/s with independent FMA chains on
 * every SM, the roofline denominator of the evaluation kernels. */
int qiw_measure_fma_peak(qiw_ctx *ctx, int32_t precision, double *tflops);

/* ---- Batched independent solves.  No counterpart in the reference, which runs one
 * inchworm! per process.  A solve is one whole inchworm! loop (src/inchworm.jl:332-498 with
 * one unscrambled Sobol sequence and one rank): the bare step tau_0 -> tau_1
 * (inchworm_step_bare, :431-447), then bold steps n = 1 .. n_steps (inchworm_step, :474-493),
 * each followed by set_ppgf! and normalize!(P, tau_{n+1}).  All solves of a batch share one
 * launch queue per step -- a persistent kernel over the tiles of every (solve, group) --
 * and the loop, P update included, runs on the device, optionally as one CUDA graph. */
typedef struct qiw_batch qiw_batch;

typedef struct {
  const qiw_problem_desc *problem;
  const double *taus;           /* [n_tau] grid times */
  const double *P_init;         /* initial P (atomic), interleaved complex, layout of qiw_ppgf_set */
  int32_t n_bare, n_bold;
  const qiw_group_desc *bare;   /* groups of the bare step */
  const qiw_group_desc *bold;   /* groups of every bold step, by ascending order */
  uint64_t n_samples;           /* qMC points per group and step: a power of 2, <= 2^32 */
  int32_t n_steps;              /* bold steps, 0 .. n_tau - 2 */
  int32_t reserved;
} qiw_solve_desc;

#define QIW_BATCH_GRAPH 1       /* capture the whole loop in one CUDA graph and launch that */
#define QIW_BATCH_AUTOTUNE 2    /* time tile sizes and grids on one step first, keep the fastest */

typedef struct {
  double kernel_ms;             /* device time of the last run, all steps */
  double flops;                 /* algorithmic flops of the last run (planner counts) */
  double topology_samples;      /* (topology, qMC sample) evaluations of the last run */
  int32_t threads;              /* samples per tile (threads per CTA) */
  int32_t grid;                 /* CTAs of each evaluation launch */
  int32_t persistent;           /* 1: grid = resident CTAs, 0: one CTA per tile */
  int32_t n_steps_max;
  int32_t graph_nodes;          /* 0 without QIW_BATCH_GRAPH */
  int32_t n_plans;              /* distinct group programs (shared by solves) */
  int64_t n_tiles_bold, n_tiles_bare;
  double tune_ms[6];            /* autotuner: step time of (threads 32, 64, 128) x (persistent, one per tile) */
} qiw_batch_stats;

int qiw_batch_create(qiw_batch **out, int device);
void qiw_batch_destroy(qiw_batch *b);
const char *qiw_batch_last_error(const qiw_batch *b);
int qiw_batch_add(qiw_batch *b, const qiw_solve_desc *solve, int32_t *solve_id);
/* Runs every solve from its P_init.  sobol_m: [sobol_dims][32] direction numbers, enough rows
 * for the highest order (2 * order <= sobol_dims). */
int qiw_batch_run(qiw_batch *b, int32_t precision, int32_t flags, const uint32_t *sobol_m, int32_t sobol_dims);
/* P of a solve after the last run, interleaved complex, layout of qiw_ppgf_set. */
int qiw_batch_get_P(qiw_batch *b, int32_t solve_id, double *P);
int qiw_batch_stats_get(const qiw_batch *b, qiw_batch_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* QIW_H */
