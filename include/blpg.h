/*
 * blpg.h — C ABI of the GB300 batched LP solver (libblpg.so).
 *
 * Solves a batch of independent dense linear programs
 *
 *     maximise  c^T x   subject to  A x <= b,  x >= 0
 *
 * with the dense-tableau primal simplex method: slack-basis start, Dantzig
 * pricing (most negative reduced cost) with lowest-index ties, minimum-ratio
 * test with lowest-basic-variable-index ties, one LP per CTA (or per
 * thread-block cluster when the tableau does not fit one CTA's shared memory).
 *
 * Reference interface replaced (zzambia/simplexprojects, BLPG-Solver):
 *   class Simplex                       BLPG-Solver/src/simplex.cuh:37-83
 *     Simplex(N_S, multipleBatch)       BLPG-Solver/src/simplex.cu:387-400
 *     setConstratint(A, b)              BLPG-Solver/src/simplex.cu:463-550
 *     ComputeLP(C, number_of_streams)   BLPG-Solver/src/simplex.cu:552-977
 *     getResultAll / getStatusAll       BLPG-Solver/src/simplex.cu:424-461
 *   __global__ mykernel(...)            BLPG-Solver/src/simplex.cu:35-385
 * The C++ mirror of that class over this ABI is include/blpg_simplex.hpp.
 *
 * Conventions: plain pointers and sizes only; every entry point returns 0 on
 * success or a negative BLPG_E* code, and blpg_last_error() gives a message
 * (thread-local).  Nothing here falls back to the CPU: without a usable
 * CUDA device the solve entry points return BLPG_ENODEV.
 */
#ifndef BLPG_H_
#define BLPG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BLPG_ABI_VERSION 1

/* Per-LP status: the numeric codes of GLPK's glp_get_status(), which the
 * reference's oracle wrapper reports (glpk_lp_solver.cpp:259-273).  The
 * reference kernel itself only ever reports 2 or 6 (simplex.cu:451-461). */
enum {
  BLPG_UNDEF = 1,  /* pivot cap reached before a verdict (GLPK: it_lim) */
  BLPG_FEAS = 2,
  BLPG_INFEAS = 3,
  BLPG_NOFEAS = 4, /* phase I proved that no x satisfies A x <= b, x >= 0 */
  BLPG_OPT = 5,
  BLPG_UNBND = 6
};

/* Error codes returned by the entry points. */
enum {
  BLPG_OK = 0,
  BLPG_EINVAL = -1,  /* bad argument (null pointer, m or n out of range ...) */
  BLPG_ENODEV = -2,  /* no CUDA device, or the device is not sm_103 */
  BLPG_ECUDA = -3,   /* a CUDA runtime call failed */
  BLPG_ENOMEM = -4,  /* device or pinned-host allocation failed */
  BLPG_ETOOBIG = -5, /* a tableau exceeds the largest cluster's shared memory */
  BLPG_EIO = -6,     /* file could not be read or parsed */
  BLPG_ESTATE = -7   /* call out of order (e.g. plan used after destroy) */
};

/* Arithmetic of the tableau. */
enum {
  BLPG_FP64 = 0, /* plain FP64 tableau: the drop-in path */
  BLPG_FP32 = 1  /* FP32 tableau with FP64 refresh of x_B and reduced costs */
};

/* Pricing rule of the primal simplex (blpg_options.pricing). */
enum {
  BLPG_PRICE_DANTZIG = 0, /* most negative reduced cost (the reference's rule) */
  BLPG_PRICE_STEEPEST = 1 /* largest d_j^2 / ||column j||^2, exact norms */
};

/* Largest LP handled: rows and total tableau columns (n + m + 1). */
#define BLPG_MAX_ROWS 1024
#define BLPG_MAX_COLS 8192

/* A batch of LPs in host (or, for blpg_plan_execute, device) memory.
 * LP k has m[k] rows and n[k] structural columns; its A is row-major
 * m[k] x n[k] at A + off_A[k], b at b + off_b[k], c at c + off_c[k].
 * Null offset arrays mean "packed": each LP follows the previous one.
 * The reference's batch mode (one A, b shared by all LPs, one objective
 * per LP — GPU_Tester.cu:119-127, simplex.cu:463-466) is off_A[k] = 0,
 * off_b[k] = 0 for every k. */
typedef struct blpg_batch {
  int32_t count;
  const int32_t* m;
  const int32_t* n;
  const int64_t* off_A; /* nullable */
  const int64_t* off_b; /* nullable */
  const int64_t* off_c; /* nullable */
  const double* A;
  const double* b;
  const double* c;
} blpg_batch;

typedef struct blpg_options {
  int32_t precision;       /* BLPG_FP64 (default) or BLPG_FP32 */
  int32_t max_pivots;      /* per-LP pivot cap; 0 = 50 * (m + n) + 1000 */
  int32_t bland_after;     /* consecutive degenerate pivots before Bland's
                              rule takes over for the rest of the LP; 0 = 64 */
  int32_t refactor_period; /* FP32 only: FP64 refresh of x_B, the duals and
                              the reduced costs every k pivots (always done
                              at termination too); 0 = the tuning table's
                              period ("fp32_refresh_period"; the GB300 table
                              has 0: termination only); < 0 = termination
                              only */
  double opt_tol;          /* reduced-cost tolerance; 0 = 1e-9 (FP64) / 1e-5 */
  double piv_tol;          /* pivot tolerance;       0 = 1e-7 (FP64) / 1e-5 */
  const int32_t* basis_hint; /* nullable warm start (host memory for
                                blpg_solve_batch): per LP, m[k] column ids
                                (0..n-1 structural, n..n+m-1 slack), packed in
                                LP order.  The hinted structural columns are
                                pivoted in; the LP is then finished by primal
                                simplex (hinted basis primal feasible), dual
                                simplex (dual feasible) or solved cold from
                                the slack basis (neither).  Ignored for LPs
                                with some b_i < 0. */
  int32_t device;          /* CUDA device ordinal; default 0 */
  int32_t use_graph;       /* 1 (default): replay plan launches as a CUDA graph */
  int32_t threads_per_cta; /* 0 = autotuned per size class */
  int32_t max_cluster;     /* largest cluster (CTAs per LP) allowed; 0 = 8 */
  int32_t min_cluster;     /* smallest cluster used even when one CTA would
                              do (tests of the cluster path); 0 = 1 */
  int32_t cta_smem_budget; /* shared memory per CTA that picks each LP's
                              cluster size; 0 = the tuning table's value,
                              else the whole per-CTA shared memory (the
                              fewest CTAs per LP) */
  int32_t ratio_rule;      /* 0 (default): Harris two-pass ratio test (largest
                              pivot among rows within the feas_tol-relaxed
                              step); 1: textbook minimum ratio.  Bland mode
                              always uses the textbook rule. */
  double feas_tol;         /* Harris relaxation; 0 = 1e-9 (FP64) / 1e-6 */
  int32_t warm_mode;       /* a hinted basis that is primal- and dual-
                              infeasible is finished by: 0 or 1 (default) a
                              cost-shifted dual phase (negative reduced costs
                              raised to small positive values, dual simplex
                              to primal feasibility, true costs restored,
                              primal simplex); 2 a cold solve from the slack
                              basis */
  int32_t pricing;         /* BLPG_PRICE_DANTZIG (0, default): the reference's
                              most negative reduced cost; BLPG_PRICE_STEEPEST:
                              largest d_j^2 / (1 + sum_i T_ij^2), exact column
                              norms summed every pivot (no reference
                              counterpart).  Both fall back to Bland's rule
                              after bland_after degenerate pivots. */
  const float* price_weight; /* nullable, steepest edge only (host memory for
                              blpg_solve_batch): per LP n[k] + m[k] factors
                              multiplying each variable's score (0..n-1
                              structural, n..n+m-1 slack), packed in LP order;
                              the learned warm start passes 1 + p_j, p_j the
                              network's probability that column j is basic */
} blpg_options;

/* Per-LP outputs (host memory for blpg_solve_batch, device memory for
 * blpg_plan_execute).  status and objective are required; the others may be
 * null.  x uses the off_c layout of the batch (n[k] values for LP k) when
 * off_c is given, else packed; basis is packed, m[k] ids per LP. */
typedef struct blpg_result {
  int32_t* status;
  double* objective; /* c^T x of the max problem, as the reference's Result[] */
  double* x;         /* nullable */
  int32_t* pivots;   /* nullable: simplex pivots performed per LP */
  int32_t* basis;    /* nullable: final basic column id of each row */
  int32_t* info;     /* nullable: per-LP BLPG_INFO_* bits */
} blpg_result;

/* Bits of blpg_result.info. */
enum {
  BLPG_INFO_WARM = 1,     /* a basis hint was used */
  BLPG_INFO_FALLBACK = 2, /* cold solve after a hint: the hinted basis was primal- and
                             dual-infeasible, or (FP32) the warm-started solve ended on
                             a basis the FP64 refresh could not verify */
  BLPG_INFO_PARTIAL = 4,  /* some hinted columns found no pivot (singular) */
  BLPG_INFO_DUAL = 8,     /* dual simplex pivots were taken */
  BLPG_INFO_REFRESH = 16, /* FP64 refresh of the FP32 tableau ran */
  BLPG_INFO_REPAIR = 32,  /* an FP64 check found a violation: more pivots */
  BLPG_INFO_SHIFT = 64,   /* hinted basis infeasible both ways: cost-shifted dual phase */
  BLPG_INFO_UNVERIFIED = 128, /* FP32: the FP64 refresh did not converge on the final
                                basis (the FP32 tableau is too inaccurate to check it);
                                the status is BLPG_UNDEF */
  BLPG_INFO_REINVERT = 256,  /* the tableau was rebuilt from an FP64 LU factorisation of
                                its basis: before repair pivots when an FP64 check kept
                                failing, or once in a long or degenerate FP32 solve
                                (plans only) */
  BLPG_INFO_FACTOR = 512,    /* an FP64 refresh factorised the basis (LU) instead of
                                refining through the tableau's B^-1: every phase-I LP,
                                and bases the refinement could not settle (plans only) */
  BLPG_INFO_FP64 = 1024,     /* FP32 plans: the FP32 tableau could not settle this LP
                                (unverified, at its pivot cap 4 (m + n) + 200, or
                                "infeasible" with b >= 0); the plan's FP64 pass solved it
                                from scratch with the FP64 Dantzig method */
  BLPG_INFO_RETRY = 2048,    /* a warm-started solve ended on a basis the FP64 check could
                                not verify and was re-run cold from the slack basis (one that
                                hits the pivot cap is re-run too, with BLPG_INFO_FALLBACK) */
  BLPG_INFO_LOAD = 4096      /* the bulk (TMA) copies loading the LP's tableau did not
                                complete within the kernel's wait limit: status UNDEF, and the
                                CTA that held it stopped taking LPs (never expected; it keeps
                                a stuck copy from hanging the device) */
};

/* Fill *opt with the defaults above. */
void blpg_options_init(blpg_options* opt);

/* Solve a host-resident batch; synchronous.  Replaces Simplex::ComputeLP +
 * getResultAll + getStatusAll (simplex.cu:552-977, :424-461): uploads the
 * batch, solves every LP on the GPU and downloads the results.  Every b must
 * be >= 0 except where the LP is solved by the two-phase path (b_i < 0
 * anywhere in an LP switches that LP to phase I; simplex.cu:574-583). */
int32_t blpg_solve_batch(const blpg_batch* batch, const blpg_options* opt,
                         blpg_result* out);
/* A packed batch (null offset arrays) whose uploads reach 64 MB is solved in
 * eight chunks of LPs with about equal A volume, each with its own plan and
 * stream; the uploads run one chunk after another on one stream, so that
 * each chunk's uploads overlap the previous chunks' solves (simplex.cu:914-955
 * overlaps its copies over N streams the same way).  One
 * whose inputs and outputs exceed half the device's free memory is solved in
 * as many chunks as that budget needs, taking turns in two device regions
 * (the reference's tester splits such batches by device memory on the host,
 * GPU_Tester.cu:194-238).  Results are the same as one plan's.  Tuning-table
 * keys "overlap_mb" and "device_budget_mb" change the two thresholds,
 * "overlap_chunks" the chunk count and "overlap_order" the enqueue order
 * (0: all uploads first from pinned memory, alternating from pageable; 1:
 * always alternating; 2: always uploads first).
 * blpg_solve_batch_chunks returns how many chunks the last call used
 * (1: one plan). */
int32_t blpg_solve_batch_chunks(void);
/* blpg_solve_batch keeps its last plans and device buffers for the next call
 * with the same shapes (grow-only); this frees them (the next call rebuilds
 * what it needs).  Safe to call at any time between solves. */
int32_t blpg_release_workspace(void);

/* Plans: the size classes, work queues, device scratch and CUDA graph for
 * one batch shape, built once and replayed.  blpg_plan_create reads only the
 * shapes (count, m, n, offsets) of a HOST batch; A, b, c may be null.  An
 * FP32 plan whose LPs share A (each element of A read by two LPs or more on
 * average, e.g. one A for the whole batch) also holds an FP32 copy of A (4
 * bytes per element up to the end of the last LP's A), rounded from the
 * executed A at the start of every execute. */
typedef struct blpg_plan blpg_plan;

int32_t blpg_plan_create(const blpg_batch* host_shapes, const blpg_options* opt,
                         blpg_plan** plan);

/* Run a plan on DEVICE-resident data (A, b, c device pointers with the
 * offsets given at plan creation) into DEVICE-resident outputs, enqueued on
 * `stream` (a cudaStream_t; null = the legacy default stream).  Asynchronous:
 * synchronise the stream before reading the outputs.  `basis_hint` (device,
 * nullable) overrides opt->basis_hint for this run. */
int32_t blpg_plan_execute(blpg_plan* plan, const double* dA, const double* db,
                          const double* dc, const int32_t* basis_hint,
                          blpg_result* dev_out, void* stream);
/* blpg_plan_execute with steepest-edge score weights in device memory
 * (n[k] + m[k] floats per LP, packed; see blpg_options.price_weight).  The
 * plan must have been made with pricing = BLPG_PRICE_STEEPEST. */
int32_t blpg_plan_execute_weighted(blpg_plan* plan, const double* dA, const double* db,
                                   const double* dc, const int32_t* basis_hint,
                                   const float* price_weight, blpg_result* dev_out,
                                   void* stream);

/* Number of size classes and, per class, CTAs per LP (cluster size),
 * threads per CTA, dynamic shared memory per CTA and LPs in the class. */
int32_t blpg_plan_num_classes(const blpg_plan* plan);
int32_t blpg_plan_class_info(const blpg_plan* plan, int32_t cls,
                             int32_t* cluster, int32_t* threads,
                             int32_t* smem_bytes, int32_t* num_lps);
/* Residency of size class `cls`: CTAs of it resident per SM and the
 * persistent grid (CTAs) it is launched with. */
int32_t blpg_plan_class_residency(const blpg_plan* plan, int32_t cls,
                                  int32_t* ctas_per_sm, int32_t* grid);
/* Tuning key of size class `cls` (the CTAs per SM its layout admits for a
 * single-CTA class, 100 + K for a class of K-CTA clusters: the "fpXX_cC"
 * entries of blpg_set_tuning) and, when lp_ids is non-null, the ids of its
 * LPs (num_lps of them, blpg_plan_class_info), in the order it solves them. */
int32_t blpg_plan_class_key(const blpg_plan* plan, int32_t cls, int32_t* key,
                            int32_t* lp_ids);
/* Kernel launches one blpg_plan_execute performs. */
int32_t blpg_plan_launches(const blpg_plan* plan);
void blpg_plan_destroy(blpg_plan* plan);

/* Size-class table (JSON text, as written by the autotuner,
 * simplexprojects_gb300/autotune.py): threads per CTA per precision and
 * cluster size ("fp64_k1": 256), per size class ("fp32_c2": 224, the class
 * key of blpg_plan_class_key) with the CTAs per SM it runs with
 * ("fp32_c2_ctas": 2), the per-CTA shared-memory budget ("fp32_smem": bytes)
 * and the cap on CTAs per SM of single-CTA classes ("fp32_ctas": 2; default:
 * as many as shared memory admits, at most 16 in FP32 and 4 in FP64).  The
 * library starts from the table tuned on GB300 that the build compiles in
 * (simplexprojects_gb300/tuning/gb300.json); a table given here replaces it,
 * a null table restores it.  Later plans and blpg_solve_batch calls use it. */
int32_t blpg_set_tuning(const char* json_text);

const char* blpg_last_error(void);
const char* blpg_version(void);

/* Solve without allocating any memory.  No counterpart in the reference (its
 * ComputeLP allocates device memory on every call).  For callers that cannot
 * call cudaMalloc — code running inside a memory pool or arena it does not
 * own, or a host framework that hands all device memory to its own allocator:
 * every input and output is a caller-provided DEVICE pointer, and the kernel's
 * scratch (the work-queue ticket and the LP order it hands out) lives in a
 * fixed array compiled into the library (about 1 MiB, held on every GPU that
 * loads the library until exit).
 *  - count <= 262144 LPs per call (larger counts: BLPG_EINVAL, no GPU work);
 *  - max_m / max_n bound every LP's shape (they size shared memory); offsets
 *    are required (device arrays, as blpg_batch); x (nullable) uses off_c;
 *  - single-phase LPs only: an LP with b_i < 0 or outside the bounds gets
 *    status BLPG_UNDEF and pivots -1;
 *  - the first call on a device does set-up (looks up the scratch address,
 *    sets kernel attributes): make it before any stream capture;
 *  - all calls share the scratch array (each call resets it first), so calls
 *    whose GPU work overlaps race: serialise them;
 *  - asynchronous on `stream`; default tolerances and rules of blpg_options. */
int32_t blpg_solve_noalloc(int32_t count, int32_t max_m, int32_t max_n,
                           const int32_t* d_m, const int32_t* d_n,
                           const int64_t* d_off_A, const int64_t* d_off_b,
                           const int64_t* d_off_c, const double* dA,
                           const double* db, const double* dc,
                           int32_t precision, int32_t* d_status,
                           double* d_objective, double* d_x, int32_t* d_pivots,
                           void* stream);

/* FP64 -> FP32 rounding of FP32 tableaux, over `count` device doubles into
 * device floats, asynchronous on `stream`.  mode 0: the rounding the FP32
 * tableau loaders and the FP32 copy of A use (IEEE round-to-nearest-even,
 * built from integer operations; values below FP32's normal range, |x| <
 * 2^-126, become zero of their sign instead of FP32 subnormals); mode 1:
 * CUDA's __double2float_rn, for comparison.  No reference counterpart (the
 * reference's FP32 kernel, CPLEXvsGLPK/SourceCode/src/simplex.cu, reads
 * float input directly). */
int32_t blpg_round_f32(const double* d_in, float* d_out, int64_t count, int32_t mode,
                       void* stream);

/* Roofline denominators of the pivot kernels, timed on `device` by synthetic
 * kernels: shared-memory bandwidth (GB/s, bytes read + written) and FP64 /
 * FP32 FMA throughput (TFLOP/s, 2 flops per FMA).  No reference counterpart
 * (the reference publishes no performance figures). */
int32_t blpg_measure_peaks(int32_t device, double* smem_gbs, double* fp64_tflops,
                           double* fp32_tflops);

/* ---------------------------------------------------------------------------
 * Learned warm start (no reference counterpart): a multilayer perceptron that
 * scores the n + m columns of an LP for membership in the optimal basis, from
 * the LP's normalised [c; b; family one-hot].  BF16 tensor-core GEMMs with
 * FP32 accumulation, FP32 master weights, Adam.  Dimensions are padded to
 * multiples of 64 (blpg_mlp_dims); batches are multiples of 64 rows.  All
 * data pointers are device pointers; X rows have width d_in_pad, label and
 * logit rows width d_out_pad.
 * ------------------------------------------------------------------------- */
typedef struct blpg_mlp blpg_mlp;

int32_t blpg_mlp_create(int32_t d_in, int32_t hidden, int32_t layers,
                        int32_t d_out, int32_t max_batch, uint64_t seed,
                        blpg_mlp** out);
void blpg_mlp_destroy(blpg_mlp* mlp);
int32_t blpg_mlp_dims(const blpg_mlp* mlp, int32_t* d_in_pad, int32_t* d_out_pad);
int64_t blpg_mlp_num_params(const blpg_mlp* mlp);
/* FP32 master parameters, packed W_1 b_1 ... W_L b_L (W_l: out_pad x in_pad). */
int32_t blpg_mlp_get_params(const blpg_mlp* mlp, float* host_params);
int32_t blpg_mlp_set_params(blpg_mlp* mlp, const float* host_params);
/* One Adam step on a minibatch of B rows (labels 0/1); mean binary
 * cross-entropy sum into *host_loss (nullable). */
int32_t blpg_mlp_train_step(blpg_mlp* mlp, const float* dX, const float* dY,
                            int32_t B, float lr, float* host_loss, void* stream);
/* Logits of B rows (B a multiple of 64; larger than the training batch is
 * fine, it is processed in chunks). */
int32_t blpg_mlp_predict(blpg_mlp* mlp, const float* dX, int32_t B,
                         float* dlogits, void* stream);
/* Forward + backward without an update (gradient checks): packed gradients
 * and the summed loss to host memory. */
int32_t blpg_mlp_gradients(blpg_mlp* mlp, const float* dX, const float* dY,
                           int32_t B, float* host_grads, float* host_loss);
/* Features of `count` LPs with the same m, n: row k of dX (width ldx) is
 * ((c_k, b_k) - mean[f]) / std[f] for the LP's family f = d_family[k]
 * (mean/std: families x (n + m)), then the one-hot of f. */
int32_t blpg_features(int32_t count, int32_t m, int32_t n, int32_t families,
                      const int64_t* d_offb, const int64_t* d_offc,
                      const double* db, const double* dc,
                      const int32_t* d_family, const float* d_mean,
                      const float* d_std, float* dX, int32_t ldx, void* stream);
/* Steepest-edge weights from scores (blpg_options.price_weight): for LP k,
 * d_weight[d_offw[k] + j] = 1 + beta * sigmoid(score[k][j]) over its
 * n[k] + m[k] columns (max_cols the widest, lds >= max_cols). */
int32_t blpg_price_weights(const float* d_scores, int32_t lds, int32_t count,
                           const int32_t* d_m, const int32_t* d_n, int32_t max_cols,
                           const int64_t* d_offw, float beta, float* d_weight,
                           void* stream);
/* Basis hint from scores: for LP k, the m[k] highest-scoring of its
 * n[k] + m[k] columns, in decreasing score order, at d_hint + d_offhint[k]. */
int32_t blpg_topm_hint(const float* d_scores, int32_t lds, int32_t count,
                       const int32_t* d_m, const int32_t* d_n, int32_t max_cols,
                       const int64_t* d_offhint, int32_t* d_hint, void* stream);

/* The learned warm start end to end, for a batch of LPs of one shape (no
 * reference counterpart).  blpg_learned_create takes a trained network
 * (blpg_mlp, not owned: it must outlive the solver), the feature statistics
 * of its training set (HOST arrays, families x (n + m): per family the mean
 * and the standard deviation of each of c_1..c_n, b_1..b_m), the guidance
 * strength beta (weights 1 + beta * p_j) and the batch's shapes and offsets
 * (A, b, c may be null); it builds an FP32 steepest-edge plan (the options'
 * precision and tolerances are kept, pricing is set to steepest edge) and
 * the device buffers.  blpg_learned_solve then takes HOST arrays of that
 * batch (same shapes and offsets) and the family id of each LP, uploads
 * them, runs features -> network -> weights -> solve and downloads status,
 * objective and (when non-null) x, pivots and info; synchronous.  From 512
 * LPs on, b, c and the family ids upload in two halves and each half's
 * features and network run as soon as it has landed, while the rest (then
 * A) uploads.  Pinned host arrays upload fastest. */
typedef struct blpg_learned blpg_learned;
int32_t blpg_learned_create(blpg_mlp* mlp, int32_t families, const float* host_mean,
                            const float* host_std, float beta, const blpg_batch* shapes,
                            const blpg_options* opt, blpg_learned** out);
int32_t blpg_learned_solve(blpg_learned* solver, const blpg_batch* host_batch,
                           const int32_t* host_family, blpg_result* host_out);
void blpg_learned_destroy(blpg_learned* solver);

/* ---------------------------------------------------------------------------
 * Reference batch files and synthetic workloads (host only, no GPU needed).
 * ------------------------------------------------------------------------- */

/* Read the reference's dense A/B/C text files (parseBenchmark.cpp:59-126):
 * A file: first line "m n", then m lines of n numbers; B: m lines; C: n lines.
 * Call once with null A, b, c to get *m and *n, then with buffers of
 * m*n, m and n doubles.  No sign change is applied here: the reference's
 * driver negates c to turn its minimisation files into max form
 * (GPU_Tester.cu:119-127); callers do the same. */
int32_t blpg_read_abc(const char* path_A, const char* path_B,
                      const char* path_C, int32_t* m, int32_t* n, double* A,
                      double* b, double* c);

/* Batch files: a whole batch (shapes, offsets, A, b, c) in one binary file
 * ("BLPGBAT1", little-endian: magic, version, counts, m[], n[], off_A[],
 * off_b[], off_c[], A, b, c; offsets always stored, so LPs that share A keep
 * sharing it).  blpg_read_batch: call once with null arrays to get count
 * and the stored element counts of A, b, c, then with buffers of those
 * sizes (m, n: count int32; offsets: count int64).  blpg_write_results
 * writes one line per LP, "status objective" and, when res->x is set, the
 * LP's n values of x, all doubles as %.17g (exact round trip); path "-" is
 * standard output.  No reference counterpart (the reference reads one LP's
 * A/B/C files and replicates it). */
int32_t blpg_write_batch(const char* path, const blpg_batch* batch);
int32_t blpg_read_batch(const char* path, int64_t* count, int64_t* nA,
                        int64_t* nb, int64_t* nc, int32_t* m, int32_t* n,
                        int64_t* off_A, int64_t* off_b, int64_t* off_c,
                        double* A, double* b, double* c);
int32_t blpg_write_results(const char* path, const blpg_batch* batch,
                           const blpg_result* res);

/* Synthetic workloads.  kind 0..4:
 *  0  m=28, n=32, density 0.6
 *  1  m in {50,56,74,105}, n uniform on [m, 1.8m], density 0.6,
 *     10% unbounded LPs, 5% of rows with b_i = 0
 *  2  m=205, n=203, density 0.15
 *  3  64 base LPs (m=174, n=142, density 0.2), instance k perturbs base
 *     k % 64: c_j *= 1 + N(0, 0.1) (clipped > 0), b_i *= U[0.8, 1.2]
 *  4  m log-uniform on [16, 256], n uniform on [m/2, 2m], density
 *     U[0.1, 0.6]; 5% unbounded, 5% with degenerate rows, 30% from the
 *     kind-3 families
 * A_ij = U[0,1] kept with probability `density`, b_i ~ U[1,10], c_j ~ U[1,5];
 * LP k draws from its own counter stream seeded with seed + k, so any subset
 * of a batch can be regenerated alone (first = index of the first LP).
 * blpg_gen_shapes fills m[count], n[count] (and family[count] if non-null:
 * the base LP of kind-3 instances, -1 otherwise) and returns the total
 * number of A elements; blpg_gen_fill writes packed A, b, c. */
int64_t blpg_gen_shapes(int32_t kind, int64_t first, int32_t count,
                        uint64_t seed, int32_t* m, int32_t* n,
                        int32_t* family);
int32_t blpg_gen_fill(int32_t kind, int64_t first, int32_t count,
                      uint64_t seed, const int32_t* m, const int32_t* n,
                      double* A, double* b, double* c, int32_t threads);

#ifdef __cplusplus
}
#endif

#endif /* BLPG_H_ */
