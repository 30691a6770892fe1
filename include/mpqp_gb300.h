/*
 * mpqp_gb300 -- combinatorial mpQP active-set check on one GB300 (sm_103a).
 *
 * C ABI of libmpqp_gb300.so.  The first block is a drop-in for the library
 * the reference loads through ctypes (mpqp_cuda.so): same symbol names, same
 * argument order and meaning, same result structure prefix.  The second block
 * is this library's native interface (many instances in one launch, mixed
 * precision, device-resident plans for timing).
 *
 * Threading: one call at a time per process (the reference's driver calls
 * it from a single Python thread).  All entry points return an error code or
 * a NULL pointer instead of terminating the process.
 */
#ifndef MPQP_GB300_H
#define MPQP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Drop-in boundary (reference: main.py:12-50, 60, 144)                 */
/* ------------------------------------------------------------------ */

/* Result of mpqp().  The first eight fields are the reference's
 * GPUResults (main.py:12-22); the rest are appended, so a caller that maps
 * only the prefix keeps working.
 *   n_batches        number of enumeration levels that were run
 *   n_splits         1 + the levels that did not fit device memory whole:
 *                    the LP1 tableaus of their feasible sets are kept while
 *                    the arena has room, and the children of the others
 *                    start LP1 from the root tableau (the reference splits
 *                    such a level into n_splits chunks, batched_simplex.cu:
 *                    1141-1158; verdicts are the same either way)
 *   n_feasible_lps   candidate active sets found feasible (LP1)
 *   n_final_lps      candidate active sets found optimal (LP2); their sets
 *                    are in active_sets, row-major n_final_lps x n_x,
 *                    ascending indices, unused entries -1 (utils.py:105-116)
 *   time_feas        seconds in the enumeration and LP1 kernels (events
 *                    around each launch)
 *   time_opti        seconds in the optimality kernels
 *   time_GPU         seconds of device time for the whole call
 * mpqp() runs in mixed precision (FP32 pivots, every verdict certified or
 * re-solved in FP64; the same sets as the FP64 path); the environment
 * variable MPQP_PRECISION=fp64 selects the plain FP64 kernels.
 * The structure and its arrays stay valid until mpqp_free() or the next
 * mpqp() call, whichever comes first. */
typedef struct GPUResults {
    int n_batches;
    int n_splits;
    int n_feasible_lps;
    int n_final_lps;
    double time_feas;
    double time_opti;
    double time_GPU;
    int *active_sets;
    /* appended */
    int status;              /* 0 on success, else an MPQP_E* code         */
    int n_regions;           /* optimal sets whose Chebyshev radius >= 1e-8 */
    long long n_candidates;  /* candidate active sets checked               */
    long long n_pruned;      /* children dropped by the subset test         */
    double *t_star;          /* n_final_lps: LP2 optimum (max margin)       */
    double *radius;          /* n_final_lps: Chebyshev radius               */
    int *is_region;          /* n_final_lps: 1 when radius >= 1e-8          */
    double *law_error;       /* n_final_lps: stated relative error of the
                                set's affine laws (see mpqp_opt_set.err)   */
} GPUResults;

/* Replaces mpqp_cuda.so:mpqp (called at main.py:144, argtypes main.py:28-50).
 * AxT      n_x x n_c column-major (= A^T, main.py:100,130)
 * A1, xb1  LP1 standard form, M1 x N1 column-major and M1 (main.py:91-98)
 * b1       LP1 initial basis (main.py:121)
 * A2, xb2  LP2 standard form, M2 x N2 column-major and M2 (main.py:102-118)
 * b2, non_b2  LP2 initial basis / non-basis (main.py:123-128)
 * k_min, k_max  cardinality range of the active sets to report
 * extra_batches  accepted for compatibility (levels split by themselves)
 * reserved_memory  MiB left free on the device when the call sizes its
 *          buffers (the environment variable MPQP_ARENA_BYTES caps the LP1
 *          tableau arena in bytes).
 * The problem data are read back from A1/xb1/A2/xb2; the LP layouts are
 * validated and a malformed input returns a result with status != 0.  Every
 * failure is such a result; NULL only when the host cannot allocate even
 * that. */
GPUResults *mpqp(const double *AxT, int n_c, int n_x, int n_t, int k_min, int k_max, int extra_batches,
                 const double *A1, const double *xb1, const int *b1, int M1, int N1,
                 const double *A2, const double *xb2, const int *b2, const int *non_b2, int M2, int N2,
                 int n_eqs, int reserved_memory);

/* Replaces mpqp_cuda.so:warm_up (main.py:60): creates the CUDA context,
 * loads the kernels and runs one tiny problem. */
void warm_up(void);

/* Releases a result of mpqp() (the reference never frees; this is optional). */
void mpqp_free(GPUResults *res);

/* The problem mpqp() reads back from the reference's LP matrices, without
 * touching the GPU: Q (n_x^2), c (n_x), H (n_x*n_t), A (n_c*n_x), b (n_c),
 * F (n_c*n_t), At (n_cp*n_t), bt (n_cp), row-major; *n_cp = M1 - n_c.
 * Pass NULL for outputs you do not need.  Returns MPQP_OK or MPQP_ELAYOUT. */
int mpqp_unpack_lp(const double *AxT, int n_c, int n_x, int n_t, const double *A1, const double *xb1, int M1,
                   int N1, const double *A2, const double *xb2, int M2, int N2, int n_eqs, double *Q, double *c,
                   double *H, double *A, double *b, double *F, double *At, double *bt, int *n_cp);

/* ------------------------------------------------------------------ */
/* Native interface                                                      */
/* ------------------------------------------------------------------ */

enum {
    MPQP_OK = 0,
    MPQP_EINVAL = -1,      /* bad sizes or pointers                        */
    MPQP_ENOTSPD = -2,     /* Q is neither positive definite nor zero      */
    MPQP_EORIGIN = -3,     /* b < 0 or CRb < 0: the origin is infeasible   */
    MPQP_ELAYOUT = -4,     /* LP matrices do not have the reference layout */
    MPQP_ECUDA = -5,       /* CUDA runtime error                           */
    MPQP_ECAPACITY = -6,   /* a device buffer overflowed                   */
    MPQP_ENOMEM = -7       /* device (or host) allocation failed           */
};

enum { MPQP_FP64 = 0, MPQP_MIXED = 1 };

/* One mpQP instance: min 1/2 x'Qx + (c + H theta)'x  s.t.  A x <= b + F theta,
 * At theta <= bt.  Row-major host arrays.  Q positive definite, or Q = 0
 * exactly: a multiparametric LP (the reference's README.md:5 names mpLP;
 * its LP2 of main.py:102-108 keeps x, so Q = 0 needs no Q^-1).  For an
 * mpLP the KKT factor is that of A_S A_S^T, a set with |S| < n keeps a
 * null-space direction and the stationarity residual in its LP2 and is
 * never a region (x(theta) is not unique); limits: m + ncp + 3n + p <= 252. */
typedef struct {
    int n, m, p, ncp;
    int k_min, k_max;        /* cardinalities to check (k_max <= min(n, m))  */
    long long budget;        /* max candidates checked (0 = no limit)       */
    const double *Q, *c, *H, *A, *b, *F, *At, *bt;
} mpqp_problem;

typedef struct {
    int precision;           /* MPQP_FP64 or MPQP_MIXED                     */
    int exhaustive;          /* 1: every combination is a candidate          */
    int record;              /* 1: keep one record per checked candidate    */
    int use_graph;           /* 1: capture the level loop in a CUDA graph   */
    long long cand_cap;      /* candidates per level (0: derived)           */
    long long node_cap;      /* nodes per level (0: = cand_cap)             */
    long long arena_bytes;   /* tableau arena (0: derived)                  */
    long long rec_cap;       /* records (record = 1)                        */
    long long opt_cap;       /* optimal-set records (0: derived)            */
    double mem_fraction;     /* of free device memory used when derived     */
    /* tolerances (0 selects the default) */
    double tol_feas, tol_opt, tol_licq, r_min, tol_piv, tol_dj;
    int max_pivots, degen_switch;
    /* margin_z: an FP32 LP1 optimum that is not certified feasible goes to the
     * FP64 dual certificate when its z exceeds margin_z, else straight to the
     * FP64 re-solve (routing only: no verdict rests on it) */
    double tol_piv32, tol_dj32, margin_z, margin_beta, margin_t, margin_licq;
    double tol_zero_row;     /* region row zero when max|g| <= tol * max(1,|h|) */
    int lp2_screen;          /* MPQP_MIXED, FP32 optimality screen: 0 the dual
                                bound on instances whose parameter set is a
                                box (the primal tableau screen elsewhere),
                                1 the primal tableau screen everywhere      */
    /* Launch settings (0: the default, or the autotuner's choice):
     *   tile_w      threads per LP in the first stage of the FP32 screen
     *               (8, 16 or 32: 4, 2 or 1 LPs per warp)
     *   feas_warps  warps (one LP each) per LP1 block, 1..4
     *   feas_chunk  consecutive candidates an LP1 warp claims, 1..32
     * autotune = 1: settings left at 0 are chosen by timing the candidate
     * settings on a short slice of the batch (each instance under a small
     * candidate budget) when the plan is created; the choice is kept per
     * batch shape (precision, screen mode, rows, free variables, parameters,
     * instance count) for the rest of the process.  Any setting gives the
     * same verdicts. */
    int tile_w, feas_warps, feas_chunk;
    int autotune;
    /* lp2_warm = 1 (MPQP_MIXED): LP2 basis sharing, the reference's
     * copy_basis_dual_1/2 (batched_simplex.cu:525-590).  The first stage of
     * the dual screen starts each set's LP from its parent set's final basis
     * (S minus its largest element), inverted on the device; a singular or
     * infeasible basis falls back to the usual single-row start.  Off by
     * default: slower on the measured workloads (the verdicts are the same
     * either way). */
    int lp2_warm;
} mpqp_options;

/* One optimal active set */
typedef struct {
    uint64_t mask_lo, mask_hi;   /* bit i set: constraint i is active        */
    int inst, level;
    double t;                    /* LP2 optimum                              */
    double r;                    /* Chebyshev radius                         */
    int region, fp64;
    long long rec;
    /* The error stated for this result: the size of one FP64 iterative-
     * refinement step of the KKT solve (residual of Wm[S,S] Lambda =
     * [Wh_S | wc_S] solved with the same factor) relative to the largest
     * entry of Lambda -- an estimate of the relative forward error of the
     * multiplier law lambda(theta) and of the primal law x(theta), which is
     * linear in it.  The laws themselves are the unrefined FP64 values (the
     * oracle's operations); t and r are FP64 LP optima. */
    double err;
} mpqp_opt_set;

/* Per-instance counters */
typedef struct {
    long long candidates, pruned, feasible, optimal, regions;
    long long lp1_pivots, lp2_pivots, cheb_pivots, fallback_lp1, fallback_opt;
    long long stored;             /* LP1 tableaus kept for warm starts      */
    /* order-independent digests of the feasible / optimal / region sets:
     * sum mod 2^64 of a 64-bit hash of each set's mask (equal digests =
     * equal sets, up to hash collisions) */
    unsigned long long feasible_digest, optimal_digest, region_digest;
    int last_level, truncated;
    /* mixed precision: FP32 LP1 optima proven infeasible by the FP64 dual
     * certificate of their final basis, those it could not prove (re-solved
     * in FP64; fallback_lp1 counts every re-solve), and of those the ones
     * with a free variable nonbasic in the final basis */
    long long lp1_certified, lp1_cert_missed, lp1_cert_freevar;
    /* LP1 traffic model (bytes a launch must move, each item once): the
     * distinct parents whose children were checked (count, and the bytes of
     * their live tableau rows, basis ids and node records) and the stored
     * child tableaus with their ids */
    long long lp1_parents, lp1_parent_bytes, lp1_store_bytes;
    /* LP1 solves started from the root tableau because the parent's tableau
     * did not fit the arena, and the feasible sets kept without a tableau */
    long long lp1_cold, nodes_without_tableau;
    /* the first stage of the dual screen (mixed precision): LPs run and
     * their iterations; with lp2_warm, the LPs offered a valid parent basis
     * and those that started from it */
    long long lp2_first_stage_lps, lp2_first_stage_pivots, lp2_warm_offered, lp2_warm_started;
    /* mixed precision: sets found not optimal in FP64 from the final basis
     * of the FP32 dual screen, without the FP64 LP2 (counted in fallback_opt) */
    long long lp2_certified;
    /* mixed precision: last-level FP32 LP1 optima whose smallest basic slack
     * lay inside the FP32 margin, found feasible by the FP64 vertex check of
     * their final basis (no FP64 re-solve) */
    long long lp1_vertex_checked;
} mpqp_inst_stats;

typedef struct {
    int status;
    int n_inst;
    int n_levels;
    int overflow;                 /* MPQP_ECAPACITY detail bits             */
    double device_ms;             /* events around the device work          */
    mpqp_inst_stats *inst;        /* n_inst                                 */
    long long n_opt;
    mpqp_opt_set *opt;            /* n_opt, ordered by instance, then |S|,
                                     then the ascending element lists of S
                                     (lexicographic); the same order on
                                     every run                               */
    long long n_rec;
    void *rec;                    /* n_rec records (112 bytes each) or NULL */
    long long h2d_bytes;          /* problem data uploaded by the plan      */
    long long d2h_bytes;          /* result bytes copied back               */
    int tile_w, feas_warps, feas_chunk; /* the launch settings of the run    */
    int tuned;                    /* 1: chosen by the autotuner             */
    int split_levels;             /* levels whose feasible sets did not all
                                     keep an LP1 tableau (arena full)       */
    int pad_;
} mpqp_batch_result;

void mpqp_default_options(mpqp_options *opt);

/* Solve a batch of independent instances in one launch sequence. */
int mpqp_solve_batch(int n_inst, const mpqp_problem *probs, const mpqp_options *opt, mpqp_batch_result **out);
void mpqp_batch_free(mpqp_batch_result *res);

/* Device-resident plans: upload once, run many times (timing). */
typedef struct mpqp_plan mpqp_plan;
int mpqp_plan_create(int n_inst, const mpqp_problem *probs, const mpqp_options *opt, mpqp_plan **out);
/* Enqueue one full enumeration on `stream` (a cudaStream_t, NULL = default). */
int mpqp_plan_run(mpqp_plan *plan, void *stream);
/* Copy the results of the last run to the host (synchronises the stream). */
int mpqp_plan_results(mpqp_plan *plan, mpqp_batch_result **out);
/* Number of kernel launches one run enqueues. */
int mpqp_plan_launches(const mpqp_plan *plan);
/* Like mpqp_plan_run, without the graph and with a CUDA event before every
 * launch; mpqp_plan_kernel_times then returns, per kernel name (64-byte
 * slots), the summed milliseconds and the launch count.  Returns the number
 * of distinct kernels (or an error code). */
int mpqp_plan_run_timed(mpqp_plan *plan, void *stream);
int mpqp_plan_kernel_times(mpqp_plan *plan, int max_kernels, char *names, double *ms, int *count);
void mpqp_plan_destroy(mpqp_plan *plan);

/* Plans take their device memory from a pool (one per device) that keeps
 * freed memory for the next plan, so destroying a plan is cheap; the pool's
 * idle memory counts as free when a plan sizes its buffers.  This returns the
 * idle memory of the current device's pool to the driver.  No counterpart in
 * the reference (its buffers live inside each mpqp() call). */
int mpqp_release_cached_memory(void);

/* Region laws of optimal sets, computed in FP64 on the device:
 *   lagrange_A (k x p), lagrange_b (k), parameter_A (n x p), parameter_b (n),
 *   CR rows (n_cr x (p+1)): [CR_As | CR_bs] normalised, reference order.
 * Sizes per set are written to `sizes` (4 ints: k, n, p, n_cr; k = -1 when
 * the set fails the LICQ test, k = -2 for an mpLP set with |S| < n, whose
 * law is not unique -- nothing else is written for those); `laws` must
 * hold n_sets * (mmax*(p+1) + n*(p+1) + (m+ncp)*(p+1)) doubles (see
 * mpqp_region_laws_stride). */
long long mpqp_region_laws_stride(const mpqp_problem *prob);
int mpqp_region_laws(const mpqp_problem *prob, long long n_sets, const uint64_t *masks /* 2 per set */,
                     double *laws, int *sizes);

/* Replaces compute_critical_region (utils.py:23-97) for a list of active
 * sets: mpqp_region_laws plus each set's Chebyshev radius (radius: n_sets
 * doubles; NaN when the set fails the LICQ test or has no unique law).  A
 * set is a critical region when radius >= 1e-8 (utils.py:86), so a caller
 * needs no enumeration to filter the sets it holds. */
int mpqp_critical_regions(const mpqp_problem *prob, long long n_sets, const uint64_t *masks, double *laws,
                          int *sizes, double *radius, double *err /* n_sets, may be NULL: the stated law error */);

/* Region laws without any device allocation.  No counterpart in the
 * reference: its region laws are computed on the host (utils.py:23-97).
 * For callers that may not call cudaMalloc -- a control loop past its
 * start-up, where an allocation can stall or fail, or a host application
 * that owns the device memory through its own allocator.  Same results as
 * mpqp_region_laws, but `masks` (2 per set) stays on the host while `laws`
 * (n_sets * mpqp_region_laws_stride doubles) and `sizes` (4 ints per set)
 * are device buffers the caller allocated.  The work is queued on `stream`
 * (a cudaStream_t, NULL = default stream); synchronise it before reading.
 * Scratch: a fixed MPQP_NOALLOC_SCRATCH_BYTES (1 MiB) device array holds the
 * instance's FP64 KKT blocks plus 16 bytes per set; larger calls return
 * MPQP_ECAPACITY.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress).  Calls may not be captured into a CUDA
 * graph (the data are staged through one host buffer that every call
 * rewrites): a call on a stream that is being captured returns MPQP_EINVAL.
 * All calls share the array: calls whose work overlaps on the GPU race.
 * Inputs are checked as mpqp_region_laws checks them (same codes), plus
 * n <= 32. */
#define MPQP_NOALLOC_SCRATCH_BYTES (1 << 20)
int mpqp_region_laws_noalloc(const mpqp_problem *prob, long long n_sets, const uint64_t *masks, double *laws,
                             int *sizes, void *stream);

/* Constraint reduction before the enumeration.  Replaces the ppopt steps of
 * MPQPProb.process_constraints (utils.py:163-190: process_program_constraints,
 * find_implicit_equalities, find_redundant_constraints of ppopt 1.5.1) on the
 * rows of [A -F; 0 At] u <= [b; bt], u = (x, theta):
 *   1. a row whose x- and theta-parts are zero is dropped (MPQP_ROW_ZERO);
 *   2. rows are compared after dividing each by the 2-norm of its [A -F]
 *      (or At) part; a row equal to an earlier one of the same block, within
 *      a squared distance of 1e-16, is dropped (MPQP_ROW_DUPLICATE);
 *   3. a row of A that is the negation of an earlier one (b included) is
 *      dropped (MPQP_ROW_EQUALITY_PAIR) and the earlier one is kept as an
 *      implicit equality (MPQP_ROW_EQUALITY);
 *   4. every other row is redundant (MPQP_ROW_REDUNDANT) when max a_i u over
 *      all remaining rows, row i relaxed by 1, is at most its right-hand side
 *      + 1e-9 (normalised rows): one FP64 LP per row on the device, all rows
 *      against the same row set.
 * row_status: m + ncp ints, A's rows then At's rows.  Requires b >= 0 and
 * bt >= 0 (the origin feasible), m + ncp + n + p <= 255. */
#define MPQP_ROW_KEPT 0
#define MPQP_ROW_ZERO 1
#define MPQP_ROW_DUPLICATE 2
#define MPQP_ROW_EQUALITY_PAIR 3
#define MPQP_ROW_REDUNDANT 4
#define MPQP_ROW_EQUALITY 5
int mpqp_reduce_constraints(const mpqp_problem *prob, int *row_status);

const char *mpqp_version(void);
/* The text of the last error of the calling thread. */
const char *mpqp_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
