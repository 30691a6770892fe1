/*
 * CPU oracle for the combinatorial mpQP active-set check.
 *
 * TEST INFRASTRUCTURE ONLY.  The product library never links this code; only
 * the tests, the smoke check and the CPU-baseline leg of bench.py load it, as
 * the checker.
 *
 * It restates, in plain C with a fixed floating-point operation order, the
 * algorithm the reference runs for each candidate active set S:
 *   - LP1 feasibility: min sum_{i in S} w_i over [A -F; 0 At] u + w = [b; bt],
 *     w >= 0, u free (reference main.py:91-98,121; batched_simplex.cu:26-36,
 *     256-316, 901-942, 990-1258); S is feasible when z* <= tol_feas;
 *   - superset pruning: a child is only checked when every subset obtained by
 *     dropping one element was found feasible (batched_simplex.cu:747-766);
 *   - LP2 optimality: max t over the KKT system of S with lambda_S >= t,
 *     inactive slacks >= t, t >= 0 (main.py:103-128;
 *     batched_simplex.cu:635-650, 230-240, 243-254, 1633-1676), after
 *     eliminating x and lambda through the KKT factor;
 *   - critical region rows, normalisation and the Chebyshev-ball LP with the
 *     1e-8 radius test (utils.py:18-97).
 * Q = 0 (an mpLP, README.md:5) runs the same LP1 and the same LP2 verdict
 * (main.py:107 with the Q block zero): the KKT factor is that of A_S A_S^T,
 * x(theta) = A_S^T (A_S A_S^T)^-1 (b_S + F_S theta) and lambda(theta) =
 * -(A_S A_S^T)^-1 A_S (c + H theta); a set with |S| < n keeps a null-space
 * direction of A_S and the stationarity residual in its LP2 (lp2_short_mplp)
 * and is never a region (no unique law x(theta)).
 * Parity of the verdict definitions with the reference's own LP matrices is
 * checked independently (HiGHS on the matrices main.py builds) in the tests.
 */
#ifndef MPQP_ORACLE_H
#define MPQP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n, m, p, ncp;
    const double *Q;   /* n x n, row-major, symmetric positive definite, or all zero (mpLP) */
    const double *c;   /* n */
    const double *H;   /* n x p */
    const double *A;   /* m x n */
    const double *b;   /* m */
    const double *F;   /* m x p */
    const double *At;  /* ncp x p  (CRA) */
    const double *bt;  /* ncp      (CRb) */
} orc_problem;

typedef struct {
    double tol_feas;   /* LP1: feasible when z* <= tol_feas                  */
    double tol_opt;    /* LP2: optimal when t* > tol_opt                     */
    double tol_licq;   /* KKT: Cholesky pivot / diagonal must exceed this   */
    double r_min;      /* Chebyshev: region when r* >= r_min (utils.py:86)  */
    double tol_piv;    /* ratio test: |pivot| must exceed this               */
    double tol_dj;     /* pricing: |reduced cost| must exceed this           */
    int max_pivots;    /* per LP */
    int degen_switch;  /* consecutive degenerate pivots before Bland's rule */
    double tol_zero_row; /* region row counts as zero when max|g| <= this * max(1,|h|) */
} orc_tol;

/* LP status codes (shared with the device code) */
enum { ORC_OPTIMAL = 0, ORC_UNBOUNDED = 1, ORC_ITER_LIMIT = 2, ORC_SKIPPED = 3, ORC_LICQ_FAIL = 4,
       ORC_INFEASIBLE = 5 };
#define ORC_ENOMEM (-5)   /* host memory exhausted */

typedef struct {
    uint64_t mask_lo, mask_hi;
    int32_t level;
    int32_t parent;       /* index of S minus max(S) in the previous level's feasible list */
    int32_t lp1_status, lp1_pivots;
    double z;             /* LP1 optimum */
    int32_t feasible, licq, optimal, region;
    int32_t lp2_status, lp2_pivots, cheb_status, cheb_pivots;
    double t;             /* LP2 optimum (max margin), NaN when not evaluated */
    double r;             /* Chebyshev radius, NaN when not evaluated */
} orc_cand;

typedef struct {
    int64_t n_cand;       /* candidates checked (LP1 verdict given) */
    int64_t n_pruned;     /* children dropped by the subset test */
    int64_t n_feasible, n_optimal, n_region;
    int64_t n_lp1_pivots, n_lp2_pivots, n_cheb_pivots;
    int32_t n_levels;
    int32_t truncated;
    orc_cand *cand;       /* n_cand records, level by level, lexicographic within a level */
} orc_result;

void orc_default_tol(orc_tol *tol);

/* Full level-by-level enumeration for k = 0..k_max.  Optimality is evaluated
 * for levels >= k_min; lower levels are still enumerated for pruning.
 * budget > 0: a level is checked only when the candidates checked so far
 * plus the whole level fit in the budget; otherwise the enumeration stops
 * there (out->truncated = 1).  exhaustive = 1: every combination is a
 * candidate (children of all candidates, no subset test).
 * nthreads <= 1 runs serially.  The LP1 tableaus of a level are computed in
 * chunks of ORC_CHUNK candidates; only children that become parents of the
 * next level are kept (none at k_max unless exhaustive), so host memory
 * grows with the feasible sets, not with the candidates.
 * Returns 0 on success, negative on error (ORC_ENOMEM: out of memory). */
int orc_enumerate(const orc_problem *pr, const orc_tol *tol, int k_min, int k_max,
                  int64_t budget, int exhaustive, int nthreads, int keep_records, orc_result *out);
void orc_free_result(orc_result *res);

/* The same enumeration restricted to the active sets whose elements are all
 * >= j_first (no records).  Those sets are closed under taking subsets, so
 * every candidate, its subset test, warm-start chain and LPs are exactly the
 * full enumeration's: a sample of the full workload with all its levels,
 * used to time the CPU baseline on a bounded share of a large instance. */
int orc_enumerate_tail(const orc_problem *pr, const orc_tol *tol, int k_min, int k_max, int64_t budget,
                       int nthreads, int j_first, orc_result *out);

/* Check one sorted active set S (|S| = k) by replaying the warm-start chain
 * {} -> {s0} -> {s0,s1} -> ... exactly as the enumeration does.  Fills *rec.
 * When laws is non-NULL and S is a region it receives, row-major,
 *   lagrange_A (k x p), lagrange_b (k), parameter_A (n x p), parameter_b (n).
 * cr_rows (optional, capacity (m+ncp) x (p+1)) receives the normalised region
 * rows [CR_As | CR_bs] in the reference's order; *n_cr_rows their count. */
int orc_check_set(const orc_problem *pr, const orc_tol *tol, const int *S, int k,
                  orc_cand *rec, double *laws, double *cr_rows, int *n_cr_rows);

/* Precomputed KKT data, exposed for tests: Wm (m x m), Wh (m x p), wc (m). */
/* Dual certificate of LP1 infeasibility: replays S's warm-start chain up to its
 * first infeasible prefix (k_used elements) and builds the dual y of that
 * final basis (y_i = 1 on the prefix's basic slacks, the nonbasic slacks' duals
 * from G_N^T y_N = -G_B^T c_B).  Returns 1 with *bound = beta.y <= z* when
 * y <= c + sign_tol holds, 0 when the basis gives no such y, < 0 on bad input.
 * *z_out: the LP1 value of that prefix. */
int orc_lp1_dual_bound(const orc_problem *pr, const orc_tol *tol, const int *S, int k, double sign_tol,
                       double *bound, double *z_out, int *k_used);
int orc_kkt_data(const orc_problem *pr, double *Wm, double *Wh, double *wc);

#ifdef __cplusplus
}
#endif
#endif
