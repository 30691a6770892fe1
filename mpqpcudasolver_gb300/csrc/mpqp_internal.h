// Internal types shared by the device kernels and the host engine.
//
// Layout in HBM (one solve = one batch of independent mpQP instances):
//   InstDesc[n_inst]           per-instance sizes, limits and offsets
//   dbl pool                   per-instance FP64 data (KKT blocks, boxes,
//                              laws data, LP1 root tableau)
//   flt pool                   FP32 copies of the KKT blocks, boxes and root
//   node arrays x2             feasible active sets of the previous / current
//                              level (ping-pong), 32 B each
//   tableau arena x2           LP1 final tableaus of those sets (bump
//                              allocated, per-instance size), + basis ids
//   mask hash x2               tagged open-addressing table of feasible masks
//   candidate list             (parent node, added constraint) pairs, 8 B
//   fallback queues            candidates / nodes re-solved in FP64
//   certificate queue          FP32 LP1 optima to certify infeasible in FP64
//                              (candidate index + final nonbasic ids)
//   optimal-set list           one OptRec per optimal active set
//   records (optional)         one CandRec per checked candidate (parity)
#pragma once
#include <stdint.h>

namespace mq {

constexpr int kMaxM = 128;        // constraints per instance (128-bit masks)
constexpr int kMaxIds = 255;      // ids are uint8
constexpr int kMaxK = 32;         // largest active-set cardinality supported
constexpr int kMaxP = 30;         // parameters

// LP_INFEASIBLE: an mpLP set with |S| < n whose stationarity residual cannot
// vanish inside the parameter set (its LP2 has no feasible point)
enum LpStatus : int { LP_OPTIMAL = 0, LP_UNBOUNDED = 1, LP_ITER_LIMIT = 2, LP_SKIPPED = 3, LP_LICQ_FAIL = 4,
                      LP_INFEASIBLE = 5 };

enum Precision : int { PREC_FP64 = 0, PREC_MIXED = 1 };

struct Tol {
    double tol_feas;    // LP1 feasible when z* <= tol_feas
    double tol_opt;     // LP2 optimal when t* > tol_opt
    double tol_licq;    // Cholesky pivot must exceed tol_licq * diagonal
    double r_min;       // Chebyshev radius threshold (region when r >= r_min)
    double tol_piv;     // FP64 ratio-test pivot threshold
    double tol_dj;      // FP64 pricing threshold
    int max_pivots;
    int degen_switch;
    // mixed precision: FP32 thresholds and the margins that send a
    // candidate to the FP64 re-solve
    float tol_piv32;
    float tol_dj32;
    double margin_z;    // FP32 LP1 z above this -> the FP64 dual certificate, else the FP64 re-solve (routing only)
    double margin_beta; // FP32 basic slacks above margin_beta * max(1, tableau growth) certify feasibility
    double margin_t;    // FP32 LP2 t below -margin_t * error scale -> not optimal without FP64
    double margin_licq; // FP32 Cholesky pivot ratio below this -> FP64
    double tol_zero_row;// region row is zero when max|g| <= tol_zero_row * max(1, |h|)
    // FP32 copies of the margins: the FP32 kernels decide without FP64
    // arithmetic (GB300's FP64 pipe is a small fraction of its FP32 rate)
    float margin_z32, margin_beta32, margin_t32, margin_licq32;
};

struct InstDesc {
    int n, m, p, ncp;
    int M1, nv;                 // LP1 rows, LP1 free variables
    int ld1, ld2;               // strides of the plan's LP1 / LP2 tableaus (FP32: = 4 mod 8, FP64: odd)
    int ld1d, ld2d;             // strides of the FP64 re-solve tableaus (odd)
    int k_min, k_max;
    int tab_elems;              // (M1+1)*ld1 rounded up to a multiple of 4
    int ids_bytes;              // M1 + nv rounded up to 16
    long long budget;           // max candidates checked for this instance (0 = no limit)
    // offsets (elements) into the FP64 pool.  mpLP (Q = 0): Wm = A A^T,
    // Wh = F, wc = b, QiAT = A^T, QiH = Qic = 0, and WhL = A H, wcL = A c,
    // Hm = H, cv = c (the multiplier law and the stationarity residual)
    long long o_Wm, o_Wh, o_wc, o_At, o_bt, o_QiAT, o_QiH, o_Qic, o_root;
    long long o_WhL, o_wcL, o_Hm, o_cv;
    // offsets (elements) into the FP32 pool
    long long f_Wm, f_Wh, f_wc, f_At, f_bt, f_root;
    long long f_blo, f_bhi;     // parameter box lo <= theta <= hi (FP32), valid when box
    // mpLP only (else -1): FP32 copies of A H, A c (the multiplier law) and of
    // A^T (n x m), H, c (the stationarity residual)
    long long f_WhL, f_wcL, f_AT, f_Hm, f_cv;
    int box;                    // 1: At = [diag(+); diag(-)] (rows c, then p + c), a box
    int lp;                     // 1: Q = 0 (mpLP)
    int ld2lp;                  // mpLP, |S| < n: FP64 LP2 row stride (>= p + n + 3, odd)
    int root_rows;              // live rows of the FP32 LP1 root (its basis ids follow it in the
                                // FP32 pool at f_root + tab_elems: bid over M1, then nid over nv)
};

struct Node {                   // a feasible (or, when exhaustive, any) active set
    uint64_t lo, hi;            // 128-bit mask
    int inst;
    int flags;                  // NodeFlags
    long long tab_off;          // element offset into the tableau arena (-1: none)
    long long ids_off;          // byte offset into the ids arena
    long long rec;              // record index (or -1)
};

// NODE_CERT: the stored FP32 tableau is the one whose basic solution
// certified this set feasible (every slack of the set nonbasic, every basic
// slack clear of the growth-scaled margin).
enum NodeFlags : int { NODE_FEASIBLE = 1, NODE_VALID = 2, NODE_CERT = 8 };
// bits 8..16 of the flags: 1 + the live rows of the stored FP32 LP1 tableau
// (rows of basic free variables dropped, the objective row right after them);
// 0: all M1 rows
constexpr int kNodeRowsShift = 8;
// bits 17..24: 1 + the live columns of the stored FP32 LP1 tableau (the
// columns of the set's own nonbasic slacks, fixed at zero for every
// descendant, moved past the right-hand side); 0: all nv columns
constexpr int kNodeColsShift = 17;

struct Cand { int parent; int j; };

struct OptRec {
    uint64_t lo, hi;
    int inst, level;
    double t, r;
    int region;
    int fp64;                   // verdict decided by the FP64 kernels
    long long rec;
    double err;                 // estimated relative error of the set's law (FP64 refinement step)
};

struct CandRec {                // identical field layout to the oracle's record
    uint64_t mask_lo, mask_hi;
    int32_t level, parent;
    int32_t lp1_status, lp1_pivots;
    double z;
    int32_t feasible, licq, optimal, region;
    int32_t lp2_status, lp2_pivots, cheb_status, cheb_pivots;
    double t, r;
    int32_t inst, fp64;         // instance; bit0 LP1 / bit1 LP2 decided in FP64, bit2 LP1
                                // infeasible by the FP64 dual certificate of the final FP32 basis,
                                // bit3 LP2 not optimal by the FP64 check of the FP32 dual basis,
                                // bit4 LP1 feasible by the FP64 vertex check of the final FP32 basis
    float lp1_growth;           // FP32 LP1: max |T_ij| of the final tableau (mixed precision)
    float lp1_minbeta;          // FP32 LP1: smallest basic slack value
    double lp1_bound;           // FP64 dual certificate: the lower bound on z* it proved (NaN: none)
};

// w = (tag << 40) | bits 24..63 of the set's 64-bit hash; tag = a function
// of the run's epoch (drawn from one counter per device) and the level, never
// 0.  An entry matches only the run and level that wrote it, so a plan's hash
// memory (from the pool, possibly an earlier plan's) needs no clearing.
struct HashSlot { unsigned long long w; };

// Per-instance level bookkeeping
struct InstCtl {
    long long lvl_cand;         // candidates generated at the current level
    long long cum_cand;         // candidates checked before the current level
    long long pruned;           // children dropped by the subset test
    long long feasible, optimal, region;
    long long lp1_piv, lp2_piv, cheb_piv;
    long long fb_lp1, fb_opt;   // FP64 fallbacks (mixed precision)
    long long cert_lp1;         // FP32 LP1 optima certified infeasible by the FP64 dual bound
    long long cert_miss;        // ... that the certificate could not prove (sent to the FP64 re-solve)
    long long cert_free;        // ... of those, the misses with a free variable nonbasic (no square system)
    long long cert_lp2;         // sets found not optimal by the FP64 check of their FP32 dual basis
    long long vtx_lp1;          // last-level LP1 optima found feasible by the FP64 vertex check
    long long lp1_cold;         // LP1 solves started from the root (the parent kept no tableau)
    long long no_tab;           // nodes kept without a tableau (the arena was full)
    long long stored;           // LP1 tableaus written for the next level
    // LP1 bytes for the roofline: the distinct parents of each checked level
    // (live tableau rows, basis ids and node, each parent once) and the
    // stored children (their live rows and ids); lvl_*: the current level,
    // added when the level is checked (within the budget)
    long long lvl_parents, parents, lvl_par_bytes, par_bytes, store_bytes;
    // first stage of the dual screen: LPs run and their iterations; with
    // LP2 basis sharing, the LPs offered the parent's final basis and those
    // that started from it
    long long s0_lps, s0_piv, warm_try, warm_used;
    // order-independent digests (sum mod 2^64 of a 64-bit hash of each mask)
    unsigned long long feas_digest, opt_digest, reg_digest;
    int stopped;                // budget exhausted or max level reached
    int truncated;              // stopped by the budget
    int last_level;
    int pad;
};

constexpr int kCtlCounters = 13;

// levels whose sets have at most this many elements run the first stage of
// the FP32 dual screen with one set per thread (k_opt_screen_lanes)
constexpr int kLaneMaxK = 6;

struct Ctl {
    long long n_cand;           // candidates at the current level
    long long n_node[2];        // nodes per ping-pong side
    long long tab_used[2];      // elements used per tableau arena
    long long ids_used[2];      // bytes used per ids arena
    long long n_opt;            // optimal sets found so far
    long long n_rec;            // records written so far
    long long rec_base;         // record index of the current level's first candidate
    long long n_q_lp1, n_q_opt; // FP64 fallback queue lengths
    long long n_q_scr;          // sets the first stage of the dual screen left to its second
    long long n_q_cert;         // FP32 LP1 optima waiting for the FP64 dual certificate
    long long n_q_s0;           // first-stage dual LPs cut off at the first pass's cap, run again
    long long n_q_s1;           // ... and those cut off again at the second pass's cap
    long long n_q_c2;           // sets for the FP64 kernel with an FP32 dual basis to check first
    unsigned long long ctr[kCtlCounters];  // work counters (reset every level)
    int overflow;               // bit mask of overflowed buffers
    int level;
    int epoch;                  // this run's number from the device's counter (hash tags)
    int pad;
    long long hcap[2];          // slots of the hash in use per side (a power of 2 <= hash_cap)
    // 1 once a side's tableau (or ids) arena had no room for a reservation:
    // later nodes of that level keep no tableau, and their children start
    // LP1 from the root tableau (the arena's overflow is not an error)
    int tab_full[2];
    long long split_levels;     // levels whose parents did not all keep a tableau
};

// OV_WAIT: a bounded wait for a bulk copy ran out (the launch's results are void)
enum Overflow : int { OV_CAND = 1, OV_NODE = 2, OV_TAB = 4, OV_IDS = 8, OV_OPT = 16, OV_REC = 32, OV_QUEUE = 64, OV_HASH = 128,
                      OV_WAIT = 256 };

// Largest per-warp shared-memory footprint over the instances of a batch
struct SlotDims {
    int maxM1, maxLD1, maxNv;       // LP1 tableau
    int maxK, maxP1, maxR2, maxLD2; // KKT factor and LP2 / Chebyshev tableau
    int maxLD1d, maxLD2d;           // strides of the FP64 re-solve tableaus
    int maxR2d;                     // rows of the FP64 LP2 tableau (mpLP, |S| < n: m + ncp + 2n + 1)
    int maxN;                       // mpLP instances: largest n (0: none), sizes Psi and Phi
};

struct DevBuffers {
    const InstDesc *inst;
    int n_inst;
    const double *dpool;
    const float *fpool;
    Node *node[2];
    long long node_cap;
    void *tab[2];               // double or float elements
    long long tab_cap;          // elements per arena
    uint8_t *ids[2];
    long long ids_cap;
    HashSlot *hash[2];
    long long hash_cap;         // power of two
    Cand *cand;
    long long cand_cap;
    int *q_lp1;                 // candidate indices for the FP64 LP1 re-solve
    int *q_opt;                 // node indices for the FP64 optimality re-solve
    int *q_s0;                  // node indices for the second pass of the first-stage dual LP
    long long q_s0_cap;         // (a full queue sends a set to the second stage instead)
    int *q_s1;                  // node indices for its third pass (uncapped)
    long long q_s1_cap;
    int *q_c2;                  // node indices for the FP64 kernel whose FP32 dual bound was negative
    unsigned long long *q_c2b;  // ... and their final FP32 dual bases (p + 1 row numbers, a byte each)
    long long q_c2_cap;         // (a full queue sends a set to q_opt without its basis)
    long long q_cap;
    uint8_t *cert_q;            // certificate queue: entries of cert_stride bytes, an int candidate
                                // index then the nv nonbasic ids of its final FP32 basis
    long long cert_cap;         // entries (a full queue sends candidates to the FP64 re-solve)
    int cert_stride;
    OptRec *opt;
    long long opt_cap;
    CandRec *rec;               // may be null
    long long rec_cap;
    unsigned long long *lp2b[2]; // LP2 basis sharing (may be null): per node, the final basis of its
                                 // first-stage dual LP (p + 1 row numbers, 0xff past them or none)
    InstCtl *ictl;
    Ctl *ctl;
    int exhaustive;             // 1: every combination is a candidate (no pruning)
    int precision;
};

}  // namespace mq
