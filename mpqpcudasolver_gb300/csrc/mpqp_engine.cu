// Host engine and C ABI of libmpqp_gb300.so.
//
//  * prepare_instance: FP64 precompute of the KKT blocks (host, once per
//    instance, fixed operation order with explicit fma, -ffp-contract=off);
//  * mpqp_plan: device buffers sized for the batch, the level loop captured
//    in one CUDA graph, results copied back on demand;
//  * mpqp / warm_up: the drop-in boundary of the reference's mpqp_cuda.so
//    (main.py:12-50), which rebuilds the problem from the LP matrices that
//    main.py:87-137 builds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <new>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mpqp_gb300.h"
#include "mpqp_internal.h"

namespace mq {
size_t lp1_smem_per_warp(int prec_bytes, const SlotDims &sd);
size_t feas_smem_per_warp(int prec_bytes, const SlotDims &sd);
size_t opt_smem_per_warp(int prec_bytes, const SlotDims &sd);
size_t screen_smem_per_warp(const SlotDims &sd, int route);
size_t screen_tiles_smem(const SlotDims &sd, int tile_w);
size_t screen_lanes_smem();
cudaError_t launch_opt_screen_lanes(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int mode,
                                    int grid, size_t smem, cudaStream_t s, int pass, int cap);
bool screen_dual_route(int mode, const InstDesc &I, const SlotDims &sd);
bool screen_lanes_route(int mode, const InstDesc &I, const SlotDims &sd);
size_t laws_smem_per_warp(const SlotDims &sd);
const void *kernel_ptr(const char *name);
cudaError_t launch_enumerate(const DevBuffers &B, int level, int grid, cudaStream_t s);
cudaError_t launch_feasibility(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int prec,
                               int grid, size_t smem, cudaStream_t s, int warps, int chunk);
cudaError_t launch_lp1_fp64(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int grid,
                            size_t smem, cudaStream_t s);
cudaError_t launch_lp1_cert(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int grid,
                            size_t smem, cudaStream_t s);
size_t cert_smem_per_warp(const SlotDims &sd);
cudaError_t launch_optimality(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, bool lp,
                              int grid, size_t smem, cudaStream_t s);
cudaError_t launch_opt_screen(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int mode, int route,
                              int grid, size_t smem, cudaStream_t s, int tile_w);
cudaError_t launch_optimality_fp64(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, bool lp,
                                   int grid, size_t smem, cudaStream_t s);
cudaError_t launch_level0(const DevBuffers &B, int prec, cudaStream_t s);
cudaError_t launch_reset(const DevBuffers &B, cudaStream_t s);
cudaError_t launch_finalize(const DevBuffers &B, int level, cudaStream_t s);
cudaError_t launch_region_laws(const DevBuffers &B, const Tol &tol, const SlotDims &sd, const uint64_t *masks,
                               long long n_sets, double *laws, int *sizes, long long stride, int grid,
                               size_t smem, cudaStream_t s);
cudaError_t launch_region_laws_r(const DevBuffers &B, const Tol &tol, const SlotDims &sd, const uint64_t *masks,
                                 long long n_sets, double *laws, int *sizes, long long stride, double *radius,
                                 double *err, int grid, size_t smem, cudaStream_t s);
}  // namespace mq

using namespace mq;

// the last error text of each calling thread (mpqp_last_error)
static thread_local std::string g_err;
static std::mutex g_mu;

static void set_err(const std::string &s) { g_err = s; }

namespace mq {
void set_error_text(const char *msg) { set_err(msg ? msg : ""); }
}  // namespace mq

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t _e = (call);                                                                       \
        if (_e != cudaSuccess) {                                                                       \
            set_err(std::string(#call) + ": " + cudaGetErrorString(_e));                               \
            return MPQP_ECUDA;                                                                         \
        }                                                                                              \
    } while (0)

// ---------------------------------------------------------------------
// FP64 precompute (operation order identical to the CPU oracle)
// ---------------------------------------------------------------------
struct Prepared {
    InstDesc d;
    std::vector<double> Wm, Wh, wc, At, bt, QiAT, QiH, Qic;
    std::vector<double> WhL, wcL, Hm, cv;   // mpLP only: A H, A c, H, c
    std::vector<double> blo, bhi;   // parameter box, when At is [diag(+); diag(-)]
    std::vector<double> root;    // LP1 root tableau, FP64 stride ld1d
    std::vector<double> root_f;  // the same values at the plan's stride ld1 (FP32 copy)
};

static inline int odd_up(int x) { return (x & 1) ? x : x + 1; }
// smallest y >= x with y = 4 (mod 8): FP32 rows 16-byte aligned and
// conflict-free for 128-bit shared-memory accesses
static inline int four_mod8_up(int x) { int y = (x + 3) & ~3; return (y & 4) ? y : y + 4; }

// The FP32 LP1 root.  From the origin (every slack basic, b >= 0), each
// free variable (x, theta) is pivoted into the basis by a ratio test in the
// direction whose blocking row has the larger pivot, so the basic solution
// stays feasible; a free variable unbounded both ways stays nonbasic.  The
// rows of basic free variables are dropped (they never leave the basis and
// no later decision reads them) and the objective row follows the live rows.
// Every FP32 LP1 solve descends from this root, so none carries rows of free
// variables or prices a free column with a zero reduced cost.  root_f gets
// the tableau (stride ld1, tab_elems) followed by the basis ids as numbers
// (bid over M1, 255 past the live rows, then nid over nv); d.root_rows the
// live rows.  Pivots in FP64: T_r /= T_rq (T_rq -> 1 / T_rq), then
// T_i -= T_iq T_r (T_iq -> -T_iq / T_rq), the Tucker pivot of the kernels.
static void prepivot_root_f(InstDesc &d, std::vector<double> &root_f)
{
    const int ld = d.ld1, nv = d.nv, M1 = d.M1;
    std::vector<double> T(root_f.begin(), root_f.begin() + (size_t)(M1 + 1) * ld);
    std::vector<int> bid(M1), nid(nv);
    for (int i = 0; i < M1; i++) bid[i] = nv + i;
    for (int j = 0; j < nv; j++) nid[j] = j;
    for (int q = 0; q < nv; q++) {
        double cmax = 0.0;
        for (int i = 0; i < M1; i++) if (bid[i] >= nv) cmax = std::max(cmax, std::fabs(T[(size_t)i * ld + q]));
        if (!(cmax > 0.0)) continue;
        int r = -1;
        double ra = 0.0;
        for (int dir = 1; dir >= -1; dir -= 2) {
            int rd = -1;
            double rr = 0.0, rad = 0.0;
            for (int i = 0; i < M1; i++) {
                if (bid[i] < nv) continue;
                const double a = dir * T[(size_t)i * ld + q];
                if (!(a > 1e-9 * cmax)) continue;
                const double ratio = std::max(T[(size_t)i * ld + nv], 0.0) / a;
                if (rd < 0 || ratio < rr || (ratio == rr && a > rad)) { rd = i; rr = ratio; rad = a; }
            }
            if (rd >= 0 && rad > ra) { r = rd; ra = rad; }
        }
        if (r < 0) continue;
        double *R = T.data() + (size_t)r * ld;
        const double inv = 1.0 / R[q];
        for (int j = 0; j <= nv; j++) if (j != q) R[j] *= inv;
        R[q] = inv;
        for (int i = 0; i <= M1; i++) {
            if (i == r) continue;
            double *Ti = T.data() + (size_t)i * ld;
            const double f = Ti[q];
            if (f == 0.0) continue;
            for (int j = 0; j <= nv; j++) if (j != q) Ti[j] -= f * R[j];
            Ti[q] = -f * inv;
        }
        std::swap(bid[r], nid[q]);
    }
    std::vector<double> out((size_t)d.tab_elems + M1 + nv, 0.0);
    int rows = 0;
    for (int i = 0; i < M1; i++) {
        if (bid[i] < nv) continue;
        for (int j = 0; j <= nv; j++) out[(size_t)rows * ld + j] = T[(size_t)i * ld + j];
        out[(size_t)d.tab_elems + rows] = bid[i];
        rows++;
    }
    for (int j = 0; j <= nv; j++) out[(size_t)rows * ld + j] = T[(size_t)M1 * ld + j];
    for (int i = rows; i < M1; i++) out[(size_t)d.tab_elems + i] = 255;
    for (int j = 0; j < nv; j++) out[(size_t)d.tab_elems + M1 + j] = nid[j];
    root_f.swap(out);
    d.root_rows = rows;
}

static void fwd_sub(const double *L, int n, const double *rhs, int rs, double *y, int ys)
{
    for (int i = 0; i < n; i++) {
        double acc = rhs[(size_t)i * rs];
        for (int l = 0; l < i; l++) acc = std::fma(-L[i * n + l], y[(size_t)l * ys], acc);
        y[(size_t)i * ys] = acc / L[i * n + i];
    }
}

static void bwd_sub(const double *L, int n, const double *y, int ysd, double *x, int xs)
{
    for (int i = n - 1; i >= 0; i--) {
        double acc = y[(size_t)i * ysd];
        for (int l = i + 1; l < n; l++) acc = std::fma(-L[l * n + i], x[(size_t)l * xs], acc);
        x[(size_t)i * xs] = acc / L[i * n + i];
    }
}

static int prepare_instance(const mpqp_problem &P, Prepared &out, int prec)
{
    const int n = P.n, m = P.m, p = P.p, ncp = P.ncp;
    if (n < 1 || m < 1 || p < 1 || ncp < 1 || m > kMaxM || p > kMaxP) {
        set_err("instance sizes out of range (need 1<=m<=128, 1<=p<=30, n>=1, ncp>=1)");
        return MPQP_EINVAL;
    }
    if (m + ncp + n + p > kMaxIds || m + ncp + p + 1 > kMaxIds) {
        set_err("instance too large for 8-bit basis ids (m+ncp+n+p must be <= 255)");
        return MPQP_EINVAL;
    }
    if (!P.Q || !P.c || !P.H || !P.A || !P.b || !P.F || !P.At || !P.bt) {
        set_err("null problem pointer");
        return MPQP_EINVAL;
    }
    for (int i = 0; i < m; i++)
        if (!(P.b[i] >= 0.0)) { set_err("b has a negative entry: the origin must be feasible"); return MPQP_EORIGIN; }
    for (int i = 0; i < ncp; i++)
        if (!(P.bt[i] >= 0.0)) { set_err("CRb has a negative entry: the origin must be feasible"); return MPQP_EORIGIN; }
    int kmax = P.k_max;
    if (kmax > m) kmax = m;
    if (kmax > kMaxK) kmax = kMaxK;
    if (kmax < 0) kmax = 0;
    InstDesc &d = out.d;
    memset(&d, 0, sizeof(d));
    d.n = n; d.m = m; d.p = p; d.ncp = ncp;
    d.M1 = m + ncp; d.nv = n + p;
    d.ld1d = odd_up(d.nv + 1);
    d.ld2d = odd_up(p + 2);
    d.ld1 = prec == PREC_MIXED ? four_mod8_up(d.nv + 1) : d.ld1d;
    d.ld2 = prec == PREC_MIXED ? four_mod8_up(p + 2) : d.ld2d;
    d.k_min = P.k_min < 0 ? 0 : P.k_min;
    d.k_max = kmax;
    d.tab_elems = ((d.M1 + 1) * d.ld1 + 3) & ~3;
    d.ids_bytes = (d.M1 + d.nv + 15) & ~15;
    d.budget = P.budget;
    d.lp = 1;
    for (int i = 0; i < n * n && d.lp; i++) if (P.Q[i] != 0.0) d.lp = 0;
    d.ld2lp = odd_up(p + n + 3);
    if (d.lp) {
        // mpLP (Q = 0): Wm = A A^T, Wh = F, wc = b, QiAT = A^T, QiH = Qic = 0,
        // WhL = A H, wcL = A c (each sum over ascending i from 0, the oracle's order)
        if ((p + n + 2) + (m + ncp + 2 * n + 1) > kMaxIds) {
            set_err("mpLP instance too large for 8-bit basis ids (m + ncp + 3n + p must be <= 252)");
            return MPQP_EINVAL;
        }
        out.Wm.assign((size_t)m * m, 0.0);
        out.Wh.assign(P.F, P.F + (size_t)m * p);
        out.wc.assign(P.b, P.b + m);
        out.WhL.assign((size_t)m * p, 0.0);
        out.wcL.assign(m, 0.0);
        out.QiAT.assign((size_t)n * m, 0.0);
        out.QiH.assign((size_t)n * p, 0.0);
        out.Qic.assign(n, 0.0);
        out.Hm.assign(P.H, P.H + (size_t)n * p);
        out.cv.assign(P.c, P.c + n);
        for (int r = 0; r < m; r++) {
            for (int s = 0; s < m; s++) {
                double acc = 0.0;
                for (int i = 0; i < n; i++) acc = std::fma(P.A[(size_t)r * n + i], P.A[(size_t)s * n + i], acc);
                out.Wm[(size_t)r * m + s] = acc;
            }
            for (int c = 0; c < p; c++) {
                double acc = 0.0;
                for (int i = 0; i < n; i++) acc = std::fma(P.A[(size_t)r * n + i], P.H[(size_t)i * p + c], acc);
                out.WhL[(size_t)r * p + c] = acc;
            }
            double acc = 0.0;
            for (int i = 0; i < n; i++) acc = std::fma(P.A[(size_t)r * n + i], P.c[i], acc);
            out.wcL[r] = acc;
            for (int i = 0; i < n; i++) out.QiAT[(size_t)i * m + r] = P.A[(size_t)r * n + i];
        }
    }
    std::vector<double> L((size_t)n * n, 0.0), V((size_t)n * m, 0.0), U((size_t)n * p, 0.0), u(n, 0.0);
    for (int j = 0; j < n && !d.lp; j++) {
        for (int i = j; i < n; i++) {
            double acc = P.Q[i * n + j];
            for (int l = 0; l < j; l++) acc = std::fma(-L[i * n + l], L[j * n + l], acc);
            if (i == j) {
                if (!(acc > 0.0)) { set_err("Q is neither positive definite nor zero"); return MPQP_ENOTSPD; }
                L[j * n + j] = std::sqrt(acc);
            } else {
                L[i * n + j] = acc / L[j * n + j];
            }
        }
    }
    if (!d.lp) {
    for (int r = 0; r < m; r++) fwd_sub(L.data(), n, P.A + (size_t)r * n, 1, V.data() + r, m);
    for (int c = 0; c < p; c++) fwd_sub(L.data(), n, P.H + c, p, U.data() + c, p);
    fwd_sub(L.data(), n, P.c, 1, u.data(), 1);
    out.Wm.assign((size_t)m * m, 0.0);
    out.Wh.assign((size_t)m * p, 0.0);
    out.wc.assign(m, 0.0);
    for (int r = 0; r < m; r++) {
        for (int s = 0; s < m; s++) {
            double acc = 0.0;
            for (int i = 0; i < n; i++) acc = std::fma(V[i * m + r], V[i * m + s], acc);
            out.Wm[r * m + s] = acc;
        }
        for (int c = 0; c < p; c++) {
            double acc = P.F[r * p + c];
            for (int i = 0; i < n; i++) acc = std::fma(V[i * m + r], U[i * p + c], acc);
            out.Wh[r * p + c] = acc;
        }
        double acc = P.b[r];
        for (int i = 0; i < n; i++) acc = std::fma(V[i * m + r], u[i], acc);
        out.wc[r] = acc;
    }
    out.QiAT.assign((size_t)n * m, 0.0);
    out.QiH.assign((size_t)n * p, 0.0);
    out.Qic.assign(n, 0.0);
    for (int r = 0; r < m; r++) bwd_sub(L.data(), n, V.data() + r, m, out.QiAT.data() + r, m);
    for (int c = 0; c < p; c++) bwd_sub(L.data(), n, U.data() + c, p, out.QiH.data() + c, p);
    bwd_sub(L.data(), n, u.data(), 1, out.Qic.data(), 1);
    }
    out.At.assign(P.At, P.At + (size_t)ncp * p);
    out.bt.assign(P.bt, P.bt + ncp);
    auto fill_root = [&](std::vector<double> &root, int ld) {
        root.assign(((size_t)(d.M1 + 1) * ld + 3) & ~(size_t)3, 0.0);
        for (int i = 0; i < m; i++) {
            for (int j = 0; j < n; j++) root[i * ld + j] = P.A[i * n + j];
            for (int j = 0; j < p; j++) root[i * ld + n + j] = -P.F[i * p + j];
            root[i * ld + d.nv] = P.b[i];
        }
        for (int i = 0; i < ncp; i++) {
            for (int j = 0; j < p; j++) root[(m + i) * ld + n + j] = P.At[i * p + j];
            root[(m + i) * ld + d.nv] = P.bt[i];
        }
    };
    fill_root(out.root, d.ld1d);
    fill_root(out.root_f, d.ld1);
    prepivot_root_f(d, out.root_f);
    // parameter box: row c reads s theta_c <= bt_c (s > 0), row p + c reads
    // s' theta_c <= bt_{p+c} (s' < 0), nothing else nonzero
    d.box = ncp == 2 * p;
    out.blo.assign(p, 0.0);
    out.bhi.assign(p, 0.0);
    for (int c = 0; c < p && d.box; c++) {
        for (int j = 0; j < p; j++) {
            const double up = P.At[c * p + j], dn = P.At[(p + c) * p + j];
            if (j == c ? !(up > 0.0 && dn < 0.0) : (up != 0.0 || dn != 0.0)) { d.box = 0; break; }
        }
        if (!d.box) break;
        out.bhi[c] = P.bt[c] / P.At[c * p + c];
        out.blo[c] = P.bt[p + c] / P.At[(p + c) * p + c];
        if (!(out.blo[c] <= out.bhi[c])) d.box = 0;
    }
    return MPQP_OK;
}

// ---------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------
struct mpqp_plan {
    int n_inst = 0;
    std::vector<InstDesc> desc;
    std::vector<mpqp_problem> probs;
    mpqp_options opt{};
    Tol tol{};
    SlotDims sd{};
    DevBuffers B{};
    std::vector<void *> allocs;
    int kmax = 0;
    int prec = PREC_FP64;
    int lp2_screen = 0;         // mixed precision: 0 dual bound on box instances, 1 primal tableau screen
    bool screen_dual = false, screen_primal = false;   // which FP32 screen routes the instances need
    bool lanes_lp = false;      // mpLP instances the first stage of the dual screen takes
    bool has_qp = false, has_lp = false;   // mpQP / mpLP (Q = 0) instances in the batch
    int grid_opt_lp = 0, grid_optfb_lp = 0;   // FP64 optimality kernels of the mpLP instances
    bool pooled = false;        // allocations came from the device pool
    int grid_opt2 = 0;          // grid of the primal route (grid_opt: the dual route)
    int grid_opt3 = 0;          // grid of the dual route's second stage
    int grid_opt_lprows = 0;    // the dual route's second stage for mpLP sets with |S| = n
    int grid_tiles = 0;         // the dual route's first stage (one set per tile of tile_w threads)
    size_t smem_tiles = 0;
    int grid_lanes = 0;         // ... at levels |S| <= kLaneMaxK: one set per thread
    size_t smem_lanes = 0;
    int lane_cap = 3;           // pivots of its first pass (MPQP_SCREEN_CAP)
    int lane_cap2 = 6;          // ... of its second (MPQP_SCREEN_CAP2; 0: uncapped, no third pass)
    // launch settings the autotuner chooses: threads per set in the screen's
    // first stage, warps per LP1 block, candidates an LP1 warp claims at once
    int tile_w = 8, feas_warps = 4, feas_chunk = 32;
    int tuned = 0;              // 1: the settings came from the autotuner (or its cache)
    size_t smem_opt2 = 0;       // shared memory per block of the primal route
    int grid_enum = 0, grid_feas = 0, grid_lp1fb = 0, grid_opt = 0, grid_optfb = 0, grid_cert = 0;
    size_t smem_feas = 0, smem_lp1fb = 0, smem_opt = 0, smem_optfb = 0, smem_cert = 0;
    int n_launches = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_mid = nullptr;
    bool ran = false;
    // timed runs: one event before every launch and one after the last
    std::vector<cudaEvent_t> kev;
    std::vector<const char *> kname;
    bool timed = false;
    double last_ms = 0;
    double feas_ms = 0, opt_ms = 0;
    long long h2d_bytes = 0;
};

// An exported entry point lets no C++ exception through (a failed host
// allocation inside becomes MPQP_ENOMEM).
static int host_failure(const char *where)
{
    try {
        set_err(std::string(where) + ": host memory allocation failed");
    } catch (...) {
    }
    return MPQP_ENOMEM;
}

extern "C" void mpqp_default_options(mpqp_options *o)
{
    memset(o, 0, sizeof(*o));
    o->precision = MPQP_FP64;
    o->use_graph = 1;
    o->mem_fraction = 0.6;
    o->tol_feas = 1e-9;
    o->tol_opt = 1e-9;
    o->tol_licq = 1e-10;
    o->r_min = 1e-8;
    o->tol_piv = 1e-9;
    o->tol_dj = 1e-9;
    o->max_pivots = 256;
    o->degen_switch = 8;
    o->tol_piv32 = 1e-6;
    o->tol_dj32 = 1e-6;
    o->margin_z = 1e-6;      // routing only: FP32 z above it -> FP64 dual certificate
    o->margin_beta = 3e-5;   // x max(1, max |T_ij|) of the final FP32 LP1 tableau
    o->margin_t = 1e-5;   // x (row magnitude / pivot ratio) x (1 + p |theta|max)
    o->margin_licq = 1e-3;
    o->tol_zero_row = 1e-12;
    o->lp2_screen = 0;
}

static void fill_defaults(mpqp_options &o)
{
    mpqp_options d;
    mpqp_default_options(&d);
#define DEF(f) if (o.f == 0) o.f = d.f
    DEF(mem_fraction); DEF(tol_feas); DEF(tol_opt); DEF(tol_licq); DEF(r_min); DEF(tol_piv); DEF(tol_dj);
    DEF(max_pivots); DEF(degen_switch); DEF(tol_piv32); DEF(tol_dj32); DEF(margin_z); DEF(margin_beta);
    DEF(margin_t); DEF(margin_licq); DEF(tol_zero_row);
#undef DEF
}

// Plan memory comes from one stream-ordered pool per device that keeps what
// is freed (release threshold: everything).  Freeing the tens of GB of a
// large plan with cudaFree unmaps them and takes over 100 ms; from the pool,
// a plan's teardown is cheap and the next plan reuses the memory.  The idle
// bytes of the pool count as free when a plan sizes its buffers, and
// mpqp_release_cached_memory() hands them back to the driver.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pools[64] = {};

static cudaMemPool_t plan_pool(int dev)
{
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (dev < 0 || dev >= 64) return nullptr;
    if (!g_pools[dev]) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}

// bytes the pool of `dev` holds but no plan uses
static size_t pool_idle_bytes(int dev)
{
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (dev < 0 || dev >= 64 || !g_pools[dev]) return 0;
    uint64_t reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(g_pools[dev], cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess ||
        cudaMemPoolGetAttribute(g_pools[dev], cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return reserved > used ? (size_t)(reserved - used) : 0;
}

static size_t free_device_bytes()
{
    size_t fb = 0, tb = 0;
    int dev = 0;
    if (cudaMemGetInfo(&fb, &tb) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return 0; }
    return fb + pool_idle_bytes(dev);
}

static int dev_alloc(mpqp_plan *P, void **ptr, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool = plan_pool(dev);
    cudaError_t e = pool ? cudaMallocFromPoolAsync(ptr, bytes, pool, 0) : cudaMalloc(ptr, bytes);
    if (e == cudaSuccess && pool) P->pooled = true;
    if (e != cudaSuccess) {
        set_err(std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
        cudaGetLastError();
        return MPQP_ENOMEM;
    }
    P->allocs.push_back(*ptr);
    return MPQP_OK;
}

static void free_plan_mem(mpqp_plan *P)
{
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    P->exec = nullptr; P->graph = nullptr;
    if (P->pooled) {
        // every run of the plan has finished before its memory goes back
        cudaDeviceSynchronize();
        for (void *p : P->allocs) cudaFreeAsync(p, 0);
        cudaStreamSynchronize(0);
    } else {
        for (void *p : P->allocs) cudaFree(p);
    }
    P->allocs.clear();
    if (P->ev0) cudaEventDestroy(P->ev0);
    if (P->ev1) cudaEventDestroy(P->ev1);
    if (P->ev_mid) cudaEventDestroy(P->ev_mid);
    for (cudaEvent_t e : P->kev) cudaEventDestroy(e);
    P->kev.clear();
    P->ev0 = P->ev1 = P->ev_mid = nullptr;
}

static int grid_for(const void *fn, size_t smem, int *grid, int block = 128)
{
    int dev = 0, sms = 0, nb = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (smem > 48 * 1024) CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block, smem));
    if (nb < 1) {
        set_err("kernel does not fit on an SM (shared memory " + std::to_string(smem) + " bytes)");
        return MPQP_EINVAL;
    }
    *grid = nb * sms;
    return MPQP_OK;
}

// The fixed launch sequence of one enumeration.  timed: record an event
// before every launch (and one after the last) on the same stream.
static int enqueue(mpqp_plan *P, cudaStream_t s, bool timed)
{
    const DevBuffers &B = P->B;
    const bool mixed = P->prec == PREC_MIXED;
    const char *feas = mixed ? "k_feasibility<float>" : "k_feasibility<double>";
    int nl = 0;
    if (timed) P->kname.clear();
    auto chk = [&](const char *name, cudaError_t e) -> int {
        if (e != cudaSuccess) { set_err(std::string("launch of ") + name + ": " + cudaGetErrorString(e)); return MPQP_ECUDA; }
        return MPQP_OK;
    };
    auto pre = [&](const char *name) -> int {
        if (timed) {
            if ((int)P->kev.size() <= nl) {
                cudaEvent_t e;
                if (cudaEventCreate(&e) != cudaSuccess) { set_err("cudaEventCreate"); return MPQP_ECUDA; }
                P->kev.push_back(e);
            }
            if (cudaEventRecord(P->kev[nl], s) != cudaSuccess) { set_err("cudaEventRecord"); return MPQP_ECUDA; }
            P->kname.push_back(name);
        }
        nl++;
        return MPQP_OK;
    };
#define L(name, x) do { int _r = pre(name); if (_r) return _r; _r = chk(name, x); if (_r) return _r; } while (0)
    // FP32 screen: the dual route and/or the primal route, each launched only
    // when some instance takes it; FP64: the optimality kernel
    auto launch_opt = [&](int level) -> int {
        if (!mixed) {
            if (P->has_qp)
                L("k_optimality<double>", launch_optimality(B, P->tol, P->sd, level, false, P->grid_opt, P->smem_opt, s));
            if (P->has_lp)
                L("k_optimality<double,mplp>",
                  launch_optimality(B, P->tol, P->sd, level, true, P->grid_opt_lp, P->smem_opt, s));
            return MPQP_OK;
        }
        const bool lanes = level <= kLaneMaxK && !B.lp2b[0] && (P->screen_dual || P->lanes_lp);
        if (lanes) {
            L("k_opt_screen<dual,lanes>", launch_opt_screen_lanes(B, P->tol, P->sd, level, P->lp2_screen,
                                                                  P->grid_lanes, P->smem_lanes, s, 0, P->lane_cap));
            L("k_opt_screen<dual,lanes,rerun>", launch_opt_screen_lanes(B, P->tol, P->sd, level, P->lp2_screen,
                                                                        P->grid_lanes, P->smem_lanes, s, 1,
                                                                        P->lane_cap2));
            if (P->lane_cap2 > 0)
                L("k_opt_screen<dual,lanes,rerun2>", launch_opt_screen_lanes(B, P->tol, P->sd, level, P->lp2_screen,
                                                                             P->grid_lanes, P->smem_lanes, s, 2, 0));
            if (P->lanes_lp)
                L("k_opt_screen<dual,stationarity>", launch_opt_screen(B, P->tol, P->sd, level, P->lp2_screen, 3,
                                                                       P->grid_tiles, P->smem_tiles, s, P->tile_w));
        }
        if (!lanes && (P->screen_dual || P->lanes_lp))
            L("k_opt_screen<dual>", launch_opt_screen(B, P->tol, P->sd, level, P->lp2_screen, 0, P->grid_tiles,
                                                      P->smem_tiles, s, P->tile_w));
        if (P->lanes_lp)
            L("k_opt_screen<dual,rows,mplp>",
              launch_opt_screen(B, P->tol, P->sd, level, P->lp2_screen, 6, P->grid_opt_lprows, P->smem_opt, s,
                                P->tile_w));
        if (P->screen_dual) {
            L("k_opt_screen<dual,rows>",
              launch_opt_screen(B, P->tol, P->sd, level, P->lp2_screen, 2, P->grid_opt3, P->smem_opt, s, P->tile_w));
        }
        if (P->screen_primal)
            L("k_opt_screen<primal>", launch_opt_screen(B, P->tol, P->sd, level, P->lp2_screen, 1, P->grid_opt2, P->smem_opt2, s,
                                                        P->tile_w));
        return MPQP_OK;
    };
    // FP64 re-evaluation of the sets the FP32 screen left undecided
    auto launch_optfb = [&](int level) -> int {
        if (!mixed) return MPQP_OK;
        if (P->has_qp)
            L("k_optimality_fp64",
              launch_optimality_fp64(B, P->tol, P->sd, level, false, P->grid_optfb, P->smem_optfb, s));
        if (P->has_lp)
            L("k_optimality_fp64<mplp>",
              launch_optimality_fp64(B, P->tol, P->sd, level, true, P->grid_optfb_lp, P->smem_optfb, s));
        return MPQP_OK;
    };
    L("k_reset", launch_reset(B, s));
    L("k_level0", launch_level0(B, P->prec, s));
    { const int _o = launch_opt(0); if (_o) return _o; }
    { const int _o = launch_optfb(0); if (_o) return _o; }
    L("k_finalize", launch_finalize(B, 0, s));
    for (int k = 1; k <= P->kmax; k++) {
        L("k_enumerate", launch_enumerate(B, k, P->grid_enum, s));
        L(feas, launch_feasibility(B, P->tol, P->sd, k, P->prec, P->grid_feas, P->smem_feas, s, P->feas_warps,
                                   P->feas_chunk));
        if (mixed) {
            L("k_lp1_cert", launch_lp1_cert(B, P->tol, P->sd, k, P->grid_cert, P->smem_cert, s));
            L("k_lp1_fp64", launch_lp1_fp64(B, P->tol, P->sd, k, P->grid_lp1fb, P->smem_lp1fb, s));
        }
        { const int _o = launch_opt(k); if (_o) return _o; }
        { const int _o = launch_optfb(k); if (_o) return _o; }
        L("k_finalize", launch_finalize(B, k, s));
    }
#undef L
    if (timed) {
        if ((int)P->kev.size() <= nl) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) { set_err("cudaEventCreate"); return MPQP_ECUDA; }
            P->kev.push_back(e);
        }
        if (cudaEventRecord(P->kev[nl], s) != cudaSuccess) { set_err("cudaEventRecord"); return MPQP_ECUDA; }
    }
    P->n_launches = nl;
    return MPQP_OK;
}

// The body of mpqp_plan_create (the caller holds g_mu); the launch settings
// come from the options, 0 selecting the defaults.
static int plan_create_locked(int n_inst, const mpqp_problem *probs, const mpqp_options *opt_in, mpqp_plan **out)
{
    *out = nullptr;
    if (n_inst < 1 || !probs) { set_err("no instances"); return MPQP_EINVAL; }
    mpqp_plan *P = new mpqp_plan();
    if (opt_in) P->opt = *opt_in; else mpqp_default_options(&P->opt);
    fill_defaults(P->opt);
    const mpqp_options &o = P->opt;
    P->prec = o.precision == MPQP_MIXED ? PREC_MIXED : PREC_FP64;
    if (o.lp2_screen != 0 && o.lp2_screen != 1) {
        set_err("lp2_screen must be 0 or 1");
        delete P;
        return MPQP_EINVAL;
    }
    if ((o.tile_w && o.tile_w != 8 && o.tile_w != 16 && o.tile_w != 32) || o.feas_warps < 0 || o.feas_warps > 4 ||
        o.feas_chunk < 0 || o.feas_chunk > 32) {
        set_err("launch settings out of range (tile_w 8/16/32, feas_warps 1..4, feas_chunk 1..32)");
        delete P;
        return MPQP_EINVAL;
    }
    if (o.lp2_warm != 0 && o.lp2_warm != 1) {
        set_err("lp2_warm must be 0 or 1");
        delete P;
        return MPQP_EINVAL;
    }
    if (o.tile_w) P->tile_w = o.tile_w;
    if (o.feas_warps) P->feas_warps = o.feas_warps;
    if (o.feas_chunk) P->feas_chunk = o.feas_chunk;
    P->lp2_screen = o.lp2_screen;
    P->n_inst = n_inst;
    P->probs.assign(probs, probs + n_inst);
    Tol &t = P->tol;
    t.tol_feas = o.tol_feas; t.tol_opt = o.tol_opt; t.tol_licq = o.tol_licq; t.r_min = o.r_min;
    t.tol_piv = o.tol_piv; t.tol_dj = o.tol_dj; t.max_pivots = o.max_pivots; t.degen_switch = o.degen_switch;
    t.tol_piv32 = (float)o.tol_piv32; t.tol_dj32 = (float)o.tol_dj32;
    t.margin_z = o.margin_z; t.margin_beta = o.margin_beta; t.margin_t = o.margin_t; t.margin_licq = o.margin_licq;
    t.margin_z32 = (float)o.margin_z; t.margin_beta32 = (float)o.margin_beta;
    t.margin_t32 = (float)o.margin_t; t.margin_licq32 = (float)o.margin_licq;
    t.tol_zero_row = o.tol_zero_row;
    // host precompute
    std::vector<Prepared> prep(n_inst);
    for (int i = 0; i < n_inst; i++) {
        int rc = prepare_instance(probs[i], prep[i], P->prec);
        if (rc) { set_err("instance " + std::to_string(i) + ": " + g_err); delete P; return rc; }
    }
    // pools
    std::vector<double> dp;
    std::vector<float> fp;
    auto put = [](auto &pool, const std::vector<double> &v) -> long long {
        long long off = (long long)pool.size();
        for (double x : v) pool.push_back((typename std::remove_reference<decltype(pool)>::type::value_type)x);
        while (pool.size() % 4) pool.push_back(0);
        return off;
    };
    SlotDims &sd = P->sd;
    sd = SlotDims{};
    sd.maxK = 1;
    long long tab_tot0 = 0, ids_tot0 = 0;
    size_t max_tab_bytes = 0;
    for (int i = 0; i < n_inst; i++) {
        Prepared &pr = prep[i];
        InstDesc &d = pr.d;
        d.o_Wm = put(dp, pr.Wm); d.o_Wh = put(dp, pr.Wh); d.o_wc = put(dp, pr.wc);
        d.o_At = put(dp, pr.At); d.o_bt = put(dp, pr.bt); d.o_QiAT = put(dp, pr.QiAT);
        d.o_QiH = put(dp, pr.QiH); d.o_Qic = put(dp, pr.Qic); d.o_root = put(dp, pr.root);
        d.o_WhL = put(dp, pr.WhL); d.o_wcL = put(dp, pr.wcL); d.o_Hm = put(dp, pr.Hm); d.o_cv = put(dp, pr.cv);
        d.f_Wm = put(fp, pr.Wm); d.f_Wh = put(fp, pr.Wh); d.f_wc = put(fp, pr.wc);
        d.f_At = put(fp, pr.At); d.f_bt = put(fp, pr.bt); d.f_root = put(fp, pr.root_f);
        d.f_blo = put(fp, pr.blo); d.f_bhi = put(fp, pr.bhi);
        // mpLP: FP32 copies of the multiplier law's right-hand sides and of
        // the stationarity residual's data for the FP32 screen
        d.f_WhL = d.f_wcL = d.f_AT = d.f_Hm = d.f_cv = -1;
        if (d.lp) {
            d.f_WhL = put(fp, pr.WhL); d.f_wcL = put(fp, pr.wcL);
            d.f_AT = put(fp, pr.QiAT); d.f_Hm = put(fp, pr.Hm); d.f_cv = put(fp, pr.cv);
        }
        P->desc.push_back(d);
        P->kmax = std::max(P->kmax, d.k_max);
        sd.maxM1 = std::max(sd.maxM1, d.M1);
        sd.maxLD1 = std::max(sd.maxLD1, d.ld1);
        sd.maxNv = std::max(sd.maxNv, d.nv);
        sd.maxK = std::max(sd.maxK, std::max(1, std::min(d.k_max, d.m)));
        sd.maxP1 = std::max(sd.maxP1, d.p + 1);
        sd.maxR2 = std::max(sd.maxR2, d.m + d.ncp);
        sd.maxLD2 = std::max(sd.maxLD2, d.ld2);
        sd.maxLD1d = std::max(sd.maxLD1d, d.ld1d);
        sd.maxLD2d = std::max(sd.maxLD2d, d.lp ? std::max(d.ld2d, d.ld2lp) : d.ld2d);
        sd.maxR2d = std::max(sd.maxR2d, d.lp ? d.m + d.ncp + 2 * d.n + 1 : d.m + d.ncp);
        if (d.lp) sd.maxN = std::max(sd.maxN, d.n);
        tab_tot0 += d.tab_elems;
        ids_tot0 += d.ids_bytes;
        max_tab_bytes = std::max(max_tab_bytes, (size_t)d.tab_elems * (P->prec == PREC_MIXED ? 4 : 8));
    }
    const size_t es = P->prec == PREC_MIXED ? 4 : 8;
    // capacities
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        set_err(std::string("cudaMemGetInfo: ") + cudaGetErrorString(cudaGetLastError()));
        delete P;
        return MPQP_ECUDA;
    }
    free_b = free_device_bytes();
    const double usable = (double)free_b * o.mem_fraction;
    long long total_budget = 0;
    bool all_budget = true;
    for (int i = 0; i < n_inst; i++) {
        if (probs[i].budget > 0) total_budget += probs[i].budget; else all_budget = false;
    }
    // combinatorial ceilings: at most C(m, k) candidates / nodes at level k
    double lvl_max = 0, arena_max = 0;
    {
        std::vector<double> lvl(kMaxK + 2, 0.0), lvl_tab(kMaxK + 2, 0.0);
        for (int i = 0; i < n_inst; i++) {
            // an instance with a budget writes at most that many candidates
            // (and nodes) at any level: a level is enumerated only while it fits
            const double cap_i = P->desc[i].budget > 0 ? (double)P->desc[i].budget : 1e300;
            double cmk = 1.0;
            for (int k = 0; k <= P->desc[i].k_max; k++) {
                if (k > 0) cmk = cmk * (double)(P->desc[i].m - k + 1) / (double)k;
                const double nk = std::min(cmk, cap_i);
                lvl[k] += nk;
                if (k < P->desc[i].k_max) lvl_tab[k] += nk * (double)P->desc[i].tab_elems * (double)es;
            }
        }
        for (int k = 0; k <= kMaxK; k++) {
            lvl_max = std::max(lvl_max, lvl[k]);
            arena_max = std::max(arena_max, lvl_tab[k] + lvl_tab[k + 1]);
        }
    }
    long long cand_cap = o.cand_cap;
    if (cand_cap <= 0) {
        // per candidate: cand 8 + q_lp1 4 + node 2x48 + q_opt 4 + hash 2x2x32,
        // plus arena share; keep the candidate side at ~30 % of usable memory
        const double per = 8 + 4 + 2 * sizeof(Node) + 4 + 4 * sizeof(HashSlot);
        cand_cap = (long long)(usable * 0.3 / per);
        if (all_budget) cand_cap = std::min(cand_cap, total_budget + n_inst);
        cand_cap = (long long)std::min((double)cand_cap, lvl_max + 64);
        cand_cap = std::max(cand_cap, (long long)1024);
    }
    long long node_cap = o.node_cap > 0 ? o.node_cap : cand_cap;
    node_cap = std::max(node_cap, (long long)n_inst);
    long long hash_cap = 16;
    while (hash_cap < 2 * node_cap + 1) hash_cap <<= 1;
    long long arena_bytes = o.arena_bytes;
    if (arena_bytes <= 0) {
        const double used = (double)cand_cap * 12 + (double)node_cap * (2 * sizeof(Node) + 4) +
                            (double)hash_cap * 2 * sizeof(HashSlot) +
                            (P->prec == PREC_MIXED ? (double)cand_cap / 8 * 48 + (double)cand_cap : 0.0) +  // certificate and rerun queues
                            (o.lp2_warm && P->prec == PREC_MIXED ? 16.0 * (double)node_cap : 0.0);   // LP2 bases
        arena_bytes = (long long)std::max(usable - used, (double)(64 << 20));
        if (all_budget) {
            // parents of the deepest checked level hold at most the budget
            const double need = (double)(total_budget + n_inst) * (double)(max_tab_bytes + 64);
            arena_bytes = (long long)std::min((double)arena_bytes, need * 1.05 + (64 << 20));
        }
        arena_bytes = (long long)std::min((double)arena_bytes, arena_max * 1.05 + (16 << 20));
    }
    long long tab_cap = arena_bytes / (long long)es;
    tab_cap = std::max(tab_cap, 2 * tab_tot0 + 1024);
    tab_cap &= ~3LL;
    // basis ids: one record per stored tableau, sized by the smallest tableau
    long long min_tab = 1LL << 40, max_ids = 16;
    for (const InstDesc &d : P->desc) { min_tab = std::min(min_tab, (long long)d.tab_elems); max_ids = std::max(max_ids, (long long)d.ids_bytes); }
    long long ids_cap = std::max((tab_cap / min_tab + n_inst + 1) * max_ids, 2 * ids_tot0 + 1024);
    ids_cap = (ids_cap + 15) & ~15LL;
    long long opt_cap = o.opt_cap > 0 ? o.opt_cap : std::max(node_cap / 8, (long long)4096);
    long long rec_cap = o.record ? (o.rec_cap > 0 ? o.rec_cap : cand_cap * 4) : 0;
    DevBuffers &B = P->B;
    memset(&B, 0, sizeof(B));
    B.n_inst = n_inst;
    B.node_cap = node_cap;
    B.tab_cap = tab_cap;
    B.ids_cap = ids_cap;
    B.hash_cap = hash_cap;
    B.cand_cap = cand_cap;
    B.q_cap = cand_cap;
    // certificate queue (mixed precision): FP32 LP1 optima that are not
    // certified feasible; beyond its capacity they go to the FP64 re-solve
    // an int (the candidate), the nonbasic ids, a float (the tableau's growth)
    B.cert_stride = (int)((8 + std::min(sd.maxNv, 32) + 15) & ~15);
    B.cert_cap = P->prec == PREC_MIXED ? std::max(cand_cap / 8, (long long)4096) : 0;
    B.opt_cap = opt_cap;
    B.rec_cap = rec_cap;
    B.exhaustive = o.exhaustive ? 1 : 0;
    B.precision = P->prec;
    int rc = MPQP_OK;
    void *p;
#define AL(ptr, bytes) do { rc = dev_alloc(P, &p, (bytes)); if (rc) { free_plan_mem(P); delete P; return rc; } ptr = (decltype(ptr))p; } while (0)
    AL(B.inst, sizeof(InstDesc) * n_inst);
    AL(B.dpool, sizeof(double) * dp.size());
    AL(B.fpool, sizeof(float) * fp.size());
    AL(B.node[0], sizeof(Node) * node_cap);
    AL(B.node[1], sizeof(Node) * node_cap);
    AL(B.tab[0], es * (size_t)tab_cap);
    B.tab[1] = B.tab[0];  // one arena, two sides (see below)
    AL(B.ids[0], (size_t)ids_cap);
    B.ids[1] = B.ids[0];
    AL(B.hash[0], sizeof(HashSlot) * hash_cap);
    AL(B.hash[1], sizeof(HashSlot) * hash_cap);
    AL(B.cand, sizeof(Cand) * cand_cap);
    AL(B.q_lp1, sizeof(int) * cand_cap);
    AL(B.q_opt, sizeof(int) * cand_cap);
    B.q_s0_cap = P->prec == PREC_MIXED ? std::max(cand_cap / 4, (long long)4096) : 0;
    if (B.q_s0_cap) AL(B.q_s0, sizeof(int) * B.q_s0_cap);
    B.q_s1_cap = P->prec == PREC_MIXED ? std::max(cand_cap / 16, (long long)4096) : 0;
    if (B.q_s1_cap) AL(B.q_s1, sizeof(int) * B.q_s1_cap);
    // sets the FP32 dual screen found not optimal below its margin's reach: a
    // sixteenth of the candidates (a full queue sends the rest to q_opt)
    B.q_c2_cap = P->prec == PREC_MIXED ? std::max(cand_cap / 16, (long long)4096) : 0;
    if (B.q_c2_cap) {
        AL(B.q_c2, sizeof(int) * B.q_c2_cap);
        AL(B.q_c2b, sizeof(unsigned long long) * B.q_c2_cap);
    }
    AL(B.cert_q, (size_t)B.cert_stride * B.cert_cap);
    AL(B.opt, sizeof(OptRec) * opt_cap);
    if (rec_cap) AL(B.rec, sizeof(CandRec) * rec_cap);
    if (o.lp2_warm && P->prec == PREC_MIXED) {
        AL(B.lp2b[0], sizeof(unsigned long long) * node_cap);
        AL(B.lp2b[1], sizeof(unsigned long long) * node_cap);
    }
    AL(B.ictl, sizeof(InstCtl) * n_inst);
    AL(B.ctl, sizeof(Ctl));
#undef AL
    CK(cudaStreamSynchronize(0));   // the pool's allocations are stream-ordered on stream 0
    CK(cudaMemcpy((void *)B.inst, P->desc.data(), sizeof(InstDesc) * n_inst, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((void *)B.dpool, dp.data(), sizeof(double) * dp.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy((void *)B.fpool, fp.data(), sizeof(float) * fp.size(), cudaMemcpyHostToDevice));
    P->h2d_bytes = (long long)(sizeof(InstDesc) * n_inst + sizeof(double) * dp.size() + sizeof(float) * fp.size());
    // the hash is not cleared: a slot counts only when its tag (the run's
    // epoch from the device's counter, and the level) and its fingerprint
    // equal a query's, so an earlier plan's entries in pooled memory and any
    // other leftover bytes read as empty slots
    CK(cudaMemset(B.ctl, 0, sizeof(Ctl)));
    if (B.lp2b[0]) {
        CK(cudaMemset(B.lp2b[0], 0xff, sizeof(unsigned long long) * node_cap));
        CK(cudaMemset(B.lp2b[1], 0xff, sizeof(unsigned long long) * node_cap));
    }
    // kernel geometry
    P->smem_feas = (size_t)P->feas_warps * feas_smem_per_warp(P->prec == PREC_MIXED ? 4 : 8, sd);
    P->smem_lp1fb = 4 * lp1_smem_per_warp(8, sd);
    P->smem_cert = 4 * cert_smem_per_warp(sd);
    // mixed precision: the grouped FP32 screen, one warp per block
    P->smem_opt = P->prec == PREC_MIXED ? screen_smem_per_warp(sd, 0) : 4 * opt_smem_per_warp(8, sd);
    P->smem_opt2 = screen_smem_per_warp(sd, 1);
    P->smem_tiles = screen_tiles_smem(sd, P->tile_w);
    P->smem_lanes = screen_lanes_smem();
    if (const char *e = getenv("MPQP_SCREEN_CAP")) P->lane_cap = std::max(1, atoi(e));
    if (const char *e = getenv("MPQP_SCREEN_CAP2")) P->lane_cap2 = std::max(0, atoi(e));
    if (P->lane_cap2 > 0 && P->lane_cap2 <= P->lane_cap) P->lane_cap2 = 0;
    for (const InstDesc &d : P->desc) {
        if (d.lp) P->has_lp = true; else P->has_qp = true;
        if (P->prec != PREC_MIXED) continue;
        if (screen_dual_route(P->lp2_screen, d, sd)) P->screen_dual = true;
        else if (d.lp && screen_lanes_route(P->lp2_screen, d, sd)) P->lanes_lp = true;
        else P->screen_primal = true;
    }
    P->smem_optfb = 4 * opt_smem_per_warp(8, sd);
    if ((rc = grid_for(kernel_ptr("enumerate"), 0, &P->grid_enum)) ||
        (rc = grid_for(kernel_ptr(P->prec == PREC_MIXED ? "feas32" : "feas64"), P->smem_feas, &P->grid_feas,
                       32 * P->feas_warps)) ||
        (rc = grid_for(kernel_ptr("lp1_fp64"), P->smem_lp1fb, &P->grid_lp1fb)) ||
        (rc = grid_for(kernel_ptr("lp1_cert"), P->smem_cert, &P->grid_cert)) ||
        (rc = P->prec == PREC_MIXED
                  ? grid_for(kernel_ptr("screen_dual_rows"), P->smem_opt, &P->grid_opt, 32)
                  : grid_for(kernel_ptr("opt64"), P->smem_opt, &P->grid_opt)) ||
        (rc = P->prec == PREC_MIXED ? grid_for(kernel_ptr("screen_primal"), P->smem_opt2, &P->grid_opt2, 32) : 0) ||
        (rc = P->prec == PREC_MIXED ? grid_for(kernel_ptr("screen_dual_rows"), P->smem_opt, &P->grid_opt3, 32) : 0) ||
        (rc = P->prec == PREC_MIXED && P->lanes_lp ? grid_for(kernel_ptr("screen_dual_rows_lp"), P->smem_opt,
                                                              &P->grid_opt_lprows, 32)
                                                   : 0) ||
        (rc = P->prec == PREC_MIXED
                  ? grid_for(kernel_ptr(P->B.lp2b[0] ? (P->tile_w == 8 ? "screen_dual_tiles8w"
                                                       : P->tile_w == 16 ? "screen_dual_tiles16w"
                                                                         : "screen_dual_tiles32w")
                                                    : (P->tile_w == 8 ? "screen_dual_tiles8"
                                                       : P->tile_w == 16 ? "screen_dual_tiles16"
                                                                         : "screen_dual_tiles32")),
                             P->smem_tiles, &P->grid_tiles, 32)
                  : 0) ||
        (rc = P->prec == PREC_MIXED ? grid_for(kernel_ptr("screen_dual_lanes"), P->smem_lanes, &P->grid_lanes, 32)
                                    : 0) ||
        (rc = grid_for(kernel_ptr("opt_fp64"), P->smem_optfb, &P->grid_optfb)) ||
        (rc = P->has_lp && P->prec != PREC_MIXED ? grid_for(kernel_ptr("opt64_lp"), P->smem_opt, &P->grid_opt_lp) : 0) ||
        (rc = P->has_lp ? grid_for(kernel_ptr("opt_fp64_lp"), P->smem_optfb, &P->grid_optfb_lp) : 0)) {
        free_plan_mem(P);
        delete P;
        return rc;
    }
    CK(cudaEventCreate(&P->ev0));
    CK(cudaEventCreate(&P->ev1));
    CK(cudaEventCreate(&P->ev_mid));
    if (o.use_graph) {
        cudaStream_t cs;
        CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        rc = enqueue(P, cs, false);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (rc || e != cudaSuccess) {
            if (!rc) set_err(std::string("graph capture: ") + cudaGetErrorString(e));
            if (g) cudaGraphDestroy(g);
            free_plan_mem(P);
            delete P;
            return rc ? rc : MPQP_ECUDA;
        }
        P->graph = g;
        CK(cudaGraphInstantiate(&P->exec, g, 0));
    }
    *out = P;
    return MPQP_OK;
}

// ---------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------
// The reference passes its threads per LP (nTPB) and launch shapes from its
// host code (batched_simplex.cu:1181 and the launches around it).  Here the
// LPs per block and threads per LP are chosen by measurement: each candidate
// setting runs the batch with an event around every launch, and a setting
// replaces the default only when its kernels take at least 2 % less.  The
// whole batch is timed when it has at most kTuneWhole candidates (the
// combinatorial count under the budgets): its deepest levels dominate the
// cost and behave unlike its first ones, and a slice of the first levels
// picked settings that were slower on the full run.  Larger batches are
// timed on a slice, every instance under a kTuneSlice candidate budget.
// LP1 (warps per block x candidates per claim) and the screen's first stage
// (threads per LP) are independent kernels, tuned one after the other.  The
// choice is cached per batch shape for the process.
constexpr double kTuneWhole = 1.5e8;
constexpr long long kTuneSlice = 1LL << 22;
struct TuneKey {
    int prec, lp2_screen, m1, nv, p1, ninst;
    bool operator==(const TuneKey &k) const
    {
        return prec == k.prec && lp2_screen == k.lp2_screen && m1 == k.m1 && nv == k.nv && p1 == k.p1 &&
               ninst == k.ninst;
    }
};
struct TuneEntry { TuneKey key; int tile_w, feas_warps, feas_chunk; };
static int mpqp_plan_run_timed_impl(mpqp_plan *P, void *stream);
static std::vector<TuneEntry> g_tune_cache;   // guarded by g_mu

static TuneKey tune_key(int n_inst, const mpqp_problem *probs, const mpqp_options &o)
{
    TuneKey k{o.precision == MPQP_MIXED ? 1 : 0, o.lp2_screen, 0, 0, 0, 0};
    for (int i = 0; i < n_inst; i++) {
        k.m1 = std::max(k.m1, probs[i].m + probs[i].ncp);
        k.nv = std::max(k.nv, probs[i].n + probs[i].p);
        k.p1 = std::max(k.p1, probs[i].p + 1);
    }
    // shapes within a bucket share the choice: rows by 8, variables by 4,
    // instance counts by powers of two
    k.m1 = (k.m1 + 7) / 8;
    k.nv = (k.nv + 3) / 4;
    int b = 0;
    while ((1 << b) < n_inst) b++;
    k.ninst = b;
    return k;
}

// Milliseconds of the kernels whose names start with `prefix` in a timed run
// of `slice` under `o`, the best of `runs`; < 0 when the setting cannot run.
static double tune_trial(int n_inst, const mpqp_problem *slice, const mpqp_options &o, const char *prefix, int runs)
{
    mpqp_plan *P = nullptr;
    if (plan_create_locked(n_inst, slice, &o, &P) != MPQP_OK) { cudaGetLastError(); return -1.0; }
    double best = -1.0;
    for (int rep = 0; rep < runs; rep++) {
        if (mpqp_plan_run_timed_impl(P, nullptr) != MPQP_OK) { best = -1.0; break; }
        if (cudaEventSynchronize(P->ev1) != cudaSuccess) { cudaGetLastError(); best = -1.0; break; }
        double ms = 0.0;
        for (size_t i = 0; i < P->kname.size(); i++) {
            if (strncmp(P->kname[i], prefix, strlen(prefix))) continue;
            float e = 0;
            if (cudaEventElapsedTime(&e, P->kev[i], P->kev[i + 1]) == cudaSuccess) ms += e;
        }
        if (best < 0 || ms < best) best = ms;
    }
    // a run that overflowed its buffers measured nothing comparable
    Ctl ctl;
    if (best >= 0 && (cudaMemcpy(&ctl, P->B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost) != cudaSuccess || ctl.overflow))
        best = -1.0;
    cudaGetLastError();
    mpqp_plan_destroy(P);
    return best;
}

static void autotune(int n_inst, const mpqp_problem *probs, mpqp_options &o)
{
    const TuneKey key = tune_key(n_inst, probs, o);
    for (const TuneEntry &e : g_tune_cache)
        if (e.key == key) {
            if (!o.tile_w) o.tile_w = e.tile_w;
            if (!o.feas_warps) o.feas_warps = e.feas_warps;
            if (!o.feas_chunk) o.feas_chunk = e.feas_chunk;
            return;
        }
    // the candidates of the whole batch (combinatorial count, under the budgets)
    double est = 0.0;
    for (int i = 0; i < n_inst; i++) {
        const int m = probs[i].m, kmax = std::min(probs[i].k_max, std::min(m, kMaxK));
        double cmk = 1.0, tot = 1.0;
        for (int k = 1; k <= kmax; k++) { cmk = cmk * (double)(m - k + 1) / (double)k; tot += cmk; }
        est += probs[i].budget > 0 ? std::min(tot, (double)probs[i].budget) : tot;
    }
    std::vector<mpqp_problem> slice(probs, probs + n_inst);
    if (est > kTuneWhole)
        for (mpqp_problem &pr : slice) pr.budget = pr.budget > 0 ? std::min(pr.budget, kTuneSlice) : kTuneSlice;
    const int runs = est > 2e7 ? 1 : 2;
    mpqp_options t = o;
    t.autotune = 0;
    t.use_graph = 0;
    t.record = 0;
    t.cand_cap = 0; t.node_cap = 0; t.arena_bytes = 0; t.opt_cap = 0;
    // a candidate replaces the default (the first entry) only when it is at
    // least 2 % faster
    auto better = [](double ms, double best) { return ms >= 0 && (best < 0 || ms < 0.98 * best); };
    int best_w = o.feas_warps ? o.feas_warps : 4, best_c = o.feas_chunk ? o.feas_chunk : 32;
    if (!o.feas_warps || !o.feas_chunk) {
        double best = -1.0;
        const int grid[][2] = {{4, 32}, {4, 16}, {2, 32}, {4, 8}, {2, 16}};
        for (const auto &g : grid) {
            const int w = g[0], c = g[1];
            if ((o.feas_warps && w != o.feas_warps) || (o.feas_chunk && c != o.feas_chunk)) continue;
            t.feas_warps = w; t.feas_chunk = c; t.tile_w = 8;
            const double ms = tune_trial(n_inst, slice.data(), t, "k_feasibility", runs);
            if (better(ms, best)) { best = ms; best_w = w; best_c = c; }
        }
    }
    int best_t = o.tile_w ? o.tile_w : 8;
    if (!o.tile_w && o.precision == MPQP_MIXED) {
        double best = -1.0;
        t.feas_warps = best_w; t.feas_chunk = best_c;
        for (int tw : {8, 16, 32}) {
            t.tile_w = tw;
            const double ms = tune_trial(n_inst, slice.data(), t, "k_opt_screen<dual>", runs);
            if (ms > 0 && better(ms, best)) { best = ms; best_t = tw; }
        }
    }
    if (!o.tile_w) o.tile_w = best_t;
    if (!o.feas_warps) o.feas_warps = best_w;
    if (!o.feas_chunk) o.feas_chunk = best_c;
    g_tune_cache.push_back(TuneEntry{key, o.tile_w, o.feas_warps, o.feas_chunk});
}

static int mpqp_plan_create_impl(int n_inst, const mpqp_problem *probs, const mpqp_options *opt_in, mpqp_plan **out)
{
    std::lock_guard<std::mutex> lk(g_mu);
    *out = nullptr;
    if (n_inst < 1 || !probs) { set_err("no instances"); return MPQP_EINVAL; }
    mpqp_options o;
    if (opt_in) o = *opt_in; else mpqp_default_options(&o);
    const bool tune = o.autotune && (!o.tile_w || !o.feas_warps || !o.feas_chunk);
    if (tune) autotune(n_inst, probs, o);
    const int rc = plan_create_locked(n_inst, probs, &o, out);
    if (rc == MPQP_OK && tune) (*out)->tuned = 1;
    return rc;
}

extern "C" int mpqp_plan_create(int n_inst, const mpqp_problem *probs, const mpqp_options *opt_in, mpqp_plan **out)
{
    try {
        return mpqp_plan_create_impl(n_inst, probs, opt_in, out);
    } catch (...) {
        return host_failure("mpqp_plan_create");
    }
}

static int mpqp_plan_run_impl(mpqp_plan *P, void *stream)
{
    if (!P) return MPQP_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaEventRecord(P->ev0, s));
    if (P->exec) {
        CK(cudaGraphLaunch(P->exec, s));
    } else {
        int rc = enqueue(P, s, true);
        if (rc) return rc;
    }
    CK(cudaEventRecord(P->ev1, s));
    P->ran = true;
    return MPQP_OK;
}

extern "C" int mpqp_plan_run(mpqp_plan *P, void *stream)
{
    try {
        return mpqp_plan_run_impl(P, stream);
    } catch (...) {
        return host_failure("mpqp_plan_run");
    }
}

extern "C" int mpqp_plan_launches(const mpqp_plan *P) { return P ? P->n_launches : 0; }

static int mpqp_plan_run_timed_impl(mpqp_plan *P, void *stream)
{
    if (!P) return MPQP_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaEventRecord(P->ev0, s));
    int rc = enqueue(P, s, true);
    if (rc) return rc;
    CK(cudaEventRecord(P->ev1, s));
    P->ran = true;
    P->timed = true;
    return MPQP_OK;
}

extern "C" int mpqp_plan_run_timed(mpqp_plan *P, void *stream)
{
    try {
        return mpqp_plan_run_timed_impl(P, stream);
    } catch (...) {
        return host_failure("mpqp_plan_run_timed");
    }
}

static int mpqp_plan_kernel_times_impl(mpqp_plan *P, int max_kernels, char *names, double *ms, int *count)
{
    if (!P || !P->timed) { set_err("no timed run"); return MPQP_EINVAL; }
    CK(cudaEventSynchronize(P->ev1));
    std::vector<std::string> nm;
    std::vector<double> t;
    std::vector<int> c;
    for (size_t i = 0; i < P->kname.size(); i++) {
        float e = 0;
        CK(cudaEventElapsedTime(&e, P->kev[i], P->kev[i + 1]));
        size_t j = 0;
        while (j < nm.size() && nm[j] != P->kname[i]) j++;
        if (j == nm.size()) { nm.push_back(P->kname[i]); t.push_back(0); c.push_back(0); }
        t[j] += e;
        c[j] += 1;
    }
    const int n = std::min((int)nm.size(), max_kernels);
    for (int i = 0; i < n; i++) {
        strncpy(names + 64 * i, nm[i].c_str(), 63);
        names[64 * i + 63] = 0;
        ms[i] = t[i];
        count[i] = c[i];
    }
    return n;
}

extern "C" int mpqp_plan_kernel_times(mpqp_plan *P, int max_kernels, char *names, double *ms, int *count)
{
    try {
        return mpqp_plan_kernel_times_impl(P, max_kernels, names, ms, count);
    } catch (...) {
        return host_failure("mpqp_plan_kernel_times");
    }
}

// Device time of the last timed run split into the LP1 phase (reset, level
// 0, enumeration, LP1 and its FP64 certificate / re-solve, level
// bookkeeping) and the optimality phase (screens and FP64 optimality), the
// split main.py:18-20 reads as time_feas / time_opti.
static int phase_times(mpqp_plan *P, double *feas_ms, double *opti_ms)
{
    *feas_ms = *opti_ms = 0.0;
    if (!P || !P->timed) { set_err("no timed run"); return MPQP_EINVAL; }
    CK(cudaEventSynchronize(P->ev1));
    for (size_t i = 0; i < P->kname.size(); i++) {
        float e = 0;
        CK(cudaEventElapsedTime(&e, P->kev[i], P->kev[i + 1]));
        if (!strncmp(P->kname[i], "k_opt", 5)) *opti_ms += e; else *feas_ms += e;
    }
    return MPQP_OK;
}

static uint64_t bit_reverse64(uint64_t x)
{
    x = ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
    x = ((x >> 2) & 0x3333333333333333ULL) | ((x & 0x3333333333333333ULL) << 2);
    x = ((x >> 4) & 0x0F0F0F0F0F0F0F0FULL) | ((x & 0x0F0F0F0F0F0F0F0FULL) << 4);
    x = ((x >> 8) & 0x00FF00FF00FF00FFULL) | ((x & 0x00FF00FF00FF00FFULL) << 8);
    x = ((x >> 16) & 0x0000FFFF0000FFFFULL) | ((x & 0x0000FFFF0000FFFFULL) << 16);
    return (x >> 32) | (x << 32);
}

// Sort keys of the optimal-set records, by record index: the order is
// (grp, ~lo, ~hi) ascending, grp = (inst, level), lo / hi the bit-reversed
// mask words (the complements order the sorted element lists of equal-size
// sets lexicographically).
struct OptKeys {
    std::vector<uint64_t> hi, lo, grp;
    uint64_t or_hi = 0, or_lo = 0, or_grp = 0;   // which bits occur at all
};

static bool opt_key_less(const OptKeys &K, uint32_t a, uint32_t b)
{
    if (K.grp[a] != K.grp[b]) return K.grp[a] < K.grp[b];
    if (K.lo[a] != K.lo[b]) return K.lo[a] > K.lo[b];
    return K.hi[a] > K.hi[b];
}

// Stable LSD radix sort of the record indices [b, e) into out[0, e - b): per
// key all digit histograms in one pass, then a scatter pass per digit that
// varies; digits above the highest bit any key has are skipped.
static void radix_order_range(const OptKeys &K, size_t b, size_t e, uint32_t *out)
{
    const size_t n = e - b;
    std::vector<uint32_t> order(n), tmp(n);
    for (size_t i = 0; i < n; i++) order[i] = (uint32_t)(b + i);
    constexpr int kBits = 11, kBins = 1 << kBits;
    std::vector<uint32_t> hist((size_t)6 * kBins);
    auto phase = [&](const std::vector<uint64_t> &key, uint64_t any, bool flip) {
        if (!any || n < 2) return;
        const int nd = (64 - __builtin_clzll(any) + kBits - 1) / kBits;
        const uint64_t fl = flip ? ~0ULL : 0ULL;
        std::fill(hist.begin(), hist.begin() + (size_t)nd * kBins, 0u);
        for (size_t i = 0; i < n; i++) {
            const uint64_t k = key[order[i]] ^ fl;
            for (int d = 0; d < nd; d++) hist[(size_t)d * kBins + ((k >> (d * kBits)) & (kBins - 1))]++;
        }
        for (int d = 0; d < nd; d++) {
            uint32_t *h = &hist[(size_t)d * kBins];
            const int sh = d * kBits;
            if (h[((key[order[0]] ^ fl) >> sh) & (kBins - 1)] == n) continue;   // all keys share this digit
            uint32_t sum = 0;
            for (int q = 0; q < kBins; q++) { const uint32_t c = h[q]; h[q] = sum; sum += c; }
            for (size_t i = 0; i < n; i++) {
                const uint32_t r = order[i];
                tmp[h[((key[r] ^ fl) >> sh) & (kBins - 1)]++] = r;
            }
            order.swap(tmp);
        }
    };
    // least significant first: high mask word, low mask word, (inst, level);
    // a zero word is skipped whole (every mask of an m <= 64 problem)
    phase(K.hi, K.or_hi, true);
    phase(K.lo, K.or_lo, true);
    phase(K.grp, K.or_grp, false);
    std::copy(order.begin(), order.end(), out);
}

// f(0) .. f(T-1) on up to T threads (the calling thread included); when a
// thread cannot be started, the calling thread runs the rest.  An exception
// of any f(t) is rethrown in the calling thread once all have finished.
template <typename F>
static void run_parallel(unsigned T, F f)
{
    std::vector<std::exception_ptr> err(T);
    auto guarded = [&](unsigned t) {
        try { f(t); } catch (...) { err[t] = std::current_exception(); }
    };
    std::vector<std::thread> th;
    try {
        for (unsigned t = 1; t < T; t++) th.emplace_back(guarded, t);
    } catch (...) {
    }
    guarded(0u);
    for (unsigned t = (unsigned)th.size() + 1; t < T; t++) guarded(t);
    for (std::thread &x : th) x.join();
    for (const std::exception_ptr &e : err)
        if (e) std::rethrow_exception(e);
}

// indices of the optimal-set records in (inst, level, set) order
static std::vector<uint32_t> sorted_opt_order(const OptRec *ov, size_t n)
{
    OptKeys K;
    K.hi.resize(n); K.lo.resize(n); K.grp.resize(n);
    for (size_t i = 0; i < n; i++) {
        K.hi[i] = bit_reverse64(ov[i].hi);
        K.lo[i] = bit_reverse64(ov[i].lo);
        K.grp[i] = ((uint64_t)(uint32_t)ov[i].inst << 32) | (uint32_t)ov[i].level;
        K.or_hi |= K.hi[i]; K.or_lo |= K.lo[i]; K.or_grp |= K.grp[i];
    }
    std::vector<uint32_t> order(n);
    // large result sets: T contiguous chunks sorted concurrently, then merged
    // pairwise; a merge takes the earlier chunk first on ties, so the result
    // is the same stable order as one sort
    unsigned T = std::thread::hardware_concurrency();
    T = n >= ((size_t)1 << 16) ? std::min(std::max(T, 1u), 8u) : 1u;
    if (T == 1) {
        radix_order_range(K, 0, n, order.data());
        return order;
    }
    std::vector<size_t> cut(T + 1);
    for (unsigned t = 0; t <= T; t++) cut[t] = n * t / T;
    run_parallel(T, [&](unsigned t) { radix_order_range(K, cut[t], cut[t + 1], order.data() + cut[t]); });
    std::vector<uint32_t> tmp(n);
    const auto less = [&K](uint32_t a, uint32_t b) { return opt_key_less(K, a, b); };
    for (unsigned width = 1; width < T; width *= 2) {
        const unsigned pairs = (T + 2 * width - 1) / (2 * width);
        run_parallel(pairs, [&](unsigned q) {
            const unsigned t = q * 2 * width;
            const size_t a = cut[t], m = cut[std::min(t + width, T)], e = cut[std::min(t + 2 * width, T)];
            std::merge(order.begin() + a, order.begin() + m, order.begin() + m, order.begin() + e, tmp.begin() + a, less);
        });
        order.swap(tmp);
    }
    return order;
}

// The body of mpqp_plan_results: R is built here; *complete is set only when
// the whole result is in R (the caller frees a partial one).  Host
// allocation failures throw std::bad_alloc.
static int plan_results_impl(mpqp_plan *P, mpqp_batch_result *&R, bool *complete)
{
    CK(cudaEventSynchronize(P->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, P->ev0, P->ev1));
    P->last_ms = ms;
    Ctl ctl;
    CK(cudaMemcpy(&ctl, P->B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    std::vector<InstCtl> ic(P->n_inst);
    CK(cudaMemcpy(ic.data(), P->B.ictl, sizeof(InstCtl) * P->n_inst, cudaMemcpyDeviceToHost));
    R = (mpqp_batch_result *)calloc(1, sizeof(mpqp_batch_result));
    if (!R) throw std::bad_alloc();
    R->n_inst = P->n_inst;
    R->device_ms = ms;
    R->overflow = ctl.overflow;
    R->status = ctl.overflow ? ((ctl.overflow & OV_WAIT) ? MPQP_ECUDA : MPQP_ECAPACITY) : MPQP_OK;
    if (ctl.overflow & OV_WAIT) set_err("a bulk copy did not complete within its bounded wait");
    else if (ctl.overflow) set_err("device buffer overflow (bits " + std::to_string(ctl.overflow) + ")");
    R->inst = (mpqp_inst_stats *)calloc(P->n_inst, sizeof(mpqp_inst_stats));
    if (!R->inst) throw std::bad_alloc();
    int nlev = 0;
    for (int i = 0; i < P->n_inst; i++) {
        mpqp_inst_stats &s = R->inst[i];
        s.candidates = ic[i].cum_cand; s.pruned = ic[i].pruned; s.feasible = ic[i].feasible;
        s.optimal = ic[i].optimal; s.regions = ic[i].region; s.lp1_pivots = ic[i].lp1_piv;
        s.lp2_pivots = ic[i].lp2_piv; s.cheb_pivots = ic[i].cheb_piv; s.fallback_lp1 = ic[i].fb_lp1;
        s.fallback_opt = ic[i].fb_opt; s.stored = ic[i].stored;
        s.lp1_certified = ic[i].cert_lp1; s.lp1_cert_missed = ic[i].cert_miss; s.lp1_cert_freevar = ic[i].cert_free;
        s.lp1_parents = ic[i].parents; s.lp1_parent_bytes = ic[i].par_bytes; s.lp1_store_bytes = ic[i].store_bytes;
        s.lp1_cold = ic[i].lp1_cold; s.nodes_without_tableau = ic[i].no_tab;
        s.lp2_first_stage_lps = ic[i].s0_lps; s.lp2_first_stage_pivots = ic[i].s0_piv;
        s.lp2_warm_offered = ic[i].warm_try; s.lp2_warm_started = ic[i].warm_used;
        s.lp2_certified = ic[i].cert_lp2;
        s.lp1_vertex_checked = ic[i].vtx_lp1;
        s.feasible_digest = ic[i].feas_digest; s.optimal_digest = ic[i].opt_digest;
        s.region_digest = ic[i].reg_digest;
        s.last_level = ic[i].last_level; s.truncated = ic[i].truncated;
        nlev = std::max(nlev, ic[i].last_level + 1);
    }
    R->n_levels = nlev;
    R->split_levels = (int)ctl.split_levels;
    long long nopt = std::min(ctl.n_opt, P->B.opt_cap);
    std::vector<OptRec> ov(nopt);
    if (nopt) CK(cudaMemcpy(ov.data(), P->B.opt, sizeof(OptRec) * nopt, cudaMemcpyDeviceToHost));
    // order (inst, level, set), sets of one size in the lexicographic order of
    // their sorted element lists: for equal-size sets that is the ascending
    // order of the bit-reversed, complemented masks.  An LSD radix sort on
    // those integer keys (high mask word, low mask word, then instance and
    // level) moves indices, not records, and skips every digit that all sets
    // share.
    std::vector<uint32_t> order = sorted_opt_order(ov.data(), ov.size());
    R->n_opt = nopt;
    R->opt = (mpqp_opt_set *)calloc(nopt ? nopt : 1, sizeof(mpqp_opt_set));
    if (!R->opt) throw std::bad_alloc();
    for (long long i = 0; i < nopt; i++) {
        const OptRec &v = ov[order[i]];
        mpqp_opt_set &o = R->opt[i];
        o.mask_lo = v.lo; o.mask_hi = v.hi; o.inst = v.inst; o.level = v.level;
        o.t = v.t; o.r = v.r; o.region = v.region; o.fp64 = v.fp64; o.rec = v.rec; o.err = v.err;
    }
    R->h2d_bytes = P->h2d_bytes;
    R->tile_w = P->tile_w; R->feas_warps = P->feas_warps; R->feas_chunk = P->feas_chunk; R->tuned = P->tuned;
    R->d2h_bytes = (long long)(sizeof(Ctl) + sizeof(InstCtl) * P->n_inst + sizeof(OptRec) * nopt);
    if (P->B.rec) {
        long long nrec = std::min(ctl.rec_base, P->B.rec_cap);
        R->d2h_bytes += (long long)sizeof(CandRec) * nrec;
        R->n_rec = nrec;
        R->rec = malloc(sizeof(CandRec) * (nrec ? nrec : 1));
        if (!R->rec) throw std::bad_alloc();
        if (nrec) CK(cudaMemcpy(R->rec, P->B.rec, sizeof(CandRec) * nrec, cudaMemcpyDeviceToHost));
    }
    *complete = true;
    return R->status;
}

extern "C" int mpqp_plan_results(mpqp_plan *P, mpqp_batch_result **out)
{
    *out = nullptr;
    if (!P || !P->ran) { set_err("plan has not run"); return MPQP_EINVAL; }
    mpqp_batch_result *R = nullptr;
    bool complete = false;
    int rc;
    try {
        rc = plan_results_impl(P, R, &complete);
    } catch (const std::bad_alloc &) {
        set_err("host memory allocation failed while reading the results back");
        rc = MPQP_ENOMEM;
    } catch (...) {
        set_err("host error while reading the results back");
        rc = MPQP_ENOMEM;
    }
    if (!complete) {
        mpqp_batch_free(R);
        return rc;
    }
    *out = R;
    return rc;
}

extern "C" void mpqp_plan_destroy(mpqp_plan *P)
{
    if (!P) return;
    free_plan_mem(P);
    delete P;
}

extern "C" void mpqp_batch_free(mpqp_batch_result *R)
{
    if (!R) return;
    free(R->inst);
    free(R->opt);
    free(R->rec);
    free(R);
}

extern "C" int mpqp_solve_batch(int n_inst, const mpqp_problem *probs, const mpqp_options *opt,
                                mpqp_batch_result **out)
{
    *out = nullptr;
    mpqp_plan *P = nullptr;
    int rc = mpqp_plan_create(n_inst, probs, opt, &P);
    if (rc) return rc;
    rc = mpqp_plan_run(P, nullptr);
    if (!rc) rc = mpqp_plan_results(P, out);
    mpqp_plan_destroy(P);
    return rc;
}

// ---------------------------------------------------------------------
// region laws
// ---------------------------------------------------------------------
extern "C" long long mpqp_region_laws_stride(const mpqp_problem *pr)
{
    const long long P1 = pr->p + 1;
    return (long long)pr->m * P1 + (long long)pr->n * P1 + (long long)(pr->m + pr->ncp) * P1;
}

static int mpqp_region_laws_impl(const mpqp_problem *prob, long long n_sets, const uint64_t *masks, double *laws,
                                 int *sizes, double *radius, double *err)
{
    if (!prob || n_sets < 0 || (n_sets && (!masks || !laws || !sizes))) { set_err("bad arguments"); return MPQP_EINVAL; }
    if (n_sets == 0) return MPQP_OK;
    const int kcap = std::min(prob->m, std::min(prob->n, kMaxK));
    for (long long i = 0; i < n_sets; i++) {
        const uint64_t lo = masks[2 * i], hi = masks[2 * i + 1];
        const int k = __builtin_popcountll(lo) + __builtin_popcountll(hi);
        const bool out_of_range = prob->m < 64 ? ((lo >> prob->m) != 0 || hi != 0)
                                               : (prob->m < 128 && (hi >> (prob->m - 64)) != 0);
        if (k > kcap || out_of_range) { set_err("active set " + std::to_string(i) + " is out of range"); return MPQP_EINVAL; }
    }
    mpqp_options o;
    mpqp_default_options(&o);
    o.use_graph = 0;
    o.cand_cap = 1024;
    o.arena_bytes = 1 << 20;
    mpqp_problem pr = *prob;
    pr.k_max = 0;
    mpqp_plan *P = nullptr;
    int rc = mpqp_plan_create(1, &pr, &o, &P);
    if (rc) return rc;
    // sizes for any set of the instance: use the instance's own bounds
    SlotDims sd = P->sd;
    sd.maxK = std::max(1, kcap);
    const long long stride = mpqp_region_laws_stride(prob);
    uint64_t *dm = nullptr; double *dl = nullptr, *dr = nullptr, *de = nullptr; int *ds = nullptr;
    size_t smem = 4 * laws_smem_per_warp(sd);
    int grid = 0;
    rc = grid_for(kernel_ptr("laws"), smem, &grid);
    if (!rc) {
        CK(cudaMalloc(&dm, sizeof(uint64_t) * 2 * n_sets));
        CK(cudaMalloc(&dl, sizeof(double) * stride * n_sets));
        CK(cudaMalloc(&ds, sizeof(int) * 4 * n_sets));
        if (radius) CK(cudaMalloc(&dr, sizeof(double) * n_sets));
        if (err) CK(cudaMalloc(&de, sizeof(double) * n_sets));
        CK(cudaMemcpy(dm, masks, sizeof(uint64_t) * 2 * n_sets, cudaMemcpyHostToDevice));
        CK(launch_region_laws_r(P->B, P->tol, sd, dm, n_sets, dl, ds, stride, dr, de, grid, smem, nullptr));
        CK(cudaMemcpy(laws, dl, sizeof(double) * stride * n_sets, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(sizes, ds, sizeof(int) * 4 * n_sets, cudaMemcpyDeviceToHost));
        if (radius) CK(cudaMemcpy(radius, dr, sizeof(double) * n_sets, cudaMemcpyDeviceToHost));
        if (err) CK(cudaMemcpy(err, de, sizeof(double) * n_sets, cudaMemcpyDeviceToHost));
        cudaFree(dm); cudaFree(dl); cudaFree(ds);
        if (dr) cudaFree(dr);
        if (de) cudaFree(de);
    }
    mpqp_plan_destroy(P);
    return rc;
}

extern "C" int mpqp_region_laws(const mpqp_problem *prob, long long n_sets, const uint64_t *masks, double *laws,
                                int *sizes)
{
    try {
        return mpqp_region_laws_impl(prob, n_sets, masks, laws, sizes, nullptr, nullptr);
    } catch (...) {
        return host_failure("mpqp_region_laws");
    }
}

extern "C" int mpqp_critical_regions(const mpqp_problem *prob, long long n_sets, const uint64_t *masks, double *laws,
                                     int *sizes, double *radius, double *err)
{
    try {
        if (!radius && n_sets > 0) { set_err("radius is NULL"); return MPQP_EINVAL; }
        return mpqp_region_laws_impl(prob, n_sets, masks, laws, sizes, radius, err);
    } catch (...) {
        return host_failure("mpqp_critical_regions");
    }
}

// ---------------------------------------------------------------------
// drop-in boundary
// ---------------------------------------------------------------------
static GPUResults *g_last = nullptr;

static void free_gpu_results(GPUResults *r)
{
    if (!r) return;
    free(r->active_sets);
    free(r->t_star);
    free(r->radius);
    free(r->is_region);
    free(r->law_error);
    free(r);
}

extern "C" void mpqp_free(GPUResults *res)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (res == g_last) g_last = nullptr;
    free_gpu_results(res);
}

static GPUResults *error_result(int status)
{
    GPUResults *r = (GPUResults *)calloc(1, sizeof(GPUResults));
    if (!r) return nullptr;   // out of host memory: the caller gets NULL
    r->status = status;
    r->active_sets = (int *)calloc(1, sizeof(int));
    r->t_star = (double *)calloc(1, sizeof(double));
    r->radius = (double *)calloc(1, sizeof(double));
    r->is_region = (int *)calloc(1, sizeof(int));
    r->law_error = (double *)calloc(1, sizeof(double));
    return r;
}

// Rebuild (Q, c, H, A, b, F, At, bt) from the LP matrices of main.py:87-128.
static int unpack_lp(const double *AxT, int n_c, int n_x, int n_t, const double *A1, const double *xb1, int M1,
                     int N1, const double *A2, const double *xb2, int M2, int N2, int n_eqs,
                     std::vector<double> &Q, std::vector<double> &c, std::vector<double> &H, std::vector<double> &A,
                     std::vector<double> &b, std::vector<double> &F, std::vector<double> &At, std::vector<double> &bt,
                     int &n_cp)
{
    if (!A1 || !xb1 || !A2 || !xb2 || n_c < 1 || n_x < 1 || n_t < 1) { set_err("null or empty LP data"); return MPQP_EINVAL; }
    n_cp = M1 - n_c;
    if (n_cp < 1 || N1 != n_x + n_t + 1 + M1 || M2 != 2 * n_c + 1 + n_cp + n_x ||
        N2 != n_x + n_t + n_c + 2 + M2 || n_eqs != n_c + n_x) {
        set_err("LP dimensions do not match the reference layout (main.py:87-118)");
        return MPQP_ELAYOUT;
    }
    A.assign((size_t)n_c * n_x, 0); F.assign((size_t)n_c * n_t, 0); b.assign(n_c, 0);
    At.assign((size_t)n_cp * n_t, 0); bt.assign(n_cp, 0);
    for (int i = 0; i < n_c; i++) {
        for (int j = 0; j < n_x; j++) A[i * n_x + j] = A1[i + (size_t)j * M1];
        for (int j = 0; j < n_t; j++) F[i * n_t + j] = -A1[i + (size_t)(n_x + j) * M1];
        b[i] = xb1[i];
    }
    for (int i = 0; i < n_cp; i++) {
        for (int j = 0; j < n_t; j++) At[i * n_t + j] = A1[(n_c + i) + (size_t)(n_x + j) * M1];
        bt[i] = xb1[n_c + i];
    }
    if (AxT) {
        for (int i = 0; i < n_c; i++)
            for (int j = 0; j < n_x; j++)
                if (AxT[j + (size_t)i * n_x] != A[i * n_x + j]) { set_err("AxT differs from A1[:n_c,:n_x]^T"); return MPQP_ELAYOUT; }
    }
    Q.assign((size_t)n_x * n_x, 0); H.assign((size_t)n_x * n_t, 0); c.assign(n_x, 0);
    const int r0 = n_c + 1 + n_cp;
    for (int i = 0; i < n_x; i++) {
        const int r = r0 + i;
        // rows with -c_i < 0 were negated (main.py:112-114); the multiplier
        // block of the row is s * A[:, i] (main.py:106), which fixes s; Q_ii
        // (positive for an mpQP, zero for an mpLP) only when that column is 0
        const double *lam = A2 + r + (size_t)(n_x + n_t) * M2;
        int jm = -1;
        double am = 0.0;
        for (int j = 0; j < n_c; j++)
            if (std::fabs(A[(size_t)j * n_x + i]) > am) { am = std::fabs(A[(size_t)j * n_x + i]); jm = j; }
        const double diag = A2[r + (size_t)i * M2];
        double s;
        if (jm >= 0) s = (lam[(size_t)jm * M2] > 0.0) == (A[(size_t)jm * n_x + i] > 0.0) ? 1.0 : -1.0;
        else if (diag != 0.0) s = diag > 0.0 ? 1.0 : -1.0;
        else { set_err("LP2 stationarity row: neither A nor Q fixes its sign"); return MPQP_ELAYOUT; }
        for (int j = 0; j < n_c; j++)
            if (lam[(size_t)j * M2] != s * A[(size_t)j * n_x + i]) {
                set_err("LP2 stationarity row does not hold A^T (main.py:106)");
                return MPQP_ELAYOUT;
            }
        for (int j = 0; j < n_x; j++) Q[i * n_x + j] = s * A2[r + (size_t)j * M2];
        for (int j = 0; j < n_t; j++) H[i * n_t + j] = s * A2[r + (size_t)(n_x + j) * M2];
        c[i] = -s * xb2[r];
    }
    return MPQP_OK;
}

static int mpqp_unpack_lp_impl(const double *AxT, int n_c, int n_x, int n_t, const double *A1, const double *xb1,
                               int M1, int N1, const double *A2, const double *xb2, int M2, int N2, int n_eqs,
                               double *Q, double *c, double *H, double *A, double *b, double *F, double *At,
                               double *bt, int *n_cp)
{
    std::vector<double> q, cc, h, a, bb, f, at, btv;
    int ncp = 0;
    const int rc = unpack_lp(AxT, n_c, n_x, n_t, A1, xb1, M1, N1, A2, xb2, M2, N2, n_eqs, q, cc, h, a, bb, f, at,
                             btv, ncp);
    if (n_cp) *n_cp = ncp;
    if (rc) return rc;
    auto out = [](double *dst, const std::vector<double> &v) { if (dst) memcpy(dst, v.data(), sizeof(double) * v.size()); };
    out(Q, q); out(c, cc); out(H, h); out(A, a); out(b, bb); out(F, f); out(At, at); out(bt, btv);
    return MPQP_OK;
}

extern "C" int mpqp_unpack_lp(const double *AxT, int n_c, int n_x, int n_t, const double *A1, const double *xb1,
                              int M1, int N1, const double *A2, const double *xb2, int M2, int N2, int n_eqs,
                              double *Q, double *c, double *H, double *A, double *b, double *F, double *At,
                              double *bt, int *n_cp)
{
    try {
        return mpqp_unpack_lp_impl(AxT, n_c, n_x, n_t, A1, xb1, M1, N1, A2, xb2, M2, N2, n_eqs, Q, c, H, A, b, F,
                                   At, bt, n_cp);
    } catch (...) {
        return host_failure("mpqp_unpack_lp");
    }
}

static GPUResults *mpqp_impl(const double *AxT, int n_c, int n_x, int n_t, int k_min, int k_max, int extra_batches,
                             const double *A1, const double *xb1, const int *b1, int M1, int N1, const double *A2,
                             const double *xb2, const int *b2, const int *non_b2, int M2, int N2, int n_eqs,
                             int reserved_memory)
{
    (void)b1; (void)b2; (void)non_b2; (void)extra_batches;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_last) { free_gpu_results(g_last); g_last = nullptr; }
    }
    std::vector<double> Q, c, H, A, b, F, At, bt;
    int n_cp = 0;
    int rc = unpack_lp(AxT, n_c, n_x, n_t, A1, xb1, M1, N1, A2, xb2, M2, N2, n_eqs, Q, c, H, A, b, F, At, bt, n_cp);
    if (rc) return g_last = error_result(rc);
    mpqp_problem pr;
    memset(&pr, 0, sizeof(pr));
    pr.n = n_x; pr.m = n_c; pr.p = n_t; pr.ncp = n_cp;
    pr.k_min = k_min; pr.k_max = k_max;
    pr.Q = Q.data(); pr.c = c.data(); pr.H = H.data(); pr.A = A.data(); pr.b = b.data(); pr.F = F.data();
    pr.At = At.data(); pr.bt = bt.data();
    mpqp_options o;
    mpqp_default_options(&o);
    // mixed precision (FP32 pivots, FP64 certificates and re-solves; verdicts
    // identical to the FP64 path) unless MPQP_PRECISION=fp64
    o.precision = MPQP_MIXED;
    const char *env = getenv("MPQP_PRECISION");
    if (env && (!strcmp(env, "fp64") || !strcmp(env, "0"))) o.precision = MPQP_FP64;
    // one run: launched without a graph, with an event before every launch,
    // so that the device time splits into its LP1 and optimality phases
    o.use_graph = 0;
    // MPQP_ARENA_BYTES: a cap on the LP1 tableau arena (levels beyond it are
    // split: see n_splits)
    const char *ab = getenv("MPQP_ARENA_BYTES");
    if (ab && atoll(ab) > 0) o.arena_bytes = atoll(ab);
    if (reserved_memory > 0) {
        size_t fb = 0, tb = 0;
        if (cudaMemGetInfo(&fb, &tb) == cudaSuccess) {
            fb = free_device_bytes();
            const double keep = (double)reserved_memory * 1024.0 * 1024.0;
            o.mem_fraction = std::max(0.05, std::min(0.6, ((double)fb - keep) / std::max(1.0, (double)fb)));
        }
    }
    mpqp_batch_result *R = nullptr;
    double feas_ms = 0.0, opti_ms = 0.0;
    {
        mpqp_plan *P = nullptr;
        rc = mpqp_plan_create(1, &pr, &o, &P);
        if (!rc) rc = mpqp_plan_run_timed(P, nullptr);
        if (!rc) rc = mpqp_plan_results(P, &R);
        if (!rc) rc = phase_times(P, &feas_ms, &opti_ms);
        mpqp_plan_destroy(P);
    }
    if (rc || !R) {
        mpqp_batch_free(R);
        return g_last = error_result(rc ? rc : MPQP_ECUDA);
    }
    GPUResults *G = (GPUResults *)calloc(1, sizeof(GPUResults));
    if (!G) { mpqp_batch_free(R); throw std::bad_alloc(); }
    const long long nf = R->n_opt;
    const int kmin = k_min < 0 ? 0 : k_min;
    long long nsel = 0;
    for (long long i = 0; i < nf; i++) if (R->opt[i].level >= kmin) nsel++;
    G->n_batches = R->n_levels;
    // 1 + the levels whose feasible sets did not all keep an LP1 tableau in
    // the arena (their children's LP1 started from the root instead)
    G->n_splits = 1 + R->split_levels;
    G->n_feasible_lps = (int)R->inst[0].feasible;
    G->n_final_lps = (int)nsel;
    G->time_GPU = R->device_ms * 1e-3;
    G->time_feas = feas_ms * 1e-3;
    G->time_opti = opti_ms * 1e-3;
    G->status = R->status;
    G->n_candidates = R->inst[0].candidates;
    G->n_pruned = R->inst[0].pruned;
    G->active_sets = (int *)malloc(sizeof(int) * (size_t)(nsel ? nsel : 1) * n_x);
    G->t_star = (double *)malloc(sizeof(double) * (nsel ? nsel : 1));
    G->radius = (double *)malloc(sizeof(double) * (nsel ? nsel : 1));
    G->is_region = (int *)malloc(sizeof(int) * (nsel ? nsel : 1));
    G->law_error = (double *)malloc(sizeof(double) * (nsel ? nsel : 1));
    if (!G->active_sets || !G->t_star || !G->radius || !G->is_region || !G->law_error) {
        free_gpu_results(G);
        mpqp_batch_free(R);
        throw std::bad_alloc();   // the exported wrapper returns an MPQP_ENOMEM result
    }
    long long w = 0;
    int nreg = 0;
    for (long long i = 0; i < nf; i++) {
        const mpqp_opt_set &o2 = R->opt[i];
        if (o2.level < kmin) continue;
        int *row = G->active_sets + w * n_x;
        int e = 0;
        for (int j = 0; j < 128 && e < n_x; j++) {
            const bool on = j < 64 ? ((o2.mask_lo >> j) & 1) : ((o2.mask_hi >> (j - 64)) & 1);
            if (on) row[e++] = j;
        }
        for (; e < n_x; e++) row[e] = -1;
        G->t_star[w] = o2.t;
        G->radius[w] = o2.r;
        G->is_region[w] = o2.region;
        G->law_error[w] = o2.err;
        nreg += o2.region;
        w++;
    }
    G->n_regions = nreg;
    mpqp_batch_free(R);
    std::lock_guard<std::mutex> lk(g_mu);
    g_last = G;
    return G;
}

extern "C" GPUResults *mpqp(const double *AxT, int n_c, int n_x, int n_t, int k_min, int k_max, int extra_batches,
                            const double *A1, const double *xb1, const int *b1, int M1, int N1, const double *A2,
                            const double *xb2, const int *b2, const int *non_b2, int M2, int N2, int n_eqs,
                            int reserved_memory)
{
    try {
        return mpqp_impl(AxT, n_c, n_x, n_t, k_min, k_max, extra_batches, A1, xb1, b1, M1, N1, A2, xb2, b2, non_b2,
                         M2, N2, n_eqs, reserved_memory);
    } catch (...) {
        host_failure("mpqp");
        try {
            return g_last = error_result(MPQP_ENOMEM);
        } catch (...) {
            return nullptr;
        }
    }
}

extern "C" void warm_up(void)
{
    // Smallest meaningful problem: n = 1, m = 2, p = 1, box |theta| <= 1.
    static const double Q[1] = {1.0}, c[1] = {0.5}, H[1] = {1.0}, A[2] = {1.0, -1.0}, b[2] = {1.0, 1.0},
                        F[2] = {0.5, -0.5}, At[2] = {1.0, -1.0}, bt[2] = {1.0, 1.0};
    mpqp_problem pr = {1, 2, 1, 2, 0, 1, 0, Q, c, H, A, b, F, At, bt};
    mpqp_options o;
    mpqp_default_options(&o);
    o.cand_cap = 1024;
    o.arena_bytes = 1 << 20;
    mpqp_batch_result *R = nullptr;
    mpqp_solve_batch(1, &pr, &o, &R);
    mpqp_batch_free(R);
}

extern "C" int mpqp_release_cached_memory(void)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); set_err("cudaGetDevice failed"); return MPQP_ECUDA; }
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (dev >= 0 && dev < 64 && g_pools[dev]) {
        cudaDeviceSynchronize();
        if (cudaMemPoolTrimTo(g_pools[dev], 0) != cudaSuccess) {
            set_err(std::string("cudaMemPoolTrimTo: ") + cudaGetErrorString(cudaGetLastError()));
            return MPQP_ECUDA;
        }
    }
    return MPQP_OK;
}

extern "C" const char *mpqp_version(void) { return "mpqp_gb300 0.1 (sm_103a)"; }

extern "C" const char *mpqp_last_error(void) { return g_err.c_str(); }
