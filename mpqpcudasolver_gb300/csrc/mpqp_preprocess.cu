// Constraint reduction before the enumeration: the steps that the reference's
// MPQPProb.process_constraints takes from ppopt 1.5.1 (utils.py:163-190) --
// zero rows, duplicate rows, implicit equalities, redundant rows -- on the
// rows of [A -F; 0 At] u <= [b; bt], u = (x, theta).  The row comparisons
// are O(rows^2 (n+p)) host work; the redundancy test is one FP64 LP per row,
// solved on the device, one warp per row (k_redundancy).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/mpqp_gb300.h"
#include "mpqp_internal.h"

namespace mq {
size_t redundancy_smem_bytes(int nrows, int ld);
cudaError_t launch_redundancy(const double *M, const double *d, int nrows, int nv, int ld, const int *check, int n_check,
                              double tol, const Tol &lt, int max_piv, int *out, int grid, size_t smem, cudaStream_t s);
void set_error_text(const char *msg);
}  // namespace mq

using namespace mq;

namespace {

constexpr double kZeroNorm = 1e-12;     // a row whose x- and theta-parts have a smaller 2-norm is zero
constexpr double kSameRow = 1e-16;      // squared distance of normalised rows treated as equal
constexpr double kRedundantTol = 1e-9;  // max a_i u <= d_i + this: redundant (normalised rows)

int fail(int rc, const std::string &msg)
{
    set_error_text(msg.c_str());
    return rc;
}

struct DevMem {
    std::vector<void *> ptrs;
    ~DevMem() { for (void *p : ptrs) cudaFree(p); }
    template <typename T> T *alloc(size_t n)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T *)p;
    }
};

}  // namespace

static int mpqp_reduce_constraints_impl(const mpqp_problem *prob, int *row_status)
{
    if (!prob || !row_status) return fail(MPQP_EINVAL, "mpqp_reduce_constraints: null argument");
    const mpqp_problem &P = *prob;
    const int n = P.n, m = P.m, p = P.p, ncp = P.ncp, nv = n + p;
    if (n < 1 || m < 0 || p < 1 || ncp < 0 || !P.A || !P.b || !P.F || (ncp > 0 && (!P.At || !P.bt)))
        return fail(MPQP_EINVAL, "mpqp_reduce_constraints: bad sizes or pointers");
    const int R = m + ncp;
    if (R + nv > 255) return fail(MPQP_EINVAL, "mpqp_reduce_constraints: m + ncp + n + p must be at most 255");
    for (int i = 0; i < m; i++)
        if (!(P.b[i] >= 0.0)) return fail(MPQP_EORIGIN, "mpqp_reduce_constraints: b has a negative entry");
    for (int i = 0; i < ncp; i++)
        if (!(P.bt[i] >= 0.0)) return fail(MPQP_EORIGIN, "mpqp_reduce_constraints: CRb has a negative entry");

    // normalised rows [a | d]: a = [A_i, -F_i] / ||.|| or [0, At_i] / ||.||
    std::vector<double> a((size_t)R * nv, 0.0), d(R, 0.0);
    for (int r = 0; r < R; r++) {
        double *ar = a.data() + (size_t)r * nv;
        if (r < m) {
            for (int j = 0; j < n; j++) ar[j] = P.A[(size_t)r * n + j];
            for (int j = 0; j < p; j++) ar[n + j] = -P.F[(size_t)r * p + j];
            d[r] = P.b[r];
        } else {
            for (int j = 0; j < p; j++) ar[n + j] = P.At[(size_t)(r - m) * p + j];
            d[r] = P.bt[r - m];
        }
        double s = 0.0;
        for (int j = 0; j < nv; j++) s += ar[j] * ar[j];
        const double nrm = std::sqrt(s);
        row_status[r] = MPQP_ROW_KEPT;
        if (!(nrm > kZeroNorm)) { row_status[r] = MPQP_ROW_ZERO; continue; }
        for (int j = 0; j < nv; j++) ar[j] /= nrm;
        d[r] /= nrm;
    }
    auto dist2 = [&](int r, int s, double sign) {
        const double *x = a.data() + (size_t)r * nv, *y = a.data() + (size_t)s * nv;
        double acc = 0.0;
        for (int j = 0; j < nv; j++) { const double t = x[j] - sign * y[j]; acc += t * t; }
        const double t = d[r] - sign * d[s];
        return acc + t * t;
    };
    // duplicates within each block (A's rows, At's rows), earlier row kept
    for (int r = 0; r < R; r++) {
        if (row_status[r] != MPQP_ROW_KEPT) continue;
        const int lo = r < m ? 0 : m;
        for (int s = lo; s < r; s++)
            if (row_status[s] != MPQP_ROW_ZERO && row_status[s] != MPQP_ROW_DUPLICATE && dist2(r, s, 1.0) < kSameRow) {
                row_status[r] = MPQP_ROW_DUPLICATE;
                break;
            }
    }
    // implicit equalities among A's rows: r the negation of an earlier s
    for (int r = 0; r < m; r++) {
        if (row_status[r] != MPQP_ROW_KEPT) continue;
        for (int s = 0; s < r; s++)
            if ((row_status[s] == MPQP_ROW_KEPT || row_status[s] == MPQP_ROW_EQUALITY) && dist2(r, s, -1.0) < kSameRow) {
                row_status[r] = MPQP_ROW_EQUALITY_PAIR;
                row_status[s] = MPQP_ROW_EQUALITY;
                break;
            }
    }
    // redundancy: LP rows = every row that is neither zero nor a duplicate
    // (both rows of an equality pair stay, so the pair acts as an equality);
    // checked rows = the rows still kept
    std::vector<int> lp_rows, check, check_pos;
    std::vector<int> lp_index(R, -1);
    for (int r = 0; r < R; r++)
        if (row_status[r] != MPQP_ROW_ZERO && row_status[r] != MPQP_ROW_DUPLICATE) {
            lp_index[r] = (int)lp_rows.size();
            lp_rows.push_back(r);
        }
    for (int r = 0; r < R; r++)
        if (row_status[r] == MPQP_ROW_KEPT) { check.push_back(lp_index[r]); check_pos.push_back(r); }
    const int nrows = (int)lp_rows.size(), n_check = (int)check.size();
    if (n_check == 0) return MPQP_OK;
    std::vector<double> M((size_t)nrows * nv), dd(nrows);
    for (int i = 0; i < nrows; i++) {
        for (int j = 0; j < nv; j++) M[(size_t)i * nv + j] = a[(size_t)lp_rows[i] * nv + j];
        dd[i] = d[lp_rows[i]];
    }
    DevMem mem;
    double *dM = mem.alloc<double>(M.size()), *dd_dev = mem.alloc<double>(dd.size());
    int *dcheck = mem.alloc<int>(n_check), *dout = mem.alloc<int>(n_check);
    if (!dM || !dd_dev || !dcheck || !dout) return fail(MPQP_ENOMEM, "mpqp_reduce_constraints: device allocation failed");
    if (cudaMemcpy(dM, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dd_dev, dd.data(), dd.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dcheck, check.data(), check.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(MPQP_ECUDA, "mpqp_reduce_constraints: upload failed");
    Tol lt{};
    lt.tol_piv = 1e-9;
    lt.tol_dj = 1e-9;
    lt.degen_switch = 8;
    const int ld = (nv + 1) | 1;   // odd FP64 row stride: conflict-free scalar access
    const size_t smem = redundancy_smem_bytes(nrows, ld);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = n_check < 8 * sms ? n_check : 8 * sms;
    const int max_piv = 4 * (nrows + nv) + 64;
    cudaError_t e = launch_redundancy(dM, dd_dev, nrows, nv, ld, dcheck, n_check, kRedundantTol, lt, max_piv, dout,
                                      grid, smem, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(MPQP_ECUDA, std::string("mpqp_reduce_constraints: ") + cudaGetErrorString(e));
    std::vector<int> out(n_check);
    if (cudaMemcpy(out.data(), dout, n_check * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(MPQP_ECUDA, "mpqp_reduce_constraints: download failed");
    for (int c = 0; c < n_check; c++)
        if (out[c]) row_status[check_pos[c]] = MPQP_ROW_REDUNDANT;
    return MPQP_OK;
}

extern "C" int mpqp_reduce_constraints(const mpqp_problem *prob, int *row_status)
{
    try {
        return mpqp_reduce_constraints_impl(prob, row_status);
    } catch (...) {
        // no C++ exception leaves an exported entry point
        try {
            return fail(MPQP_ENOMEM, "mpqp_reduce_constraints: host memory allocation failed");
        } catch (...) {
            return MPQP_ENOMEM;
        }
    }
}
