// Region laws without any device allocation.
//
// Who needs this: callers that evaluate region laws from a context where
// they may not allocate device memory -- a real-time control loop that has
// finished its start-up (a cudaMalloc can block on the driver or fail under
// memory pressure at the worst moment), or a host application that owns the
// whole device-memory budget through its own allocator and does not let a
// plugin call cudaMalloc / cudaFree.  They pass their problem and active sets
// from the host and receive the laws in device buffers they allocated
// themselves, once, up front.
//
// Where the scratch lives: the per-instance FP64 KKT blocks and the staged
// masks go into g_noalloc_scratch, a fixed 1 MiB array in this file that
// every GPU loading the library keeps until the process exits.  In host code
// that name is only a stand-in for the symbol, not a device address, so the
// first call on each device (with that device current) resolves the address
// with cudaGetSymbolAddress and keeps it.  A call may not be captured into a
// CUDA graph: it stages its data through one host buffer that the next call
// rewrites, so a replay would upload whatever that buffer then holds; a call
// on a stream that is being captured is refused (MPQP_EINVAL).  Every call
// reuses the same array: a call writes all the scratch it later reads
// (nothing has to start at zero), and two calls whose work overlaps on the
// GPU -- calls on different streams, or from different threads -- race on
// it.  Calls on one stream are ordered.
//
// Inputs are checked like the allocating entry point (mpqp_region_laws)
// checks them, so both accept and reject the same problems, with one limit
// of this file's own: n <= 32 (the host work arrays of the precompute).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/mpqp_gb300.h"
#include "mpqp_internal.h"

namespace mq {
size_t laws_smem_per_warp(const SlotDims &sd);
const void *kernel_ptr(const char *name);
cudaError_t launch_region_laws(const DevBuffers &B, const Tol &tol, const SlotDims &sd, const uint64_t *masks,
                               long long n_sets, double *laws, int *sizes, long long stride, int grid,
                               size_t smem, cudaStream_t s);
void set_error_text(const char *msg);
}  // namespace mq

using namespace mq;

namespace {

constexpr size_t kScratchBytes = (size_t)MPQP_NOALLOC_SCRATCH_BYTES;
constexpr size_t kDescBytes = 512;           // InstDesc slot at the start
static_assert(sizeof(InstDesc) <= kDescBytes, "InstDesc outgrew its scratch slot");
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

alignas(256) unsigned char g_stage[kScratchBytes];   // host image of the scratch
double g_work[32 * 32 + 32 * 128 + 32 * 30 + 32];     // L, V, U, u of the precompute
void *g_scratch_dev[kMaxDevices];
std::mutex g_mu;

inline int odd_up(int x) { return (x & 1) ? x : x + 1; }

// FP64 KKT blocks of one instance (same operation order as the engine's
// precompute) written straight into `pool`; offsets go into d, the doubles
// used into *used.
int precompute(const mpqp_problem &P, InstDesc &d, double *pool, size_t pool_cap, size_t *used)
{
    const int n = P.n, m = P.m, p = P.p, ncp = P.ncp;
    memset(&d, 0, sizeof(d));
    d.n = n; d.m = m; d.p = p; d.ncp = ncp;
    d.M1 = m + ncp; d.nv = n + p; d.ld1 = odd_up(d.nv + 1); d.ld2 = odd_up(p + 2);
    d.ld1d = d.ld1; d.ld2d = d.ld2;
    d.lp = 1;
    for (int i = 0; i < n * n && d.lp; i++) if (P.Q[i] != 0.0) d.lp = 0;
    d.ld2lp = odd_up(p + n + 3);
    size_t o = 0;
    auto take = [&](size_t cnt) { const size_t at = o; o += (cnt + 3) & ~(size_t)3; return (long long)at; };
    d.o_Wm = take((size_t)m * m); d.o_Wh = take((size_t)m * p); d.o_wc = take(m);
    d.o_At = take((size_t)ncp * p); d.o_bt = take(ncp); d.o_QiAT = take((size_t)n * m);
    d.o_QiH = take((size_t)n * p); d.o_Qic = take(n);
    if (d.lp) { d.o_WhL = take((size_t)m * p); d.o_wcL = take(m); d.o_Hm = take((size_t)n * p); d.o_cv = take(n); }
    *used = o;
    if (o > pool_cap) return MPQP_ECAPACITY;
    memcpy(pool + d.o_At, P.At, sizeof(double) * (size_t)ncp * p);
    memcpy(pool + d.o_bt, P.bt, sizeof(double) * (size_t)ncp);
    if (d.lp) {
        // mpLP (Q = 0): Wm = A A^T, Wh = F, wc = b, QiAT = A^T, QiH = Qic = 0,
        // WhL = A H, wcL = A c, Hm = H, cv = c
        double *Wm = pool + d.o_Wm, *WhL = pool + d.o_WhL, *wcL = pool + d.o_wcL, *AT = pool + d.o_QiAT;
        for (int r = 0; r < m; r++) {
            for (int s = 0; s < m; s++) {
                double acc = 0.0;
                for (int i = 0; i < n; i++) acc = std::fma(P.A[(size_t)r * n + i], P.A[(size_t)s * n + i], acc);
                Wm[(size_t)r * m + s] = acc;
            }
            for (int c = 0; c < p; c++) {
                double acc = 0.0;
                for (int i = 0; i < n; i++) acc = std::fma(P.A[(size_t)r * n + i], P.H[(size_t)i * p + c], acc);
                WhL[(size_t)r * p + c] = acc;
            }
            double acc = 0.0;
            for (int i = 0; i < n; i++) acc = std::fma(P.A[(size_t)r * n + i], P.c[i], acc);
            wcL[r] = acc;
            for (int i = 0; i < n; i++) AT[(size_t)i * m + r] = P.A[(size_t)r * n + i];
        }
        memcpy(pool + d.o_Wh, P.F, sizeof(double) * (size_t)m * p);
        memcpy(pool + d.o_wc, P.b, sizeof(double) * (size_t)m);
        memset(pool + d.o_QiH, 0, sizeof(double) * (size_t)n * p);
        memset(pool + d.o_Qic, 0, sizeof(double) * (size_t)n);
        memcpy(pool + d.o_Hm, P.H, sizeof(double) * (size_t)n * p);
        memcpy(pool + d.o_cv, P.c, sizeof(double) * (size_t)n);
        return MPQP_OK;
    }
    double *L = g_work, *V = L + n * n, *U = V + (size_t)n * m, *u = U + (size_t)n * p;
    memset(g_work, 0, sizeof(g_work));
    for (int j = 0; j < n; j++) {
        for (int i = j; i < n; i++) {
            double acc = P.Q[i * n + j];
            for (int l = 0; l < j; l++) acc = std::fma(-L[i * n + l], L[j * n + l], acc);
            if (i == j) {
                if (!(acc > 0.0)) return MPQP_ENOTSPD;
                L[j * n + j] = std::sqrt(acc);
            } else {
                L[i * n + j] = acc / L[j * n + j];
            }
        }
    }
    auto fwd = [&](const double *rhs, int rs, double *y, int ys) {
        for (int i = 0; i < n; i++) {
            double acc = rhs[(size_t)i * rs];
            for (int l = 0; l < i; l++) acc = std::fma(-L[i * n + l], y[(size_t)l * ys], acc);
            y[(size_t)i * ys] = acc / L[i * n + i];
        }
    };
    auto bwd = [&](const double *y, int ysd, double *x, int xs) {
        for (int i = n - 1; i >= 0; i--) {
            double acc = y[(size_t)i * ysd];
            for (int l = i + 1; l < n; l++) acc = std::fma(-L[l * n + i], x[(size_t)l * xs], acc);
            x[(size_t)i * xs] = acc / L[i * n + i];
        }
    };
    for (int r = 0; r < m; r++) fwd(P.A + (size_t)r * n, 1, V + r, m);
    for (int c = 0; c < p; c++) fwd(P.H + c, p, U + c, p);
    fwd(P.c, 1, u, 1);
    double *Wm = pool + d.o_Wm, *Wh = pool + d.o_Wh, *wc = pool + d.o_wc;
    for (int r = 0; r < m; r++) {
        for (int s = 0; s < m; s++) {
            double acc = 0.0;
            for (int i = 0; i < n; i++) acc = std::fma(V[i * m + r], V[i * m + s], acc);
            Wm[r * m + s] = acc;
        }
        for (int c = 0; c < p; c++) {
            double acc = P.F[r * p + c];
            for (int i = 0; i < n; i++) acc = std::fma(V[i * m + r], U[i * p + c], acc);
            Wh[r * p + c] = acc;
        }
        double acc = P.b[r];
        for (int i = 0; i < n; i++) acc = std::fma(V[i * m + r], u[i], acc);
        wc[r] = acc;
    }
    for (int r = 0; r < m; r++) bwd(V + r, m, pool + d.o_QiAT + r, m);
    for (int c = 0; c < p; c++) bwd(U + c, p, pool + d.o_QiH + c, p);
    bwd(u, 1, pool + d.o_Qic, 1);
    return MPQP_OK;
}

// Every failure path: the error text, and the runtime's last-error state
// cleared so that it does not surface in a later, valid call.
int fail(int code, const char *msg)
{
    cudaGetLastError();
    set_error_text(msg);
    return code;
}

int noalloc_impl(const mpqp_problem *prob, long long n_sets, const uint64_t *masks, double *laws, int *sizes,
                 void *stream)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!prob || n_sets < 0 || (n_sets && (!masks || !laws || !sizes)))
        return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: null pointer or negative count");
    if (!prob->Q || !prob->c || !prob->H || !prob->A || !prob->b || !prob->F || !prob->At || !prob->bt)
        return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: null problem array");
    const int n = prob->n, m = prob->m, p = prob->p, ncp = prob->ncp;
    if (n < 1 || n > 32 || m < 1 || m > kMaxM || p < 1 || p > kMaxP || ncp < 1)
        return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: sizes out of range (1<=n<=32, 1<=m<=128, 1<=p<=30)");
    // the allocating entry point's limits (8-bit basis ids)
    if (m + ncp + n + p > kMaxIds || m + ncp + p + 1 > kMaxIds)
        return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: instance too large (m+ncp+n+p must be <= 255)");
    bool qzero = true;
    for (int i = 0; i < n * n && qzero; i++) if (prob->Q[i] != 0.0) qzero = false;
    if (qzero && (p + n + 2) + (m + ncp + 2 * n + 1) > kMaxIds)
        return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: mpLP instance too large (m + ncp + 3n + p must be <= 252)");
    for (int i = 0; i < m; i++)
        if (!(prob->b[i] >= 0.0)) return fail(MPQP_EORIGIN, "mpqp_region_laws_noalloc: b has a negative entry");
    for (int i = 0; i < ncp; i++)
        if (!(prob->bt[i] >= 0.0)) return fail(MPQP_EORIGIN, "mpqp_region_laws_noalloc: CRb has a negative entry");
    // a call inside a stream capture would record an upload from the host
    // staging buffer, which later calls rewrite
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &cap) != cudaSuccess)
        return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: cudaStreamIsCapturing failed");
    if (cap != cudaStreamCaptureStatusNone)
        return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: the stream is being captured; calls may not be "
                                 "captured into a CUDA graph");
    if (n_sets == 0) return MPQP_OK;
    const int kcap = m < n ? m : n;
    for (long long i = 0; i < n_sets; i++) {
        const uint64_t lo = masks[2 * i], hi = masks[2 * i + 1];
        const int k = __builtin_popcountll(lo) + __builtin_popcountll(hi);
        const bool outside = m < 64 ? ((lo >> m) != 0 || hi != 0) : (m < 128 && (hi >> (m - 64)) != 0);
        if (k > kcap || outside) return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: active set out of range");
    }
    // scratch image: InstDesc | FP64 blocks | masks
    InstDesc d;
    double *pool = (double *)(g_stage + kDescBytes);
    const size_t pool_cap = (kScratchBytes - kDescBytes) / sizeof(double);
    size_t pool_used = 0;
    int rc = precompute(*prob, d, pool, pool_cap, &pool_used);
    if (rc == MPQP_ENOTSPD) return fail(rc, "mpqp_region_laws_noalloc: Q is neither positive definite nor zero");
    const size_t mask_off = kDescBytes + ((pool_used * sizeof(double) + 255) & ~(size_t)255);
    const size_t need = mask_off + (size_t)n_sets * 2 * sizeof(uint64_t);
    if (rc == MPQP_ECAPACITY || need > kScratchBytes)
        return fail(MPQP_ECAPACITY, "mpqp_region_laws_noalloc: problem data plus 16 bytes per active set exceed "
                                    "the fixed 1 MiB scratch; pass fewer sets per call");
    memcpy(g_stage, &d, sizeof(d));
    memcpy(g_stage + mask_off, masks, (size_t)n_sets * 2 * sizeof(uint64_t));
    // per-device set-up: the device address of the scratch array
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: cudaGetDevice failed");
    if (!g_scratch_dev[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: cudaGetSymbolAddress of the scratch failed");
        }
        g_scratch_dev[dev] = ptr;
    }
    unsigned char *scratch = (unsigned char *)g_scratch_dev[dev];
    SlotDims sd{};
    sd.maxM1 = d.M1; sd.maxLD1 = d.ld1; sd.maxNv = d.nv;
    sd.maxK = kcap < 1 ? 1 : kcap;
    sd.maxP1 = p + 1; sd.maxR2 = m + ncp; sd.maxLD2 = d.ld2;
    sd.maxLD1d = d.ld1d; sd.maxLD2d = d.lp ? (d.ld2lp > d.ld2d ? d.ld2lp : d.ld2d) : d.ld2d;
    sd.maxR2d = d.lp ? m + ncp + 2 * n + 1 : m + ncp;
    sd.maxN = d.lp ? n : 0;
    const size_t smem = 4 * laws_smem_per_warp(sd);
    const void *fn = kernel_ptr("laws");
    int sms = 0, nb = 0, smem_max = 0;
    if (cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: device attribute query");
    if (smem > (size_t)smem_max)
        return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: kernel does not fit on an SM (shared memory)");
    if (smem > 48 * 1024 && cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: shared-memory attribute");
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, smem) != cudaSuccess)
        return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: occupancy query");
    if (nb < 1) return fail(MPQP_EINVAL, "mpqp_region_laws_noalloc: kernel does not fit on an SM (shared memory)");
    cudaStream_t s = (cudaStream_t)stream;
    // pageable source: the call returns once the host image has been taken,
    // so the next call may rewrite it
    e = cudaMemcpyAsync(scratch, g_stage, need, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: upload of the scratch image");
    DevBuffers B;
    memset(&B, 0, sizeof(B));
    B.inst = (const InstDesc *)scratch;
    B.dpool = (const double *)(scratch + kDescBytes);
    B.n_inst = 1;
    Tol tol{};
    memset(&tol, 0, sizeof(tol));
    mpqp_options o;
    mpqp_default_options(&o);
    tol.tol_licq = o.tol_licq;
    tol.tol_zero_row = o.tol_zero_row;
    const long long stride = (long long)m * (p + 1) + (long long)n * (p + 1) + (long long)(m + ncp) * (p + 1);
    e = launch_region_laws(B, tol, sd, (const uint64_t *)(scratch + mask_off), n_sets, laws, sizes, stride,
                           nb * sms, smem, s);
    if (e != cudaSuccess) return fail(MPQP_ECUDA, "mpqp_region_laws_noalloc: kernel launch");
    return MPQP_OK;
}

}  // namespace

// No C++ exception crosses the C ABI (std::lock_guard can throw).
extern "C" int mpqp_region_laws_noalloc(const mpqp_problem *prob, long long n_sets, const uint64_t *masks,
                                        double *laws, int *sizes, void *stream)
{
    try {
        return noalloc_impl(prob, n_sets, masks, laws, sizes, stream);
    } catch (...) {
        try {
            set_error_text("mpqp_region_laws_noalloc: host error");
        } catch (...) {
        }
        return MPQP_ENOMEM;
    }
}
