// Device kernels of the combinatorial mpQP active-set check (sm_103a).
//
// One enumeration level k runs as
//   k_enumerate      children of the level-(k-1) feasible sets, superset
//                    pruning against a tagged hash of feasible masks
//   k_feasibility<T> LP1 per candidate, one warp per LP, tableau in shared
//                    memory, warm-started from the parent's final tableau
//   k_lp1_fp64       (mixed precision) FP64 re-solve of the LP1 candidates
//                    the FP32 certificate could not decide
//   k_optimality<T>  KKT factor -> critical-region rows -> LP2 (max margin)
//                    -> Chebyshev LP, one warp per feasible set
//   k_finalize       per-instance budget bookkeeping, counter resets
// All counts live in device memory, so the whole level loop is a fixed
// launch sequence that the host captures in one CUDA graph.
//
// Floating-point contract (FP64 kernels): explicit fma for every
// multiply-add, sums in ascending index order, IEEE division and square root,
// compiled with -fmad=false.  This is the operation order of the CPU oracle,
// so FP64 LP values and verdicts are bit-identical to it.
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpqp_internal.h"

namespace mq {

#define FULLMASK 0xffffffffu

__device__ __forceinline__ double xfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float xfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double xsqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double xabs(double a) { return fabs(a); }
__device__ __forceinline__ float xabs(float a) { return fabsf(a); }

template <typename T> __device__ __forceinline__ T pos_inf();
template <> __device__ __forceinline__ double pos_inf<double>() { return __longlong_as_double(0x7ff0000000000000LL); }
template <> __device__ __forceinline__ float pos_inf<float>() { return __int_as_float(0x7f800000); }

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ bool mask_has(uint64_t lo, uint64_t hi, int j)
{
    return j < 64 ? ((lo >> j) & 1ull) : ((hi >> (j - 64)) & 1ull);
}

__device__ __forceinline__ int mask_pop(uint64_t lo, uint64_t hi) { return __popcll(lo) + __popcll(hi); }

// live rows of a stored LP1 tableau (node flags bits 8..16 hold rows + 1;
// 0: all M1 rows)
__device__ __forceinline__ int node_rows(int flags, int M1)
{
    const int r = (flags >> kNodeRowsShift) & 0x1ff;
    return r > 0 ? r - 1 : M1;
}

__device__ __forceinline__ int node_cols(int flags, int nv)
{
    const int c = (flags >> kNodeColsShift) & 0xff;
    return c > 0 ? c - 1 : nv;
}

// number of mask bits below position i
__device__ __forceinline__ int mask_rank(uint64_t lo, uint64_t hi, int i)
{
    if (i < 64) return __popcll(lo & ((i == 0) ? 0ull : (~0ull >> (64 - i))));
    const int r = i - 64;
    return __popcll(lo) + __popcll(hi & ((r == 0) ? 0ull : (~0ull >> (64 - r))));
}

__device__ __forceinline__ int mask_max(uint64_t lo, uint64_t hi)
{
    if (hi) return 127 - __clzll(hi);
    if (lo) return 63 - __clzll(lo);
    return -1;
}

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

// hash summed into the per-instance set digests
__device__ __forceinline__ unsigned long long mask_digest(uint64_t lo, uint64_t hi)
{
    return mix64(lo ^ mix64(hi ^ 0x5bd1e9955bd1e995ULL));
}

__device__ __forceinline__ uint64_t hash_key(int inst, uint64_t lo, uint64_t hi)
{
    return mix64(lo ^ mix64(hi ^ ((uint64_t)(uint32_t)inst * 0x9e3779b97f4a7c15ULL)));
}

// Slots a level's hash uses: the smallest power of 2 above twice the level's
// candidates (an upper bound on its inserts), at most the allocated table.
// A level with few sets keeps its probes inside a small, L2-resident prefix.
__device__ __forceinline__ long long hash_cap_for(const DevBuffers &B, long long n_sets)
{
    long long c = 16;
    while (c < 2 * n_sets + 1 && c < B.hash_cap) c <<= 1;
    return c < B.hash_cap ? c : B.hash_cap;
}

// Hash slots are 8 bytes: a 24-bit tag (the run and the level) above 40 bits
// of the set's 64-bit hash (its bits 24..63; the low bits pick the home
// slot).  Runs draw their epochs from one counter per device (g_hash_epoch),
// so the entries of another level, run or plan -- and any other leftover
// bytes, or the zeros of fresh memory (tag 0 is never used) -- read as empty
// slots, except a stale entry whose tag matches by wrap-around (one level of a
// run 2^18 runs earlier): it only lengthens the probe.  Two sets share a
// fingerprint with probability 2^-40 per probe of the same home slot; a set
// then found in place of an absent subset is only left unpruned, and its LP1
// (a superset of an infeasible set) is infeasible, so no verdict depends on it.
__device__ unsigned g_hash_epoch;
constexpr unsigned long long kFpMask = (1ull << 40) - 1;

__device__ __forceinline__ unsigned long long hash_tag(int epoch, int level)
{
    return (unsigned long long)(((unsigned)epoch * 64u + (unsigned)level) % 0xffffffu + 1u);
}

__device__ int hash_find_from(const HashSlot *tab, long long cap, unsigned long long tag, uint64_t fp, uint64_t s)
{
    const unsigned long long f40 = fp >> 24;
    for (long long probe = 0; probe < cap; probe++) {
        const unsigned long long w = tab[s].w;
        if ((w >> 40) != tag) return -1;
        if ((w & kFpMask) == f40) return 1;
        s = (s + 1) & (uint64_t)(cap - 1);
    }
    return -1;
}

__device__ bool hash_insert(HashSlot *tab, long long cap, unsigned long long tag, int inst, uint64_t lo, uint64_t hi)
{
    const uint64_t fp = hash_key(inst, lo, hi);
    const unsigned long long w = (tag << 40) | (fp >> 24);
    uint64_t s = fp & (uint64_t)(cap - 1);
    for (long long probe = 0; probe < cap; probe++) {
        unsigned long long *h = &tab[s].w;
        const unsigned long long t = *((volatile unsigned long long *)h);
        if ((t >> 40) != tag) {
            if (atomicCAS(h, t, w) == t) return true;
            continue;   // lost the slot to another insert: read it again
        }
        s = (s + 1) & (uint64_t)(cap - 1);
    }
    return false;
}

// ---------------------------------------------------------------------
// warp-cooperative Tucker-tableau simplex
// ---------------------------------------------------------------------
// rows 0..nrows-1 basic variables, row nrows the objective (minimised);
// columns 0..ncols-1 nonbasic variables, column ncols the right-hand side.
// x_B = T[.,ncols] - sum_j T[.,j] x_N(j).  Ids < nfree are free variables.
template <typename T>
struct Lp {
    T *tab;
    int ld, nrows, ncols, nfree;
    uint8_t *bid, *nid;
};

// Order-preserving unsigned images of non-negative values (min over the
// keys = min over the values); all-ones marks "no candidate".
__device__ __forceinline__ unsigned key_of(float v) { return __float_as_uint(v); }
__device__ __forceinline__ unsigned long long key_of(double v) { return (unsigned long long)__double_as_longlong(v); }
__device__ __forceinline__ unsigned key_none(float) { return 0xffffffffu; }
// Order-preserving unsigned image of any non-NaN float (negative included).
__device__ __forceinline__ unsigned key_signed(float v)
{
    const unsigned u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long key_none(double) { return ~0ull; }

// Warp-wide smallest (key, id); returns the winning lane's idx, or -1.  Ids
// are unique across the warp, so the result does not depend on lane order.
__device__ __forceinline__ int warp_argmin(unsigned key, unsigned id, int idx)
{
    const unsigned kmin = __reduce_min_sync(FULLMASK, key);
    if (kmin == 0xffffffffu) return -1;
    const bool m = key == kmin;
    const unsigned idm = __reduce_min_sync(FULLMASK, m ? id : 0xffffffffu);
    const unsigned win = __ballot_sync(FULLMASK, m && id == idm);
    return __shfl_sync(FULLMASK, idx, __ffs(win) - 1);
}

__device__ __forceinline__ int warp_argmin(unsigned long long key, unsigned id, int idx)
{
    const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
    const unsigned hmin = __reduce_min_sync(FULLMASK, hi);
    if (hmin == 0xffffffffu) return -1;
    const unsigned lmin = __reduce_min_sync(FULLMASK, hi == hmin ? lo : 0xffffffffu);
    const bool m = hi == hmin && lo == lmin;
    const unsigned idm = __reduce_min_sync(FULLMASK, m ? id : 0xffffffffu);
    const unsigned win = __ballot_sync(FULLMASK, m && id == idm);
    return __shfl_sync(FULLMASK, idx, __ffs(win) - 1);
}

// ratio of the ratio test: IEEE division in FP64 (the oracle's operation);
// the FP32 pass only needs an ordering, so it takes the fast division.
__device__ __forceinline__ double ratio_div(double b, double a) { return __ddiv_rn(b, a); }
__device__ __forceinline__ float ratio_div(float b, float a) { return __fdividef(b, a); }

// T[i][*] -= f * R[*] over columns 0..ncols (the pivot row R is in shared
// memory); FP32 rows are 16-byte aligned (stride = 4 mod 8) and go four
// elements per access.
__device__ __forceinline__ void row_update(double *Ti, const double *R, double nf, int ncols)
{
    for (int j = 0; j <= ncols; j++) Ti[j] = xfma(nf, R[j], Ti[j]);
}

__device__ __forceinline__ void row_update(float *Ti, const float *R, float nf, int ncols)
{
    float4 *t4 = reinterpret_cast<float4 *>(Ti);
    const float4 *r4 = reinterpret_cast<const float4 *>(R);
    const int nch = (ncols + 4) >> 2;
    for (int c = 0; c < nch; c++) {
        float4 t = t4[c];
        const float4 r = r4[c];
        t.x = __fmaf_rn(nf, r.x, t.x);
        t.y = __fmaf_rn(nf, r.y, t.y);
        t.z = __fmaf_rn(nf, r.z, t.z);
        t.w = __fmaf_rn(nf, r.w, t.w);
        t4[c] = t;
    }
}

template <typename T>
__device__ int warp_simplex(const Lp<T> &L, T tol_piv, T tol_dj, int max_piv, int degen_switch, int *piv_out)
{
    const int lane = lane_id();
    int piv = 0, degen = 0, status;
    bool bland = false;
    T *obj = L.tab + (size_t)L.nrows * L.ld;
    for (;;) {
        // pricing: largest |reduced cost|, smallest id on ties (Bland: smallest id)
        auto bkey = key_none(T(0));
        unsigned bid_ = 0xffffffffu;
        int bq = -1;
        for (int j = lane; j < L.ncols; j += 32) {
            const T g = obj[j];
            const int id = L.nid[j];
            const T sc = (id < L.nfree) ? xabs(g) : g;
            if (!(sc > tol_dj)) continue;
            const auto k = bland ? decltype(bkey)(0) : ~key_of(sc);
            if (bq < 0 || k < bkey || (k == bkey && (unsigned)id < bid_)) { bkey = k; bid_ = id; bq = j; }
        }
        const int q = warp_argmin(bkey, bid_, bq);
        if (q < 0) { status = LP_OPTIMAL; break; }
        const T sg = obj[q] > T(0) ? T(1) : T(-1);
        // ratio test: smallest max(beta,0)/a over a > tol_piv, smallest id on ties
        auto rkey = key_none(T(0));
        unsigned rid = 0xffffffffu;
        int bri = -1;
        T rval = T(0);
        for (int i = lane; i < L.nrows; i += 32) {
            const int id = L.bid[i];
            if (id < L.nfree) continue;
            const T a = sg * L.tab[(size_t)i * L.ld + q];
            if (!(a > tol_piv)) continue;
            T beta = L.tab[(size_t)i * L.ld + L.ncols];
            if (!(beta > T(0))) beta = T(0);
            const T ratio = ratio_div(beta, a);
            const auto k = key_of(ratio);
            if (bri < 0 || k < rkey || (k == rkey && (unsigned)id < rid)) { rkey = k; rid = id; bri = i; rval = ratio; }
        }
        const int r = warp_argmin(rkey, rid, bri);
        if (r < 0) { status = LP_UNBOUNDED; break; }
        if (piv >= max_piv) { status = LP_ITER_LIMIT; break; }
        // the chosen ratio, recomputed identically in every lane (degeneracy test)
        T br = L.tab[(size_t)r * L.ld + L.ncols];
        if (!(br > T(0))) br = T(0);
        const T rr = ratio_div(br, sg * L.tab[(size_t)r * L.ld + q]);
        T *R = L.tab + (size_t)r * L.ld;
        const T inv = xdiv(T(1), R[q]);
        __syncwarp();
        for (int j = lane; j <= L.ncols; j += 32) R[j] = (j == q) ? inv : xmul(R[j], inv);
        __syncwarp();
        for (int i = lane; i <= L.nrows; i += 32) {
            if (i == r) continue;
            T *Ti = L.tab + (size_t)i * L.ld;
            const T nf = -Ti[q];
            row_update(Ti, R, nf, L.ncols);
            Ti[q] = xmul(nf, inv);
        }
        __syncwarp();
        if (lane == 0) {
            const uint8_t t = L.bid[r];
            L.bid[r] = L.nid[q];
            L.nid[q] = t;
        }
        __syncwarp();
        piv++;
        (void)rval;
        degen = (rr == T(0)) ? degen + 1 : 0;
        bland = degen >= degen_switch;
    }
    *piv_out = piv;
    return status;
}

// Full-warp FP32 simplex with register bookkeeping, for tableaus of at most
// 96 rows and NCH float4 chunks per row (NCH = (ncols+4)/4, the row stride a
// multiple of 4): the pivoting rules, operations and their order are those of
// warp_simplex on the same tableau (so the same pivots and bit-identical
// values), with the bookkeeping moved to registers: each lane keeps the
// offsets and basic ids of its rows lane, lane+32, lane+64; lanes 0..ncols
// hold the objective row (lane j: column j; lane ncols: right-hand side) and
// lanes 0..ncols-1 the nonbasic ids.  The constraint rows stay in shared
// memory; the objective row and the ids are written back on return.  Ids
// below nfree are free variables (nfree >= ncols: an LP1 tableau whose fixed
// slack columns were moved past the right-hand side has fewer columns than
// free variables).
constexpr int kFastRows = 96;
constexpr int kFastChunks = 6;

// fix_lo/fix_hi (optional): variables with id fix_base + i, i in the mask,
// stay at zero while nonbasic (never priced in).  NRS: row slots per lane
// (nrows <= 32 * NRS).  compact: a free variable that enters the basis never
// leaves it again, and its row is read by no later decision (pricing uses
// the objective row, the ratio test and the pivot only slack rows), so the
// row is dropped -- the last row moves into its place and nrows shrinks;
// *nrows_out receives the final count (the objective row stays where it was).
template <int NCH, int NRS>
__device__ int simplex_fast32(float *tab, int ld, int nrows, int ncols, int nfree, uint8_t *bid, uint8_t *nid,
                              float tol_piv, float tol_dj, int max_piv, int degen_switch, int *piv_out,
                              uint64_t fix_lo, uint64_t fix_hi, int fix_base, bool compact, int *nrows_out)
{
    constexpr int NR = NRS;
    const int lane = lane_id();
    int rowoff[NR], bidr[NR];
    bool valid[NR];
#pragma unroll
    for (int s = 0; s < NR; s++) {
        const int i = lane + 32 * s;
        valid[s] = i < nrows;
        rowoff[s] = i * ld;
        bidr[s] = valid[s] ? bid[i] : 255;
    }
    float *obj = tab + nrows * ld;
    float ob = lane <= ncols ? obj[lane] : 0.0f;
    int nidl = lane < ncols ? nid[lane] : 255;
    int piv = 0, degen = 0, status;
    bool bland = false;
    for (;;) {
        // pricing: largest |reduced cost|, smallest id on ties (Bland: smallest id)
        unsigned key = 0xffffffffu, kid = 0xffffffffu;
        int kidx = -1;
        if (lane < ncols) {
            const float sc = nidl < nfree ? fabsf(ob) : ob;
            const int fi = nidl - fix_base;
            const bool fixed = fi >= 0 && fi < 128 && mask_has(fix_lo, fix_hi, fi);
            if (sc > tol_dj && !fixed) { key = bland ? 0u : ~key_of(sc); kid = (unsigned)nidl; kidx = lane; }
        }
        const int q = warp_argmin(key, kid, kidx);
        if (q < 0) { status = LP_OPTIMAL; break; }
        const float obq = __shfl_sync(FULLMASK, ob, q);
        const float sg = obq > 0.0f ? 1.0f : -1.0f;
        // ratio test: smallest max(beta,0)/a over a > tol_piv, smallest id on ties
        unsigned rkey = 0xffffffffu, rid = 0xffffffffu;
        int bri = -1;
        float aq[NR];
#pragma unroll
        for (int s = 0; s < NR; s++) {
            aq[s] = 0.0f;
            if (valid[s]) {
                aq[s] = tab[rowoff[s] + q];
                if (bidr[s] >= nfree) {
                    const float a = sg * aq[s];
                    if (a > tol_piv) {
                        float beta = tab[rowoff[s] + ncols];
                        if (!(beta > 0.0f)) beta = 0.0f;
                        const unsigned k = key_of(ratio_div(beta, a));
                        if (bri < 0 || k < rkey || (k == rkey && (unsigned)bidr[s] < rid)) {
                            rkey = k; rid = (unsigned)bidr[s]; bri = lane + 32 * s;
                        }
                    }
                }
            }
        }
        const int r = warp_argmin(rkey, rid, bri);
        if (r < 0) { status = LP_UNBOUNDED; break; }
        if (piv >= max_piv) { status = LP_ITER_LIMIT; break; }
        float *Rp = tab + r * ld;
        float br = Rp[ncols];
        if (!(br > 0.0f)) br = 0.0f;
        const float prq = Rp[q];
        const float rr = ratio_div(br, sg * prq);
        const float inv = xdiv(1.0f, prq);
        const int owner = r & 31, oslot = r >> 5;
        const int lid = __shfl_sync(FULLMASK, (int)rid, owner);   // the owner's best row is r
        const int eid = __shfl_sync(FULLMASK, nidl, q);
        __syncwarp();
        if (lane <= ncols) Rp[lane] = (lane == q) ? inv : xmul(Rp[lane], inv);
        __syncwarp();
        const float rl = lane <= ncols ? Rp[lane] : 0.0f;
        bool upd[NR];
#pragma unroll
        for (int s = 0; s < NR; s++) upd[s] = valid[s] && lane + 32 * s != r;
        // chunk by chunk (one float4 of the pivot row live), then column q
#pragma unroll
        for (int c = 0; c < NCH; c++) {
            const float4 Rc = reinterpret_cast<const float4 *>(Rp)[c];
#pragma unroll
            for (int s = 0; s < NR; s++) {
                if (upd[s]) {
                    float4 *Tc = reinterpret_cast<float4 *>(tab + rowoff[s]) + c;
                    const float nf = -aq[s];
                    float4 t = *Tc;
                    t.x = __fmaf_rn(nf, Rc.x, t.x);
                    t.y = __fmaf_rn(nf, Rc.y, t.y);
                    t.z = __fmaf_rn(nf, Rc.z, t.z);
                    t.w = __fmaf_rn(nf, Rc.w, t.w);
                    *Tc = t;
                }
            }
        }
#pragma unroll
        for (int s = 0; s < NR; s++) if (upd[s]) tab[rowoff[s] + q] = xmul(-aq[s], inv);
        if (lane <= ncols) {
            const float nfo = -obq;
            ob = (lane == q) ? xmul(nfo, inv) : __fmaf_rn(nfo, rl, ob);
        }
        if (lane == owner) {
#pragma unroll
            for (int s = 0; s < NR; s++) if (s == oslot) bidr[s] = eid;
        }
        if (lane == q) nidl = lid;
        __syncwarp();
        if (compact && eid < nfree) {
            // row r now belongs to a free variable: the last row takes its place
            const int last = nrows - 1;
            if (r != last) {
                const float v = lane <= ncols ? tab[last * ld + lane] : 0.0f;
                int lb = 0;
#pragma unroll
                for (int s = 0; s < NR; s++) if (s == (last >> 5)) lb = bidr[s];
                lb = __shfl_sync(FULLMASK, lb, last & 31);
                if (lane <= ncols) Rp[lane] = v;
                if (lane == owner) {
#pragma unroll
                    for (int s = 0; s < NR; s++) if (s == oslot) bidr[s] = lb;
                }
            }
            nrows = last;
#pragma unroll
            for (int s = 0; s < NR; s++) valid[s] = lane + 32 * s < nrows;
            __syncwarp();
        }
        piv++;
        degen = (rr == 0.0f) ? degen + 1 : 0;
        bland = degen >= degen_switch;
    }
    // write the bookkeeping back
    if (lane <= ncols) obj[lane] = ob;
    if (lane < ncols) nid[lane] = (uint8_t)nidl;
#pragma unroll
    for (int s = 0; s < NR; s++) if (valid[s]) bid[lane + 32 * s] = (uint8_t)bidr[s];
    __syncwarp();
    *piv_out = piv;
    if (nrows_out) *nrows_out = nrows;
    return status;
}

// warp_simplex for an FP32 tableau: simplex_fast32 when it fits (rows of at
// most MAXCH chunks), else the generic loop (the same pivots either way)
template <int NCH>
__device__ __forceinline__ int simplex_fast32_rows(const Lp<float> &L, float tol_piv, float tol_dj, int max_piv,
                                                   int degen_switch, int *piv_out, uint64_t fix_lo, uint64_t fix_hi,
                                                   int fix_base, bool compact, int *nrows_out)
{
    if (L.nrows <= 32)
        return simplex_fast32<NCH, 1>(L.tab, L.ld, L.nrows, L.ncols, L.nfree, L.bid, L.nid, tol_piv, tol_dj, max_piv,
                                      degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
    if (L.nrows <= 64)
        return simplex_fast32<NCH, 2>(L.tab, L.ld, L.nrows, L.ncols, L.nfree, L.bid, L.nid, tol_piv, tol_dj, max_piv,
                                      degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
    return simplex_fast32<NCH, 3>(L.tab, L.ld, L.nrows, L.ncols, L.nfree, L.bid, L.nid, tol_piv, tol_dj, max_piv,
                                  degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
}

// compact / nrows_out: see simplex_fast32 (the generic loop never compacts;
// *nrows_out is then L.nrows)
template <int MAXCH>
__device__ __forceinline__ int warp_simplex_f32(const Lp<float> &L, float tol_piv, float tol_dj, int max_piv,
                                                int degen_switch, int *piv_out, uint64_t fix_lo = 0,
                                                uint64_t fix_hi = 0, int fix_base = 0, bool compact = false,
                                                int *nrows_out = nullptr)
{
    static_assert(MAXCH >= 1 && MAXCH <= kFastChunks, "chunk count");
    const int nch = (L.ncols + 4) >> 2;
    if (L.nrows <= kFastRows && (L.ld & 3) == 0 && nch <= MAXCH) {
        switch (nch) {
        case 1: return simplex_fast32_rows<1>(L, tol_piv, tol_dj, max_piv, degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
        case 2: return simplex_fast32_rows<2>(L, tol_piv, tol_dj, max_piv, degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
        case 3: if constexpr (MAXCH >= 3) return simplex_fast32_rows<3>(L, tol_piv, tol_dj, max_piv, degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
        case 4: if constexpr (MAXCH >= 4) return simplex_fast32_rows<4>(L, tol_piv, tol_dj, max_piv, degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
        case 5: if constexpr (MAXCH >= 5) return simplex_fast32_rows<5>(L, tol_piv, tol_dj, max_piv, degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
        case 6: if constexpr (MAXCH >= 6) return simplex_fast32_rows<6>(L, tol_piv, tol_dj, max_piv, degen_switch, piv_out, fix_lo, fix_hi, fix_base, compact, nrows_out);
        default: break;
        }
    }
    if (nrows_out) *nrows_out = L.nrows;
    return warp_simplex<float>(L, tol_piv, tol_dj, max_piv, degen_switch, piv_out);
}

// ---------------------------------------------------------------------
// shared-memory slot sizes
// ---------------------------------------------------------------------
__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// column of the dual-screen row layout (stride 12: g 0..5, c 6, h 7) that
// holds each row's error scale: the sum of the magnitudes of the terms the
// FP32 row was computed from (0 for the exact box rows)
constexpr int kRowScaleCol = 8;

// LP1 buffer: tableau (maxM1+1) x maxLD1 + ids (maxM1 + maxNv)
template <typename T>
__host__ __device__ inline size_t lp1_buf_bytes(int maxM1, int maxLD1, int maxNv)
{
    return align16((((size_t)(maxM1 + 1) * maxLD1 + 3) & ~(size_t)3) * sizeof(T)) + align16((size_t)maxM1 + maxNv);
}

// LP1 slot of k_lp1_fp64: one buffer + 16 bytes
template <typename T>
__host__ __device__ inline size_t lp1_slot_bytes(int maxM1, int maxLD1, int maxNv)
{
    return lp1_buf_bytes<T>(maxM1, maxLD1, maxNv) + 16;
}

// slot of k_feasibility: one buffer and the warp's mbarrier (16 bytes, last)
template <typename T>
__host__ __device__ inline size_t feas_slot_bytes(int maxM1, int maxLD1, int maxNv)
{
    return lp1_buf_bytes<T>(maxM1, maxLD1, maxNv) + 16;
}

// candidates a warp claims at a time (a plan setting, at most 32, by default
// 32): consecutive candidates share parents (children of one parent are
// consecutive in the candidate list), so the first child loads its parent
// from DRAM and the others find it in L2, and the next candidate's parent is
// known one candidate ahead (L2 prefetch)
constexpr int kFeasChunkMax = 32;

// ---------------------------------------------------------------------
// bulk (TMA) copies between global and shared memory
// ---------------------------------------------------------------------
// Addresses 16-byte aligned and sizes multiples of 16 bytes (tableaus are
// multiples of 4 elements at offsets that are multiples of 4 elements; basis
// ids are padded to 16 bytes).  Loads complete on an mbarrier of the warp's
// slot; stores go in bulk groups that the issuing lane waits for before the
// slot is written again.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's generic shared-memory accesses before later bulk copies
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Wait for the phase of parity `parity` to complete, at most kWaitTries
// tries (each suspends for a bounded, implementation-defined time); false
// when the limit ran out.
constexpr int kWaitTries = 1 << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    for (int it = 0; it < kWaitTries; it++) {
        unsigned ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// a hint: bring [src, src + bytes) into L2 (no completion to wait for)
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, unsigned bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_store(void *dst, const void *src, unsigned bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the bulk stores issued by this thread have read their shared-memory source
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... and have completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// optimality slot: R (kmax^2), Y and Lambda (kmax x P1), G (R2 x P1),
// tableau (rows+1) x ld2, ids (rows + P1, + n + 1 with mpLP instances), S
// list; FP64 with mpLP instances also Psi (kmax x P1) and Phi (kmax x n).
// rows = R2 (FP32) or maxR2d (FP64).
template <typename T>
__host__ __device__ inline size_t opt_slot_bytes(const SlotDims &sd)
{
    const bool d = sizeof(T) == 8;
    const int rows = d ? sd.maxR2d : sd.maxR2, ld = d ? sd.maxLD2d : sd.maxLD2;
    size_t b = align16((size_t)sd.maxK * sd.maxK * sizeof(T)) + 2 * align16((size_t)sd.maxK * sd.maxP1 * sizeof(T)) +
               align16((size_t)sd.maxR2 * sd.maxP1 * sizeof(T)) + align16((size_t)(rows + 1) * ld * sizeof(T)) +
               align16((size_t)rows + sd.maxP1 + (sd.maxN ? sd.maxN + 1 : 0)) + align16((size_t)sd.maxK * sizeof(int));
    if (d && sd.maxN)
        b += align16((size_t)sd.maxK * sd.maxP1 * sizeof(T)) + align16((size_t)sd.maxK * sd.maxN * sizeof(T));
    return b;
}

// ---------------------------------------------------------------------
// K1: enumerate children, superset pruning
// ---------------------------------------------------------------------
struct LocalInstCounters {
    int inst;
    long long a, b, c, d, e, f, g;
    __device__ void reset(int i) { inst = i; a = b = c = d = e = f = g = 0; }
};

// Children of 32 parents at a time, flattened: lane l takes the l-th child of
// the chunk in (parent, j) order -- its parent found by a binary search over
// the parents' child offsets -- so the warp's 32 subset tests are 32 children
// whatever each parent's count (at the deepest levels a parent has about six).
// Candidates keep the (parent, j) order within a group of 32; the counters
// and the budget are kept per instance among the lanes of a group.
__global__ void k_enumerate(DevBuffers B, int level)
{
    const int lane = lane_id();
    const unsigned below = (1u << lane) - 1u;
    const int pside = (level - 1) & 1;
    Ctl *ctl = B.ctl;
    const long long npar = ctl->n_node[pside] < B.node_cap ? ctl->n_node[pside] : B.node_cap;
    // key of the previous level's hash entries
    const unsigned long long tag_prev = hash_tag(ctl->epoch, level - 1);
    // slots the previous level's inserts used (every expandable parent was
    // inserted, which sets it; the full table otherwise, which is always in bounds)
    const long long hcap = ctl->hcap[pside] >= 16 && ctl->hcap[pside] <= B.hash_cap ? ctl->hcap[pside] : B.hash_cap;
    const int es = B.precision == PREC_MIXED ? 4 : 8;
    const HashSlot *tab = B.hash[pside];
    for (;;) {
        // parents are claimed 32 at a time (one atomic per chunk: levels
        // past an instance's last level hold many parents that are skipped)
        long long p0;
        if (lane == 0) p0 = (long long)atomicAdd(&ctl->ctr[1], 32ull);
        p0 = __shfl_sync(FULLMASK, p0, 0);
        if (p0 >= npar) break;
        const int cnt = npar - p0 < 32 ? (int)(npar - p0) : 32;
        // lane t: parent p0 + t, whether it is expanded, its first child
        // element and child count
        bool expand = false;
        unsigned sbytes = 0;   // the bytes the LP1 kernel stored for this node (tableau rows and ids)
        int sinst = -1, pinst = -1, jmin = 0, nch = 0;
        uint64_t plo = 0, phi = 0;
        int prows = 0;
        if (lane < cnt) {
            const Node pn = B.node[pside][p0 + lane];
            expand = (pn.flags & NODE_VALID) && (B.exhaustive || (pn.flags & NODE_FEASIBLE)) &&
                     !B.ictl[pn.inst].stopped && level <= B.inst[pn.inst].k_max;
            const InstDesc &Ip = B.inst[pn.inst];
            prows = es == 4 ? node_rows(pn.flags, Ip.M1) : Ip.M1;
            if ((pn.flags & NODE_VALID) && pn.tab_off >= 0) {
                sbytes = (unsigned)((prows + 1) * Ip.ld1 * es + Ip.ids_bytes);
                sinst = pn.inst;
            }
            if (expand) {
                plo = pn.lo; phi = pn.hi; pinst = pn.inst;
                jmin = mask_max(pn.lo, pn.hi) + 1;
                nch = Ip.m > jmin ? Ip.m - jmin : 0;
            }
        }
        {
            // counted here, once per stored node, rather than by the LP1
            // kernel's store (an atomic per store there contends): one
            // atomic per instance present among these 32 nodes
            const unsigned grp = __match_any_sync(FULLMASK, sinst);
            const unsigned tot = __reduce_add_sync(grp, sbytes);
            if (sinst >= 0 && lane == __ffs(grp) - 1)
                atomicAdd((unsigned long long *)&B.ictl[sinst].store_bytes, (unsigned long long)tot);
        }
        // exclusive offsets of the parents' children
        int incl = nch;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(FULLMASK, incl, off);
            if (lane >= off) incl += v;
        }
        const int total = __shfl_sync(FULLMASK, incl, 31);
        const int excl = incl - nch;
        unsigned emitted = 0;   // bit t: parent t has a candidate at this level
        for (int g0 = 0; g0 < total; g0 += 32) {
            const int idx = g0 + lane;
            const bool valid = idx < total;
            // the parent of child idx: the last lane whose offset is <= idx
            // (it has children: the next offset is larger)
            int t = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1) {
                const int e = __shfl_sync(FULLMASK, excl, t + step);
                if (e <= idx) t += step;
            }
            const uint64_t clo0 = __shfl_sync(FULLMASK, plo, t), chi0 = __shfl_sync(FULLMASK, phi, t);
            const int cinst = __shfl_sync(FULLMASK, pinst, t);
            const int j = __shfl_sync(FULLMASK, jmin, t) + (idx - __shfl_sync(FULLMASK, excl, t));
            bool ok = valid;
            if (ok && !B.exhaustive) {
                uint64_t lo = clo0, hi = chi0;
                if (j < 64) lo |= 1ull << j; else hi |= 1ull << (j - 64);
                // the subsets child minus a, a in the parent, four at a time: the
                // home slots of all four are read before any is checked, so the
                // random accesses overlap; a collision probes on from there
                uint64_t rlo = clo0, rhi = chi0;
                while (ok && (rlo | rhi)) {
                    constexpr int G = 4;
                    uint64_t sfp[G], sidx[G];
                    int n = 0;
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        sfp[g] = 0; sidx[g] = 0;
                        if (rlo | rhi) {
                            int a;
                            if (rlo) { a = __ffsll((long long)rlo) - 1; rlo &= rlo - 1; }
                            else { a = 64 + __ffsll((long long)rhi) - 1; rhi &= rhi - 1; }
                            uint64_t slo = lo, shi = hi;
                            if (a < 64) slo &= ~(1ull << a); else shi &= ~(1ull << (a - 64));
                            sfp[g] = hash_key(cinst, slo, shi);
                            sidx[g] = sfp[g] & (uint64_t)(hcap - 1);
                            n = g + 1;
                        }
                    }
                    HashSlot hs[G];
#pragma unroll
                    for (int g = 0; g < G; g++) if (g < n) hs[g] = tab[sidx[g]];
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        if (g < n && ok) {
                            if ((hs[g].w >> 40) != tag_prev) ok = false;
                            else if ((hs[g].w & kFpMask) != (sfp[g] >> 24))
                                ok = hash_find_from(tab, hcap, tag_prev, sfp[g],
                                                    (sidx[g] + 1) & (uint64_t)(hcap - 1)) >= 0;
                        }
                    }
                }
            }
            // per instance among the group's lanes: pruned count, the budget,
            // and one range of candidate slots
            const unsigned grp = __match_any_sync(FULLMASK, valid ? cinst : -1);
            const unsigned okm = __ballot_sync(FULLMASK, ok) & grp;
            const int leader = __ffs(grp) - 1;
            long long base = 0;
            int over = 0;
            if (valid && lane == leader) {
                const int cntg = __popc(okm), pr = __popc(grp) - cntg;
                if (pr) atomicAdd((unsigned long long *)&B.ictl[cinst].pruned, (unsigned long long)pr);
                if (cntg) {
                    const InstDesc &I = B.inst[cinst];
                    const long long old = (long long)atomicAdd((unsigned long long *)&B.ictl[cinst].lvl_cand,
                                                               (unsigned long long)cntg);
                    // with a budget, the level is checked only if the whole
                    // level fits it; past that point nothing needs to be written
                    over = I.budget > 0 && B.ictl[cinst].cum_cand + old + cntg > I.budget;
                    if (!over) base = (long long)atomicAdd((unsigned long long *)&ctl->n_cand, (unsigned long long)cntg);
                }
            }
            base = __shfl_sync(FULLMASK, base, leader);
            over = __shfl_sync(FULLMASK, over, leader);
            const bool put = ok && !over;
            if (put) {
                const long long ci = base + __popc(okm & below);
                if (ci < B.cand_cap) {
                    B.cand[ci].parent = (int)(p0 + t);
                    B.cand[ci].j = j;
                } else {
                    atomicOr(&ctl->overflow, OV_CAND);
                }
            }
            emitted |= __reduce_or_sync(FULLMASK, put ? 1u << t : 0u);
        }
        {
            // the bytes the children's LP1 stages of each parent with a
            // candidate: live rows + objective row, basis ids, the node
            const bool em = (emitted >> lane) & 1u;
            const int ei = em ? pinst : -1;
            const unsigned grp = __match_any_sync(FULLMASK, ei);
            const unsigned n_em = __popc(grp);
            unsigned bytes = 0;   // a few KB each: 32 of them fit 32 bits
            if (em) {
                const InstDesc &Ip = B.inst[pinst];
                bytes = (unsigned)((prows + 1) * Ip.ld1 * es + Ip.ids_bytes + (int)sizeof(Node));
            }
            const unsigned tot = __reduce_add_sync(grp, bytes);
            if (em && lane == __ffs(grp) - 1) {
                atomicAdd((unsigned long long *)&B.ictl[pinst].lvl_parents, (unsigned long long)n_em);
                atomicAdd((unsigned long long *)&B.ictl[pinst].lvl_par_bytes, (unsigned long long)tot);
            }
        }
    }
}

// ---------------------------------------------------------------------
// helpers for K2
// ---------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ const T *pool_of(const DevBuffers &B);
template <> __device__ __forceinline__ const double *pool_of<double>(const DevBuffers &B) { return B.dpool; }
template <> __device__ __forceinline__ const float *pool_of<float>(const DevBuffers &B) { return B.fpool; }

template <typename T>
__device__ __forceinline__ long long root_off(const InstDesc &I);
template <> __device__ __forceinline__ long long root_off<double>(const InstDesc &I) { return I.o_root; }
template <> __device__ __forceinline__ long long root_off<float>(const InstDesc &I) { return I.f_root; }

template <typename TS, typename TD>
__device__ __forceinline__ void warp_copy(TD *dst, const TS *src, int n)
{
    for (int e = lane_id(); e < n; e += 32) dst[e] = (TD)src[e];
}

// 16-byte vector copy of n elements (n a multiple of 4 elements, both ends
// 16-byte aligned: tableau offsets are multiples of 4 elements).
template <typename T>
__device__ __forceinline__ void warp_copy_v(T *dst, const T *src, int n)
{
    const int n4 = n * (int)sizeof(T) / 16;
    const int4 *s4 = reinterpret_cast<const int4 *>(src);
    int4 *d4 = reinterpret_cast<int4 *>(dst);
    for (int e = lane_id(); e < n4; e += 32) d4[e] = s4[e];
}

// Append a feasible (or, exhaustive, any) candidate as a node of `side`;
// stores its tableau when it can have children.  Returns the node index or -1.
// src_ld: row stride of `tab` (0: the plan's stride, copied as is).
// bulk: tab and ids are a shared-memory slot of the plan's layout (src_ld 0,
// TT = TS); lane 0 copies them with bulk stores (bulk_wait_read before the
// slot is written again, bulk_wait_all before the kernel ends).
template <typename TT, typename TS>
__device__ long long store_node(const DevBuffers &B, int side, int level, const InstDesc &I, int inst,
                                uint64_t lo, uint64_t hi, bool feasible, const TS *tab, const uint8_t *ids,
                                long long rec, long long hcap, int extra_flags, int src_ld = 0, bool bulk = false,
                                long long pre_idx = -1, int rows_store = -1, int cols_store = -1)
{
    const int lane = lane_id();
    Ctl *ctl = B.ctl;
    const bool need_tab = level < I.k_max;
    long long idx = 0, toff = -1, ioff = -1;
    if (lane == 0) {
        // one arena per kind, side 0 filled upward from 0, side 1 downward
        // from the top; the other side holds the parents and is fixed here
        // pre_idx >= 0: the caller's slot (a candidate's node lives at the
        // candidate's index)
        idx = pre_idx >= 0 ? pre_idx : (long long)atomicAdd((unsigned long long *)&ctl->n_node[side], 1ull);
        if (idx >= B.node_cap) { atomicOr(&ctl->overflow, OV_NODE); idx = -1; }
        if (need_tab && idx >= 0 && !*((volatile int *)&ctl->tab_full[side])) {
            const long long told = (long long)atomicAdd((unsigned long long *)&ctl->tab_used[side], (unsigned long long)I.tab_elems);
            const long long iold = (long long)atomicAdd((unsigned long long *)&ctl->ids_used[side], (unsigned long long)I.ids_bytes);
            if (told + I.tab_elems + ctl->tab_used[side ^ 1] > B.tab_cap ||
                iold + I.ids_bytes + ctl->ids_used[side ^ 1] > B.ids_cap) {
                // the arena is full: this node and the later ones of the level
                // keep no tableau (a reservation past the end is abandoned, so
                // the used counts only overstate); their children start from
                // the root tableau
                atomicExch(&ctl->tab_full[side], 1);
            } else {
                toff = side == 0 ? told : B.tab_cap - told - I.tab_elems;
                ioff = side == 0 ? iold : B.ids_cap - iold - I.ids_bytes;
            }
        }
    }
    idx = __shfl_sync(FULLMASK, idx, 0);
    toff = __shfl_sync(FULLMASK, toff, 0);
    ioff = __shfl_sync(FULLMASK, ioff, 0);
    if (idx < 0) return -1;
    if (need_tab && toff < 0) {
        // a node without a tableau (still in the hash: the subset test needs it)
        if (lane == 0) {
            atomicAdd((unsigned long long *)&B.ictl[inst].no_tab, 1ull);
            Node nd;
            nd.lo = lo; nd.hi = hi; nd.inst = inst;
            nd.flags = NODE_VALID | (feasible ? NODE_FEASIBLE : 0) | (extra_flags & ~NODE_CERT);
            nd.tab_off = -1; nd.ids_off = -1; nd.rec = rec;
            B.node[side][idx] = nd;
            if (feasible && !B.exhaustive) {
                if (!hash_insert(B.hash[side], hcap, hash_tag(ctl->epoch, level), inst, lo, hi))
                    atomicOr(&ctl->overflow, OV_HASH);
            }
        }
        return idx;
    }
    if (need_tab) {
        if (lane == 0) atomicAdd((unsigned long long *)&B.ictl[inst].stored, 1ull);
        TT *dst = (TT *)B.tab[side] + toff;
        if (bulk) {
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                // rows_store >= 0: the live rows and the objective row after them
                bulk_store(dst, tab, rows_store >= 0 ? (unsigned)((rows_store + 1) * I.ld1 * sizeof(TT))
                                                     : (unsigned)(I.tab_elems * sizeof(TT)));
                bulk_store(B.ids[side] + ioff, ids, (unsigned)I.ids_bytes);
                bulk_commit();
            }
        } else if (src_ld == 0) {
            warp_copy_v<TT>(dst, (const TT *)tab, I.tab_elems);
        } else {
            // re-stride (and convert) row by row; padding columns become 0
            const int ncol = I.nv + 1;
            for (int e = lane; e < I.tab_elems; e += 32) {
                const int i = e / I.ld1, j = e - i * I.ld1;
                dst[e] = (i <= I.M1 && j < ncol) ? (TT)tab[(size_t)i * src_ld + j] : TT(0);
            }
        }
        if (!bulk) {
            uint8_t *di = B.ids[side] + ioff;
            for (int e = lane; e < I.M1 + I.nv; e += 32) di[e] = ids[e];
        }
    }
    if (lane == 0) {
        Node nd;
        nd.lo = lo; nd.hi = hi; nd.inst = inst;
        nd.flags = NODE_VALID | (feasible ? NODE_FEASIBLE : 0) | extra_flags |
                   (rows_store >= 0 ? (rows_store + 1) << kNodeRowsShift : 0) |
                   (cols_store >= 0 ? (cols_store + 1) << kNodeColsShift : 0);
        nd.tab_off = toff; nd.ids_off = ioff; nd.rec = rec;
        B.node[side][idx] = nd;
        // the hash serves the subset test of the next level only
        if (feasible && !B.exhaustive && need_tab) {
            if (!hash_insert(B.hash[side], hcap, hash_tag(ctl->epoch, level), inst, lo, hi))
                atomicOr(&ctl->overflow, OV_HASH);
        }
    }
    return idx;
}

// Before an FP32 LP1 tableau is stored for the next level: each live column
// whose nonbasic variable is a slack of the set (lo, hi) -- fixed at zero in
// every descendant's LP, so never priced or updated usefully again -- moves
// past the right-hand side.  Per such column c: the last live column takes
// its place, the right-hand side moves one left, and c goes where the
// right-hand side was (rows 0..nrows, the objective row included); its id
// moves past the live ids.  Returns the live columns left.  The children's
// row updates then cover ncols + 1 <= 4 NCH values with fewer chunks.
__device__ __noinline__ int retire_fixed_columns(float *tab, int ld, int nrows, int ncols, uint8_t *nid, int nv,
                                                 uint64_t lo, uint64_t hi)
{
    const int lane = lane_id();
    for (;;) {
        bool f = false;
        if (lane < ncols) {
            const int id = (int)nid[lane] - nv;
            f = id >= 0 && id < 128 && mask_has(lo, hi, id);
        }
        const unsigned fm = __ballot_sync(FULLMASK, f) & (ncols >= 32 ? FULLMASK : ((1u << ncols) - 1u));
        if (!fm || ncols > 32) break;
        const int c = 31 - __clz(fm);   // the highest such column first
        const int last = ncols - 1;
        for (int r = lane; r <= nrows; r += 32) {
            float *row = tab + (size_t)r * ld;
            const float vc = row[c], vl = row[last], vb = row[ncols];
            row[c] = vl;
            row[last] = vb;
            row[ncols] = vc;
        }
        if (lane == 0) {
            const uint8_t t = nid[c];
            nid[c] = nid[last];
            nid[last] = t;
        }
        __syncwarp();
        ncols = last;
    }
    return ncols;
}

// An FP32 LP1 candidate without a final verdict, by one lane: with nid (the
// nonbasic ids of its final basis) to the FP64 dual certificate's queue, else
// -- or when that queue is full -- to the FP64 re-solve.  Not inlined: the
// LP1 kernel's registers stay with its simplex.
// Entries of the certificate queue: the candidate (its complement when the
// entry asks for the FP64 vertex check instead of the dual certificate), the
// nonbasic ids of its final FP32 basis, and the final tableau's growth (in
// the entry's last 4 bytes).
__device__ __noinline__ void queue_undecided_lp1(const DevBuffers &B, int w, const uint8_t *nid, int nv,
                                                 bool vertex = false, float growth = 0.0f)
{
    Ctl *ctl = B.ctl;
    if (nid) {
        const long long ci = (long long)atomicAdd((unsigned long long *)&ctl->n_q_cert, 1ull);
        if (ci < B.cert_cap) {
            uint8_t *e = B.cert_q + ci * B.cert_stride;
            *reinterpret_cast<int *>(e) = vertex ? ~w : w;
            for (int c = 0; c < nv; c++) e[4 + c] = nid[c];
            *reinterpret_cast<float *>(e + B.cert_stride - 4) = growth;
            return;
        }
    }
    const long long qi = (long long)atomicAdd((unsigned long long *)&ctl->n_q_lp1, 1ull);
    if (qi < B.q_cap) B.q_lp1[qi] = w; else atomicOr(&ctl->overflow, OV_QUEUE);
}

// LP1 of S' = S u {j} started from the root tableau (all slacks basic) when
// the parent kept no tableau: the root copied into the warp's slot (after
// the previous child's bulk store has read it), the root basis ids, and the
// objective sum_{i in S'} w_i as the sum of those slacks' rows.  Not
// inlined: the rare path keeps its registers out of the LP1 kernel's loop.
template <typename T>
__device__ __forceinline__ void cold_stage_lp1_body(const DevBuffers &B, const InstDesc &I, int inst, T *tab,
                                                    uint8_t *ids, uint64_t lo, uint64_t hi, int j)
{
    const int lane = lane_id();
    const int M1 = I.M1, nv = I.nv, ld = I.ld1;
    if (lane == 0) {
        bulk_wait_read();
        atomicAdd((unsigned long long *)&B.ictl[inst].lp1_cold, 1ull);
    }
    __syncwarp();
    warp_copy_v<T>(tab, pool_of<T>(B) + root_off<T>(I), I.tab_elems);
    uint8_t *bid = ids, *nid = ids + M1;
    int rows = M1;
    if constexpr (sizeof(T) == 4) {
        // the FP32 root (free variables basic, their rows dropped) and its ids
        const float *rid = B.fpool + I.f_root + I.tab_elems;
        for (int i = lane; i < M1 + nv; i += 32) ids[i] = (uint8_t)(int)rid[i];
        rows = I.root_rows;
    } else {
        for (int i = lane; i < M1; i += 32) bid[i] = (uint8_t)(nv + i);
        for (int c = lane; c < nv; c += 32) nid[c] = (uint8_t)c;
    }
    __syncwarp();
    T *obj = tab + (size_t)rows * ld;
    if (j < 64) lo |= 1ull << j; else hi |= 1ull << (j - 64);
    while (lo | hi) {
        int i;
        if (lo) { i = __ffsll((long long)lo) - 1; lo &= lo - 1; }
        else { i = 64 + __ffsll((long long)hi) - 1; hi &= hi - 1; }
        // w_i basic: its row joins the objective; nonbasic: -1 in its column
        int rho = -1;
        for (int r = lane; r < rows; r += 32) if (bid[r] == nv + i) rho = r;
        rho = __reduce_max_sync(FULLMASK, rho);
        if (rho >= 0) {
            const T *row = tab + (size_t)rho * ld;
            for (int cc = lane; cc <= nv; cc += 32) obj[cc] = xadd(obj[cc], row[cc]);
        } else {
            for (int cc = lane; cc < nv; cc += 32) if (nid[cc] == nv + i) obj[cc] = obj[cc] - T(1);
        }
        __syncwarp();
    }
}

__device__ __noinline__ void cold_stage_lp1_f32(const DevBuffers &B, const InstDesc &I, int inst, float *tab,
                                                uint8_t *ids, uint64_t lo, uint64_t hi, int j)
{
    cold_stage_lp1_body<float>(B, I, inst, tab, ids, lo, hi, j);
}

// ---------------------------------------------------------------------
// K2: LP1 feasibility, warm-started from the parent
// ---------------------------------------------------------------------
// T = double: the plain FP64 path (verdict z <= tol_feas).
// T = float : the FP32 pass of the mixed path; a verdict is final only when
//             certified (see below), otherwise the candidate is queued for
//             the FP64 re-solve.
template <typename T>
__global__ void __launch_bounds__(128) k_feasibility(DevBuffers B, Tol tol, SlotDims sd, int level, int chunk)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    constexpr bool mixed = sizeof(T) == 4;
    const int mld = mixed ? sd.maxLD1 : sd.maxLD1d;
    const size_t slot = feas_slot_bytes<T>(sd.maxM1, mld, sd.maxNv);
    unsigned char *base = smem + wib * slot;
    T *tab = (T *)base;
    uint8_t *ids = base + align16((((size_t)(sd.maxM1 + 1) * mld + 3) & ~(size_t)3) * sizeof(T));
    uint64_t *bar = (uint64_t *)(base + slot - 16);
    const int side = level & 1, pside = side ^ 1;
    Ctl *ctl = B.ctl;
    const long long ncand = ctl->n_cand;
    const long long wend = ncand < B.cand_cap ? ncand : B.cand_cap;
    const long long hcap = hash_cap_for(B, ncand);   // slots of this level's hash
    if (lane == 0) mbar_init(bar);
    __syncwarp();
    unsigned parity = 0;
    bool abort = false;
    const T tpiv = mixed ? (T)tol.tol_piv32 : (T)tol.tol_piv;
    const T tdj = mixed ? (T)tol.tol_dj32 : (T)tol.tol_dj;
    LocalInstCounters lc;
    lc.reset(-1);
    for (;;) {
        long long w0;
        if (lane == 0) w0 = (long long)atomicAdd(&ctl->ctr[0], (unsigned long long)chunk);
        w0 = __shfl_sync(FULLMASK, w0, 0);
        if (w0 >= wend || abort) break;
        const int cnt = wend - w0 < chunk ? (int)(wend - w0) : chunk;
        const Cand mine = lane < cnt ? B.cand[w0 + lane] : Cand{-1, 0};
        // candidate w's node goes to slot w (also when the FP64 re-solve
        // stores it); a candidate that stores none leaves an invalid record
        const long long nbase = w0;
        if (lane == 0) atomicMax((unsigned long long *)&ctl->n_node[side], (unsigned long long)(w0 + cnt));
        if (lane < cnt && nbase + lane < B.node_cap) {
            Node gap;
            gap.lo = 0; gap.hi = 0; gap.inst = 0; gap.flags = 0; gap.tab_off = -1; gap.ids_off = -1; gap.rec = -1;
            B.node[side][nbase + lane] = gap;
        }
        // lane t holds candidate t's parent tableau offset (for the prefetch)
        const long long my_toff = lane < cnt ? B.node[pside][mine.parent].tab_off : -1;
        const int my_inst = lane < cnt ? B.node[pside][mine.parent].inst : 0;
        // Candidates of their instance's last level (nothing is stored there)
        // decided without an LP: every nonbasic slack is zero at a certified
        // vertex of the parent's face, so a child whose new slack is nonbasic
        // in the parent's certified tableau -- or, below, in the final
        // tableau of a sibling certified feasible -- is feasible with that
        // vertex's certificate.  (The zero-pivot LP of such a child ends at
        // the same vertex.)  Not with records or exhaustive enumeration.
        const bool at_vertex = mixed && !B.rec && !B.exhaustive;
        unsigned done = 0;
        if (at_vertex) {
            bool q = false;
            if (lane < cnt) {
                const Node &pn = B.node[pside][mine.parent];
                const InstDesc &Il = B.inst[pn.inst];
                if ((pn.flags & NODE_CERT) && pn.ids_off >= 0 && level == Il.k_max) {
                    const uint8_t *pnid = B.ids[pside] + pn.ids_off + Il.M1;
                    const int want = Il.nv + mine.j;
                    for (int cc = 0; cc < Il.nv; cc++) q |= (int)pnid[cc] == want;
                }
            }
            done = __ballot_sync(FULLMASK, q);
        }
    for (int t = 0; t < cnt; t++) {
        const long long w = w0 + t;
        Cand c;
        c.parent = __shfl_sync(FULLMASK, mine.parent, t);
        c.j = __shfl_sync(FULLMASK, mine.j, t);
        {
            // the next candidate's parent into L2 while this one is solved
            const int np = __shfl_sync(FULLMASK, mine.parent, (t + 1) & 31);
            const long long ntoff = __shfl_sync(FULLMASK, my_toff, (t + 1) & 31);
            const int ninst = __shfl_sync(FULLMASK, my_inst, (t + 1) & 31);
            if (lane == 0 && t + 1 < cnt && np != c.parent && ntoff >= 0)
                bulk_prefetch_l2((const T *)B.tab[pside] + ntoff, (unsigned)(B.inst[ninst].tab_elems * sizeof(T)));
        }
        const Node par = B.node[pside][c.parent];
        const int inst = par.inst;
        const InstDesc &I = B.inst[inst];
        const InstCtl &ic = B.ictl[inst];
        const long long rec = (B.rec && ctl->rec_base + w < B.rec_cap) ? ctl->rec_base + w : -1;
        if (B.rec && rec < 0 && lane == 0) atomicOr(&ctl->overflow, OV_REC);
        if (ic.stopped || (I.budget > 0 && ic.cum_cand + ic.lvl_cand > I.budget)) {
            if (rec >= 0 && lane == 0) B.rec[rec].level = -1;
            continue;
        }
        if (inst != lc.inst) {
            if (lc.inst >= 0 && lane == 0) {
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].feasible, (unsigned long long)lc.a);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp1_piv, (unsigned long long)lc.b);
                atomicAdd(&B.ictl[lc.inst].feas_digest, (unsigned long long)lc.c);
            }
            lc.reset(inst);
        }
        if ((done >> t) & 1u) {
            // the last level stores no tableau and inserts nothing into the hash
            uint64_t lo = par.lo, hi = par.hi;
            if (c.j < 64) lo |= 1ull << c.j; else hi |= 1ull << (c.j - 64);
            lc.a++;
            lc.c += (long long)mask_digest(lo, hi);
            if (lane == 0) {
                if (nbase + t < B.node_cap) {
                    Node nd;
                    nd.lo = lo; nd.hi = hi; nd.inst = inst;
                    nd.flags = NODE_VALID | NODE_FEASIBLE;
                    nd.tab_off = -1; nd.ids_off = -1; nd.rec = -1;
                    B.node[side][nbase + t] = nd;
                } else {
                    atomicOr(&ctl->overflow, OV_NODE);
                }
            }
            continue;
        }
        const int M1 = I.M1, nv = I.nv, ld = I.ld1;
        // a parent kept without a tableau (the arena was full): the child
        // starts from the root tableau (all slacks basic) instead
        const bool cold = par.tab_off < 0;
        // the parent's live rows (FP32 tableaus drop the rows of basic free
        // variables; the objective row follows the live rows)
        const int prows = cold ? (mixed ? I.root_rows : M1) : node_rows(par.flags, M1);
        // the parent's live columns (FP32: the parent's own fixed slack
        // columns sit past the right-hand side, which is column pcols)
        const int pcols = (mixed && !cold) ? node_cols(par.flags, nv) : nv;
        fence_proxy_async_smem();
        __syncwarp();
        if (cold) {
            if constexpr (sizeof(T) == 4) cold_stage_lp1_f32(B, I, inst, tab, ids, par.lo, par.hi, c.j);
            else cold_stage_lp1_body<T>(B, I, inst, tab, ids, par.lo, par.hi, c.j);
        } else {
        // stage the parent tableau and basis: one bulk copy each, completing
        // on the warp's mbarrier (this warp's earlier accesses to the slot,
        // and the bulk store of the previous child, come first)
        if (lane == 0) {
            bulk_wait_read();
            const unsigned tb = mixed ? (unsigned)((prows + 1) * ld * sizeof(T)) : (unsigned)(I.tab_elems * sizeof(T));
            const unsigned ib = (unsigned)I.ids_bytes;
            mbar_expect(bar, tb + ib);
            bulk_load(tab, (const T *)B.tab[pside] + par.tab_off, tb, bar);
            bulk_load(ids, B.ids[pside] + par.ids_off, ib, bar);
        }
        if (!__all_sync(FULLMASK, mbar_wait(bar, parity))) {
            if (lane == 0) atomicOr(&ctl->overflow, OV_WAIT);
            (void)mbar_wait(bar, parity);   // the copies in flight, once more bounded
            abort = true;
            break;
        }
        parity ^= 1u;
        }
        uint8_t *bid = ids, *nid = ids + M1;
        T *obj = tab + (size_t)prows * ld;
        if (!cold) {
            // objective += w_j
            const int wid = nv + c.j;
            int rho = -1;
            for (int i = lane; i < prows; i += 32) if (bid[i] == wid) rho = i;
            rho = __reduce_max_sync(FULLMASK, rho);
            if (rho >= 0) {
                const T *row = tab + (size_t)rho * ld;
                for (int cc = lane; cc <= pcols; cc += 32) obj[cc] = xadd(obj[cc], row[cc]);
            } else {
                for (int cc = lane; cc < pcols; cc += 32) if (nid[cc] == wid) obj[cc] = obj[cc] - T(1);
            }
        }
        __syncwarp();
        Lp<T> L{tab, ld, prows, pcols, nv, bid, nid};
        int piv = 0;
        int st;
        int rows = prows;   // live rows after the simplex
        // FP32: the slacks of the parent's set stay at zero while nonbasic
        // (the parent is feasible: on that face the objective is w_j alone, so
        // the LP is min w_j there, the same verdict without detours through w_S),
        // and rows of free variables that enter the basis are dropped
        if constexpr (sizeof(T) == 4) st = warp_simplex_f32<kFastChunks>(L, tpiv, tdj, tol.max_pivots, tol.degen_switch, &piv,
                                                                          par.lo, par.hi, nv, true, &rows);
        else st = warp_simplex<T>(L, tpiv, tdj, tol.max_pivots, tol.degen_switch, &piv);
        const T z = obj[pcols];
        uint64_t lo = par.lo, hi = par.hi;
        if (c.j < 64) lo |= 1ull << c.j; else hi |= 1ull << (c.j - 64);
        bool feasible = false, decided = true, to_cert = false, to_vtx = false;
        float lp1_growth = 0.0f, lp1_minbeta = 0.0f;
        if (!mixed) {
            feasible = (st == LP_OPTIMAL) && ((double)z <= tol.tol_feas);
        } else {
            if (st != LP_OPTIMAL) decided = false;
            else {
                // the final tableau: whether a slack of S is basic, the
                // smallest basic slack and the element growth max |T_ij|
                // (~ |B^-1 N|), by which the FP32 errors of the basic values grow
                bool s_basic = false;
                T minb = pos_inf<T>(), gmax = T(1);
                if constexpr (sizeof(T) == 4) {
                    // FP32 rows are 16-byte aligned: four entries per access;
                    // the chunk holding the right-hand side (column pcols)
                    // gives that row's beta and its last live columns
                    const int cend = pcols >> 2, rem = pcols & 3;
                    for (int i = lane; i < rows; i += 32) {
                        const float *Ti = tab + (size_t)i * ld;
                        for (int c4 = 0; c4 < cend; c4++) {
                            const float4 v = reinterpret_cast<const float4 *>(Ti)[c4];
                            gmax = fmaxf(gmax, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
                        }
                        const float4 v = reinterpret_cast<const float4 *>(Ti)[cend];
                        gmax = fmaxf(gmax, fmaxf(fmaxf(rem > 0 ? fabsf(v.x) : 0.0f, rem > 1 ? fabsf(v.y) : 0.0f),
                                                 rem > 2 ? fabsf(v.z) : 0.0f));
                        const int id = bid[i];
                        if (id < nv) continue;
                        const int ci = id - nv;
                        if (ci < I.m && mask_has(lo, hi, ci)) s_basic = true;
                        const float bb = rem == 0 ? v.x : rem == 1 ? v.y : rem == 2 ? v.z : v.w;
                        if (bb < minb) minb = bb;
                    }
                    s_basic = __any_sync(FULLMASK, s_basic);
                    // the warp's max and min by integer reductions on order-preserving images
                    gmax = __uint_as_float(__reduce_max_sync(FULLMASK, __float_as_uint(gmax)));   // gmax >= 1
                    const unsigned km = __reduce_min_sync(FULLMASK, key_signed(minb));
                    minb = __uint_as_float((km & 0x80000000u) ? (km & 0x7fffffffu) : ~km);
                } else {
                    for (int i = lane; i < rows; i += 32) {
                        const T *Ti = tab + (size_t)i * ld;
                        for (int j = 0; j < pcols; j++) { const T a = xabs(Ti[j]); if (a > gmax) gmax = a; }
                        const int id = bid[i];
                        if (id < nv) continue;
                        const int ci = id - nv;
                        if (ci < I.m && mask_has(lo, hi, ci)) s_basic = true;
                        const T bb = Ti[pcols];
                        if (bb < minb) minb = bb;
                    }
                    s_basic = __any_sync(FULLMASK, s_basic);
#pragma unroll
                    for (int off = 16; off; off >>= 1) {
                        const T o = __shfl_xor_sync(FULLMASK, minb, off); if (o < minb) minb = o;
                        const T g = __shfl_xor_sync(FULLMASK, gmax, off); if (g > gmax) gmax = g;
                    }
                }
                lp1_growth = (float)gmax;
                lp1_minbeta = (float)minb;
                // feasible: every slack of S nonbasic (all rows of S tight at
                // the basic solution) and every basic slack clearly positive
                if (!s_basic && minb > (T)tol.margin_beta32 * gmax) feasible = true;
                // infeasible only by the FP64 dual certificate of this final
                // basis (k_lp1_cert); z32 near zero goes to the FP64 re-solve
                else {
                    decided = false;
                    to_cert = z > (T)tol.margin_z32 && nv <= 32 && !B.exhaustive;
                    // every slack of S' nonbasic and the smallest basic slack
                    // positive but inside the FP32 margin: at the instance's last
                    // level (no tableau to store) the FP64 vertex check decides
                    to_vtx = !to_cert && !s_basic && minb > (T)0 && level == I.k_max && nv <= 32 &&
                             !B.exhaustive;
                }
            }
        }
        lc.b += piv;
        if (rec >= 0 && lane == 0) {
            CandRec &R = B.rec[rec];
            R.mask_lo = lo; R.mask_hi = hi; R.level = level; R.parent = c.parent;
            R.lp1_status = st; R.lp1_pivots = piv; R.z = (double)z;
            R.feasible = feasible; R.licq = 0; R.optimal = 0; R.region = 0;
            R.lp2_status = LP_SKIPPED; R.lp2_pivots = 0; R.cheb_status = LP_SKIPPED; R.cheb_pivots = 0;
            R.t = __longlong_as_double(0x7ff8000000000000LL); R.r = R.t;
            R.inst = inst; R.fp64 = decided ? (mixed ? 0 : 1) : 0;
            R.lp1_growth = lp1_growth; R.lp1_minbeta = lp1_minbeta;
            R.lp1_bound = __longlong_as_double(0x7ff8000000000000LL);
        }
        if (!decided) {
            if (lane == 0) queue_undecided_lp1(B, (int)w, (to_cert || to_vtx) ? nid : nullptr, nv, to_vtx, lp1_growth);
            __syncwarp();
            continue;
        }
        if (feasible) { lc.a++; lc.c += (long long)mask_digest(lo, hi); }
        if (feasible || B.exhaustive) {
            int cols = -1;
            if (mixed && level < I.k_max) {
                if (rows != prows) {
                    // the objective row follows the live rows in the stored tableau
                    for (int cc = lane; cc < ld; cc += 32) tab[(size_t)rows * ld + cc] = obj[cc];
                    __syncwarp();
                }
                // certified: every slack of S' is nonbasic, and fixed in every
                // descendant -- its column moves past the right-hand side
                if constexpr (sizeof(T) == 4)
                    cols = feasible && !B.exhaustive
                               ? retire_fixed_columns(tab, ld, rows, pcols, nid, nv, lo, hi) : pcols;
            }
            store_node<T, T>(B, side, level, I, inst, lo, hi, feasible, tab, ids, rec, hcap,
                             mixed && feasible ? NODE_CERT : 0, 0, true, nbase + t, mixed ? rows : -1,
                             mixed ? cols : -1);
        }
        if (at_vertex && feasible && level == I.k_max) {
            // later siblings whose new slack is nonbasic at this vertex
            unsigned nb0 = 0, nb1 = 0, nb2 = 0, nb3 = 0;
            for (int cc = lane; cc < nv; cc += 32) {
                const int id = (int)nid[cc] - nv;
                if (id >= 0 && id < I.m) {
                    const unsigned bit = 1u << (id & 31);
                    const int wd = id >> 5;
                    nb0 |= wd == 0 ? bit : 0u; nb1 |= wd == 1 ? bit : 0u;
                    nb2 |= wd == 2 ? bit : 0u; nb3 |= wd == 3 ? bit : 0u;
                }
            }
            nb0 = __reduce_or_sync(FULLMASK, nb0); nb1 = __reduce_or_sync(FULLMASK, nb1);
            nb2 = __reduce_or_sync(FULLMASK, nb2); nb3 = __reduce_or_sync(FULLMASK, nb3);
            const int mj = mine.j;
            const unsigned wsel = mj < 32 ? nb0 : mj < 64 ? nb1 : mj < 96 ? nb2 : nb3;
            done |= __ballot_sync(FULLMASK, lane > t && lane < cnt && mine.parent == c.parent && ((wsel >> (mj & 31)) & 1u));
        }
    }
    }
    if (lane == 0) bulk_wait_all();
    if (lc.inst >= 0 && lane == 0) {
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].feasible, (unsigned long long)lc.a);
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp1_piv, (unsigned long long)lc.b);
        atomicAdd(&B.ictl[lc.inst].feas_digest, (unsigned long long)lc.c);
    }
}

// ---------------------------------------------------------------------
// K2b: FP64 LP1 re-solve (mixed precision), cold from the root tableau
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_lp1_fp64(DevBuffers B, Tol tol, SlotDims sd, int level)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const size_t slot = lp1_slot_bytes<double>(sd.maxM1, sd.maxLD1d, sd.maxNv);
    unsigned char *base = smem + wib * slot;
    double *tab = (double *)base;
    uint8_t *ids = base + align16((((size_t)(sd.maxM1 + 1) * sd.maxLD1d + 3) & ~(size_t)3) * sizeof(double));
    const int side = level & 1, pside = side ^ 1;
    Ctl *ctl = B.ctl;
    const long long nq = ctl->n_q_lp1 < B.q_cap ? ctl->n_q_lp1 : B.q_cap;
    const long long hcap = hash_cap_for(B, ctl->n_cand);   // slots of this level's hash
    for (;;) {
        long long x;
        if (lane == 0) x = (long long)atomicAdd(&ctl->ctr[2], 1ull);
        x = __shfl_sync(FULLMASK, x, 0);
        if (x >= nq) break;
        const long long w = B.q_lp1[x];
        const Cand c = B.cand[w];
        const Node par = B.node[pside][c.parent];
        const int inst = par.inst;
        const InstDesc &I = B.inst[inst];
        const int M1 = I.M1, nv = I.nv, ld = I.ld1d;
        uint64_t lo = par.lo, hi = par.hi;
        if (c.j < 64) lo |= 1ull << c.j; else hi |= 1ull << (c.j - 64);
        const double *root = B.dpool + I.o_root;
        warp_copy<double, double>(tab, root, (M1 + 1) * ld);
        uint8_t *bid = ids, *nid = ids + M1;
        for (int i = lane; i < M1; i += 32) bid[i] = (uint8_t)(nv + i);
        for (int j = lane; j < nv; j += 32) nid[j] = (uint8_t)j;
        __syncwarp();
        double *obj = tab + (size_t)M1 * ld;
        for (int cc = lane; cc <= nv; cc += 32) {
            double acc = 0.0;
            for (int i = 0; i < I.m; i++)
                if (mask_has(lo, hi, i)) acc = __dadd_rn(acc, root[(size_t)i * ld + cc]);
            obj[cc] = acc;
        }
        __syncwarp();
        Lp<double> L{tab, ld, M1, nv, nv, bid, nid};
        int piv = 0;
        const int st = warp_simplex<double>(L, tol.tol_piv, tol.tol_dj, tol.max_pivots, tol.degen_switch, &piv);
        const double z = obj[nv];
        const bool feasible = (st == LP_OPTIMAL) && (z <= tol.tol_feas);
        const long long rec = (B.rec && ctl->rec_base + w < B.rec_cap) ? ctl->rec_base + w : -1;
        if (lane == 0) {
            atomicAdd((unsigned long long *)&B.ictl[inst].fb_lp1, 1ull);
            atomicAdd((unsigned long long *)&B.ictl[inst].lp1_piv, (unsigned long long)piv);
            if (feasible) {
                atomicAdd((unsigned long long *)&B.ictl[inst].feasible, 1ull);
                atomicAdd(&B.ictl[inst].feas_digest, mask_digest(lo, hi));
            }
            if (rec >= 0) {
                CandRec &R = B.rec[rec];
                R.lp1_status = st; R.lp1_pivots += piv; R.z = z; R.feasible = feasible; R.fp64 |= 1;
            }
        }
        if (feasible || B.exhaustive)
            store_node<float, double>(B, side, level, I, inst, lo, hi, feasible, tab, ids, rec, hcap, 0, I.ld1d, false,
                                      w);
    }
}

// ---------------------------------------------------------------------
// K2c: FP64 dual certificate of FP32 LP1 optima (mixed precision)
// ---------------------------------------------------------------------
// LP1 of S' = S u {j}:  min c.w  s.t.  G u + w = beta, w >= 0, u free, with
// c_i = 1 on S' and 0 elsewhere (G = [A -F; 0 At], beta = [b; bt]: the FP64
// root tableau).  Its dual is  max beta.y  s.t.  G^T y = 0, y <= c, and by
// weak duality every such y gives z* >= beta.y.  The candidate's final FP32
// basis fixes y_i = c_i on its basic slacks; when every free variable is
// basic, the duals of the nv nonbasic slacks solve the square system
// M y_N = rhs,  M = G_N^T,  rhs = -G_B^T c_B.  The FP32 LP kept the parent's
// nonbasic slacks at zero, so their duals may exceed c_i = 1: y / s,
// s = max(1, max_{i in S'} y_i), is a feasible dual point as soon as
// y_i <= tol_dj (the FP64 simplex's own optimality tolerance) on the
// nonbasic slacks outside S'.  The set is infeasible when beta.y / s >
// tol_feas -- whatever path the FP32 simplex took, since only the final
// basis enters; every other candidate goes on to the FP64 re-solve.
//
// The system is solved by mixed-precision iterative refinement: an FP32 LU
// with partial pivoting, then corrections from FP64 residuals rhs - M y
// (three FP32 solves in all); y is accepted when the last FP64 residual is
// at FP64 rounding level (<= kCertResid * (|M| |y| + |rhs|)).  y, the sign
// tests and beta.y are FP64; only the correction solves run in FP32, so the
// FP64 pipe (a small fraction of the FP32 rate on this GPU) does the O(nv^2)
// residuals, not the O(nv^3) factorisation.  One warp per queued candidate,
// lane r owns row r of M (FP64 copy and FP32 LU in shared memory, row
// stride odd); instances with nv > 32 never reach this kernel.
constexpr int kCertSolves = 3;
constexpr double kCertResid = 1e-13;
// the FP64 vertex check's margin on the basic slacks, per unit of the final
// FP32 tableau's growth (the FP32 test uses margin_beta = 3e-5)
constexpr double kVertexMargin = 1e-10;

__host__ __device__ inline size_t cert_slot_bytes(int maxNv)
{
    const int nvm = maxNv < 32 ? maxNv : 32, ldm = nvm | 1;
    return align16((size_t)nvm * ldm * sizeof(double)) + align16((size_t)nvm * ldm * sizeof(float)) +
           align16((size_t)nvm * sizeof(double));
}

__device__ __forceinline__ double warp_max_d(double v)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_xor_sync(FULLMASK, v, off));
    return v;
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) v = __dadd_rn(v, __shfl_xor_sync(FULLMASK, v, off));
    return v;
}

__device__ __forceinline__ float warp_max_f(float v)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) v = fmaxf(v, __shfl_xor_sync(FULLMASK, v, off));
    return v;
}

__global__ void __launch_bounds__(128) k_lp1_cert(DevBuffers B, Tol tol, SlotDims sd, int level)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int nvm = sd.maxNv < 32 ? sd.maxNv : 32, ldm = nvm | 1;
    unsigned char *base = smem + wib * cert_slot_bytes(sd.maxNv);
    double *Md = (double *)base;                                                     // M, FP64
    float *Mf = (float *)(base + align16((size_t)nvm * ldm * sizeof(double)));      // its FP32 LU
    double *yv = (double *)((unsigned char *)Mf + align16((size_t)nvm * ldm * sizeof(float)));
    const int row = lane < nvm ? lane : 0;
    double *Mdr = Md + (size_t)row * ldm;   // this lane's row
    float *Mfr = Mf + (size_t)row * ldm;
    const int pside = (level & 1) ^ 1;
    Ctl *ctl = B.ctl;
    const long long nq = ctl->n_q_cert < B.cert_cap ? ctl->n_q_cert : B.cert_cap;
    for (;;) {
        long long x;
        if (lane == 0) x = (long long)atomicAdd(&ctl->ctr[8], 1ull);
        x = __shfl_sync(FULLMASK, x, 0);
        if (x >= nq) break;
        const uint8_t *e = B.cert_q + x * B.cert_stride;
        const int w0 = *reinterpret_cast<const int *>(e);
        // w0 < 0: the FP64 vertex check of a last-level candidate (below)
        const bool vtx = w0 < 0;
        const int w = vtx ? ~w0 : w0;
        const float growth = *reinterpret_cast<const float *>(e + B.cert_stride - 4);
        const Cand c = B.cand[w];
        const Node par = B.node[pside][c.parent];
        const int inst = par.inst;
        const InstDesc &I = B.inst[inst];
        const int nv = I.nv, ld = I.ld1d;
        uint64_t lo = par.lo, hi = par.hi;
        if (c.j < 64) lo |= 1ull << c.j; else hi |= 1ull << (c.j - 64);
        // the constraint rows: the FP64 root tableau (its FP32 copy, rounded
        // here, feeds the LU; the FP32 LP1 root is pre-pivoted and does not
        // hold them)
        const double *G = B.dpool + I.o_root;
        // lane cc < nv: the slack nonbasic in column cc (negative: a free variable)
        const int nb = lane < nv ? (int)e[4 + lane] - nv : 0;
        const bool all_slack = __all_sync(FULLMASK, nb >= 0) && nv <= nvm;
        bool ok = all_slack;
        double bound = 0.0;
        if (ok) {
            double rhs = 0.0, by = 0.0;
            if (vtx) {
                // the vertex: lane c row c of P (P[c][v] = G[nb_c][v]), rhs_c =
                // beta of row nb_c -- the nonbasic slacks at zero
                if (lane < nv) {
                    for (int v = 0; v < nv; v++) { Mdr[v] = G[(size_t)nb * ld + v]; Mfr[v] = (float)Mdr[v]; }
                    rhs = G[(size_t)nb * ld + nv];
                }
            } else {
            // lane v: row v of M (M[v][cc] = G[nb_cc][v]) and rhs_v = -sum over
            // the basic slacks i of S' of G[i][v]; by = their beta_i (y_i = 1)
            for (int cc = 0; cc < nv; cc++) {
                const int i = __shfl_sync(FULLMASK, nb, cc);
                if (lane < nv) { Mdr[cc] = G[(size_t)i * ld + lane]; Mfr[cc] = (float)Mdr[cc]; }
            }
            uint64_t rl = lo, rh = hi;
            while (rl | rh) {
                int i;
                if (rl) { i = __ffsll((long long)rl) - 1; rl &= rl - 1; }
                else { i = 64 + __ffsll((long long)rh) - 1; rh &= rh - 1; }
                if (__any_sync(FULLMASK, lane < nv && nb == i)) continue;   // nonbasic: its y is unknown
                if (lane < nv) rhs = __dsub_rn(rhs, G[(size_t)i * ld + lane]);
                by = __dadd_rn(by, G[(size_t)i * ld + nv]);
            }
            }
            __syncwarp();
            // FP32 LU with partial pivoting: the pivot of column col is the
            // unused row with the largest |entry| (smallest lane on ties); the
            // multipliers stay in the eliminated positions
            float amax = 0.0f;
            if (lane < nv) for (int cc = 0; cc < nv; cc++) amax = fmaxf(amax, fabsf(Mfr[cc]));
            amax = warp_max_f(amax);
            const float thr = 1e-6f * fmaxf(amax, 1.0f);
            bool used = lane >= nv;
            int mycol = -1, mypl = 0;   // mypl (lane col): the row that pivoted column col
            float ipiv = 0.0f;
            for (int col = 0; col < nv; col++) {
                const float a = used ? -1.0f : fabsf(Mfr[col]);
                const float amx = warp_max_f(a);
                if (!(amx > thr)) { ok = false; break; }
                const int pr = __ffs(__ballot_sync(FULLMASK, !used && a == amx)) - 1;
                const float *P = Mf + (size_t)pr * ldm;
                if (lane == col) mypl = pr;
                if (lane == pr) {
                    used = true;
                    mycol = col;
                    ipiv = __frcp_rn(P[col]);
                } else if (!used) {
                    const float f = __fdiv_rn(Mfr[col], P[col]);
                    Mfr[col] = f;
                    for (int cc = col + 1; cc < nv; cc++) Mfr[cc] = __fmaf_rn(-f, P[cc], Mfr[cc]);
                }
                __syncwarp();
            }
            if (ok) {
                double y = 0.0, rr = rhs;
                // max norms for the residual test, in FP32 (thresholds only;
                // amax is max |M| of the FP32 copy)
                const float rhsmax = warp_max_f(fabsf((float)rhs));
                for (int it = 0; it < kCertSolves; it++) {
                    // the correction d of M d = rr in FP32, scaled by a power of two
                    const float rm = warp_max_f(fabsf((float)rr));
                    if (!(rm > 0.0f)) break;
                    const int ex = ilogbf(rm);   // |ex| <= 149: 2^-ex and 2^ex are normal doubles
                    float b = (float)(rr * __longlong_as_double((long long)(1023 - ex) << 52));
                    for (int col = 0; col < nv; col++) {            // L (unit lower)
                        const float bp = __shfl_sync(FULLMASK, b, __shfl_sync(FULLMASK, mypl, col));
                        if (mycol > col) b = __fmaf_rn(-Mfr[col], bp, b);
                    }
                    float d = 0.0f;
                    for (int col = nv - 1; col >= 0; col--) {       // U
                        const int pr = __shfl_sync(FULLMASK, mypl, col);
                        const float dc = __shfl_sync(FULLMASK, b * ipiv, pr);
                        if (lane == col) d = dc;
                        if (mycol >= 0 && mycol < col) b = __fmaf_rn(-Mfr[col], dc, b);
                    }
                    y = fma((double)d, __longlong_as_double((long long)(1023 + ex) << 52), y);
                    // FP64 residual rr = rhs - M y
                    if (lane < nv) yv[lane] = y;
                    __syncwarp();
                    rr = rhs;
                    if (lane < nv) for (int cc = 0; cc < nv; cc++) rr = fma(-Mdr[cc], yv[cc], rr);
                    __syncwarp();
                }
                const float ymax = warp_max_f(lane < nv ? fabsf((float)y) : 0.0f);
                const float rres = warp_max_f(lane < nv ? fabsf((float)rr) : 0.0f);
                ok = rres <= (float)kCertResid * (amax * ymax + rhsmax) && ymax == ymax && ymax <= 1e30f;
                if (vtx) {
                    // every basic slack of the vertex (u = y, lane v) clearly
                    // positive in FP64: s_i = beta_i - G_i u > kVertexMargin *
                    // max(1, growth of the final FP32 tableau); the slacks of S'
                    // are nonbasic, so the vertex is feasible and z* = 0
                    if (lane < nv) yv[lane] = y;
                    __syncwarp();
                    const double thr = kVertexMargin * fmax(1.0, (double)growth);
                    bool bad = !ok;
                    double smin = pos_inf<double>();
                    for (int b0 = 0; b0 < I.M1; b0 += 32) {
                        const int i = b0 + lane;
                        bool nonbasic = false;
                        for (int cc = 0; cc < nv; cc++) nonbasic |= __shfl_sync(FULLMASK, nb, cc) == i;
                        if (i < I.M1 && !nonbasic) {
                            double si = G[(size_t)i * ld + nv];
                            for (int v = 0; v < nv; v++) si = fma(-G[(size_t)i * ld + v], yv[v], si);
                            if (!(si > thr)) bad = true;
                            smin = fmin(smin, si);
                        }
                    }
                    ok = !__any_sync(FULLMASK, bad);
#pragma unroll
                    for (int off = 16; off; off >>= 1) smin = fmin(smin, __shfl_xor_sync(FULLMASK, smin, off));
                    bound = smin;
                    __syncwarp();
                } else {
                // dual feasibility after scaling, and beta.y / s
                double smax = 1.0, byn = 0.0;
                bool bad = false;
                if (lane < nv) {
                    const bool inS = nb < I.m && mask_has(lo, hi, nb);
                    if (inS) smax = fmax(smax, y);
                    else bad = !(y <= tol.tol_dj);
                    byn = G[(size_t)nb * ld + nv] * y;
                }
                bad = __any_sync(FULLMASK, bad);
                smax = warp_max_d(smax);
                byn = warp_sum_d(byn);
                bound = __dadd_rn(by, byn) / smax;
                ok = ok && !bad && bound > tol.tol_feas;
                }
            }
        }
        if (vtx) {
            // the vertex check: a feasible node of the instance's last level
            // (no tableau), else the FP64 re-solve
            const long long rec = (B.rec && ctl->rec_base + w < B.rec_cap) ? ctl->rec_base + w : -1;
            if (ok) {
                if (lane == 0) {
                    InstCtl *ic = &B.ictl[inst];
                    atomicAdd((unsigned long long *)&ic->vtx_lp1, 1ull);
                    atomicAdd((unsigned long long *)&ic->feasible, 1ull);
                    atomicAdd(&ic->feas_digest, mask_digest(lo, hi));
                    if (rec >= 0) { B.rec[rec].feasible = 1; B.rec[rec].fp64 |= 16; B.rec[rec].lp1_bound = bound; }
                }
                store_node<float, double>(B, level & 1, level, I, inst, lo, hi, true, nullptr, nullptr, rec, 0, 0, 0,
                                          false, w);
            } else if (lane == 0) {
                const long long qi = (long long)atomicAdd((unsigned long long *)&ctl->n_q_lp1, 1ull);
                if (qi < B.q_cap) B.q_lp1[qi] = w; else atomicOr(&ctl->overflow, OV_QUEUE);
            }
            __syncwarp();
            continue;
        }
        if (lane == 0) {
            InstCtl *ic = &B.ictl[inst];
            const long long rec = (B.rec && ctl->rec_base + w < B.rec_cap) ? ctl->rec_base + w : -1;
            if (ok) {
                atomicAdd((unsigned long long *)&ic->cert_lp1, 1ull);
                if (rec >= 0) { B.rec[rec].fp64 |= 4; B.rec[rec].lp1_bound = bound; }
            } else {
                atomicAdd((unsigned long long *)&ic->cert_miss, 1ull);
                if (!all_slack) atomicAdd((unsigned long long *)&ic->cert_free, 1ull);
                const long long qi = (long long)atomicAdd((unsigned long long *)&ctl->n_q_lp1, 1ull);
                if (qi < B.q_cap) B.q_lp1[qi] = w; else atomicOr(&ctl->overflow, OV_QUEUE);
            }
        }
        __syncwarp();   // the slot is rewritten for the next entry
    }
}

// ---------------------------------------------------------------------
// K3: KKT factor, region rows, LP2 and the Chebyshev LP
// ---------------------------------------------------------------------
template <typename T>
struct KktData {
    const T *Wm, *Wh, *wc, *At, *bt;
};

template <typename T>
__device__ __forceinline__ KktData<T> kkt_data(const DevBuffers &B, const InstDesc &I);
template <> __device__ __forceinline__ KktData<double> kkt_data<double>(const DevBuffers &B, const InstDesc &I)
{
    return {B.dpool + I.o_Wm, B.dpool + I.o_Wh, B.dpool + I.o_wc, B.dpool + I.o_At, B.dpool + I.o_bt};
}
template <> __device__ __forceinline__ KktData<float> kkt_data<float>(const DevBuffers &B, const InstDesc &I)
{
    return {B.fpool + I.f_Wm, B.fpool + I.f_Wh, B.fpool + I.f_wc, B.fpool + I.f_At, B.fpool + I.f_bt};
}

// A region row [g | h] counts as zero (and is dropped before the Chebyshev
// LP, as utils.py:46-47 does for exact zeros) when max|g| <= tz * max(1,|h|):
// rows that vanish in exact arithmetic come out as rounding noise.
template <typename T>
__device__ __forceinline__ bool nonzero_row(const T *g, int p, double tz)
{
    T gmax = T(0);
    for (int cc = 0; cc < p; cc++) { const T a = xabs(g[cc]); if (a > gmax) gmax = a; }
    const T ah = xabs(g[p]);
    return gmax > (T)tz * (ah > T(1) ? ah : T(1));
}

constexpr int kDualMaxP = 6;      // p <= 6
constexpr int kDualMaxRows = 96;
constexpr int kDualLd = 12;       // row stride of the dual layout (conflict-free 128-bit loads)
enum : int { LP_BOUND = 6 };      // record status: "not optimal" proven by a dual bound (t = the bound)

struct OptResult {
    int licq, lp2_status, lp2_piv, cheb_status, cheb_piv, optimal, region;
    int cert = 0;       // 1: "not optimal" by the FP64 check of the FP32 dual basis (lp2_cert64)
    double t, r;
    double err;         // estimated relative error of the law (law_error), NaN when not computed
    bool decided;
};

// Workspace carved from one shared-memory slot
template <typename T>
struct OptWs {
    T *R, *Y, *Lam, *G, *Tb;
    uint8_t *ids;
    int *S;
    T *Psi, *Phi;   // mpLP (FP64 slots of batches with mpLP instances), else null
    __device__ OptWs() : Psi(nullptr), Phi(nullptr) {}
    __device__ OptWs(unsigned char *base, const SlotDims &sd)
    {
        const bool d = sizeof(T) == 8;
        const int rows = d ? sd.maxR2d : sd.maxR2;
        size_t o = 0;
        R = (T *)(base + o); o += align16((size_t)sd.maxK * sd.maxK * sizeof(T));
        Y = (T *)(base + o); o += align16((size_t)sd.maxK * sd.maxP1 * sizeof(T));
        Lam = (T *)(base + o); o += align16((size_t)sd.maxK * sd.maxP1 * sizeof(T));
        G = (T *)(base + o); o += align16((size_t)sd.maxR2 * sd.maxP1 * sizeof(T));
        Tb = (T *)(base + o); o += align16((size_t)(rows + 1) * (d ? sd.maxLD2d : sd.maxLD2) * sizeof(T));
        ids = base + o; o += align16((size_t)rows + sd.maxP1 + (sd.maxN ? sd.maxN + 1 : 0));
        S = (int *)(base + o); o += align16((size_t)sd.maxK * sizeof(int));
        Psi = Phi = nullptr;
        if (d && sd.maxN) {
            Psi = (T *)(base + o); o += align16((size_t)sd.maxK * sd.maxP1 * sizeof(T));
            Phi = (T *)(base + o);
        }
    }
};

// X = Wm[S,S]^-1 X in place, R the upper Cholesky factor of kkt_factor
// (k x k); X (k rows, stride ldx) holds the right-hand sides on entry.  Lane
// per column: a forward then a backward substitution, each accumulating in
// ascending l (the oracle's chol_solve_inplace).
template <typename T>
__device__ void chol_solve_inplace(const T *R, int k, T *X, int ldx, int ncols)
{
    for (int cc = lane_id(); cc < ncols; cc += 32) {
        for (int a = 0; a < k; a++) {
            T acc = X[a * ldx + cc];
            for (int l = 0; l < a; l++) acc = xfma(-R[l * k + a], X[l * ldx + cc], acc);
            X[a * ldx + cc] = xdiv(acc, R[a * k + a]);
        }
        for (int a = k - 1; a >= 0; a--) {
            T acc = X[a * ldx + cc];
            for (int l = a + 1; l < k; l++) acc = xfma(-R[a * k + l], X[l * ldx + cc], acc);
            X[a * ldx + cc] = xdiv(acc, R[a * k + a]);
        }
    }
    __syncwarp();
}

// mpLP: the multiplier law Psi = Wm[S,S]^-1 [WhL_S | wcL_S] (lambda(theta) =
// -(Psi theta + Psi_p)); Lambda of kkt_factor is then Gamma = Wm[S,S]^-1
// [F_S | b_S], the primal law x(theta) = A_S^T Gamma(theta).
__device__ void mplp_multipliers(const DevBuffers &B, const InstDesc &I, int k, OptWs<double> &ws)
{
    const int p = I.p, P1 = p + 1;
    for (int idx = lane_id(); idx < k * P1; idx += 32) {
        const int a = idx / P1, cc = idx - a * P1;
        ws.Psi[idx] = cc < p ? B.dpool[I.o_WhL + (size_t)ws.S[a] * p + cc] : B.dpool[I.o_wcL + ws.S[a]];
    }
    __syncwarp();
    chol_solve_inplace<double>(ws.R, k, ws.Psi, P1, P1);
}

// Stated error of a set's law: one step of iterative refinement in FP64.
// The residual [Wh_S | wc_S] - Wm[S,S] Lambda (and, for an mpLP instance,
// [WhL_S | wcL_S] - Wm[S,S] Psi) is solved with the same Cholesky factor;
// the largest correction relative to the largest law entry estimates the
// relative forward error of the multiplier law, and with it of the primal
// law (linear in Lambda).  Not applied: the law stays the oracle's values.
// Uses ws.Y (free once Lambda is known).  Warp-uniform result.
__device__ double law_error(const DevBuffers &B, const InstDesc &I, int k, OptWs<double> &ws)
{
    const int lane = lane_id();
    const int m = I.m, p = I.p, P1 = p + 1;
    const int *S = ws.S;
    const double *Wm = B.dpool + I.o_Wm;
    double *X = ws.Y;
    double num = 0.0, den = 0.0;
    for (int pass = 0; pass < (I.lp ? 2 : 1); pass++) {
        const double *L = pass ? ws.Psi : ws.Lam;
        const double *Wh = B.dpool + (pass ? I.o_WhL : I.o_Wh), *wc = B.dpool + (pass ? I.o_wcL : I.o_wc);
        for (int idx = lane; idx < k * P1; idx += 32) {
            const int a = idx / P1, cc = idx - a * P1;
            double acc = cc < p ? Wh[(size_t)S[a] * p + cc] : wc[S[a]];
            for (int b = 0; b < k; b++) acc = xfma(-Wm[(size_t)S[a] * m + S[b]], L[b * P1 + cc], acc);
            X[idx] = acc;
            den = fmax(den, fabs(L[idx]));
        }
        __syncwarp();
        chol_solve_inplace<double>(ws.R, k, X, P1, P1);
        for (int idx = lane; idx < k * P1; idx += 32) num = fmax(num, fabs(X[idx]));
        __syncwarp();
    }
    num = warp_max_d(num);
    den = warp_max_d(den);
    return den > 0.0 ? num / den : (num > 0.0 ? pos_inf<double>() : 0.0);
}

// Cholesky of Wm[S,S] (row-oriented; each entry accumulates in ascending l),
// then Y = R^-T [Wh_S | wc_S] and Lambda = R^-1 Y (lane per column).  FP64
// divides by the pivots (the oracle's operations); the FP32 screen keeps the
// correctly rounded reciprocal of each pivot on the diagonal and multiplies
// (one rounding more per entry, well inside the screen's margin).
// Returns 0 on success, 1 when a pivot fails the threshold thr (relative to
// the diagonal).  Fills ws.S with the sorted active set.
template <typename T>
__device__ int kkt_factor(const KktData<T> &D, const InstDesc &I, uint64_t lo, uint64_t hi, T thr,
                          OptWs<T> &ws, int *k_out, T *rho_out = nullptr)
{
    const int lane = lane_id();
    const int m = I.m, p = I.p, P1 = p + 1;
    const int k = mask_pop(lo, hi);
    *k_out = k;
    for (int i = lane; i < m; i += 32)
        if (mask_has(lo, hi, i)) ws.S[mask_rank(lo, hi, i)] = i;
    __syncwarp();
    const int *S = ws.S;
    T *R = ws.R;
    T rho = T(1);   // smallest pivot / diagonal ratio (lane 0)
    for (int a = 0; a < k; a++) {
        int fail = 0;
        if (lane == 0) {
            const T d0 = D.Wm[(size_t)S[a] * m + S[a]];
            T acc = d0;
            for (int l = 0; l < a; l++) acc = xfma(-R[l * k + a], R[l * k + a], acc);
            if (!(acc > thr * d0)) fail = 1;
            else if constexpr (sizeof(T) == 4) R[a * k + a] = __frcp_rn(__fsqrt_rn(acc));   // FP32: 1 / pivot
            else R[a * k + a] = xsqrt(acc);
            if (rho_out && !fail) {
                T rr;
                if constexpr (sizeof(T) == 4) rr = __fdividef(acc, d0); else rr = acc / d0;
                if (rr < rho) rho = rr;
            }
        }
        fail = __shfl_sync(FULLMASK, fail, 0);
        if (fail) return 1;
        __syncwarp();
        for (int b = a + 1 + lane; b < k; b += 32) {
            T acc = D.Wm[(size_t)S[a] * m + S[b]];
            for (int l = 0; l < a; l++) acc = xfma(-R[l * k + a], R[l * k + b], acc);
            if constexpr (sizeof(T) == 4) R[a * k + b] = acc * R[a * k + a];
            else R[a * k + b] = xdiv(acc, R[a * k + a]);
        }
        __syncwarp();
    }
    T *Y = ws.Y, *Lam = ws.Lam;
    for (int cc = lane; cc < P1; cc += 32) {
        for (int a = 0; a < k; a++) {
            T acc = (cc < p) ? D.Wh[(size_t)S[a] * p + cc] : D.wc[S[a]];
            for (int l = 0; l < a; l++) acc = xfma(-R[l * k + a], Y[l * P1 + cc], acc);
            if constexpr (sizeof(T) == 4) Y[a * P1 + cc] = acc * R[a * k + a];
            else Y[a * P1 + cc] = xdiv(acc, R[a * k + a]);
        }
        for (int a = k - 1; a >= 0; a--) {
            T acc = Y[a * P1 + cc];
            for (int l = a + 1; l < k; l++) acc = xfma(-R[a * k + l], Lam[l * P1 + cc], acc);
            if constexpr (sizeof(T) == 4) Lam[a * P1 + cc] = acc * R[a * k + a];
            else Lam[a * P1 + cc] = xdiv(acc, R[a * k + a]);
        }
    }
    __syncwarp();
    if (rho_out) *rho_out = __shfl_sync(FULLMASK, rho, 0);
    return 0;
}

// Region rows in the reference order (utils.py:39-57): lambda rows (S
// order), inactive rows (ascending), parameter box rows.  G is R2 x (p+1),
// each row [g | h] meaning g theta <= h.
// track = true also returns a bound on the magnitude of the terms summed
// into any row, max_i (sum_c |Wh_ic| + |wc_i| + sum_l |Wm_i,S_l| |Lambda_l|_1),
// the scale of the FP32 rounding error of the rows (warp-uniform result).
// out = nullptr writes ws.G (row stride p+1, h in column p); otherwise the
// rows go to out with row stride ldo and h in column hcol.  t0_out / g0_out
// (optional, warp-uniform results): min h over the constraint rows and
// max(1, max |g|) over all rows, the start value and growth reference of LP2.
template <typename T, bool track = false, bool LP = false>
__device__ T region_rows(const KktData<T> &D, const InstDesc &I, uint64_t lo, uint64_t hi, int k, OptWs<T> &ws,
                         T *out = nullptr, int ldo = 0, int hcol = 0, T *t0_out = nullptr, T *g0_out = nullptr,
                         bool lpm = LP)
{
    const int lane = lane_id();
    const int m = I.m, p = I.p, ncp = I.ncp, P1 = p + 1;
    const int *S = ws.S;
    const T *Lam = ws.Lam;
    // lambda rows: Lambda (mpQP) or Psi (lpm: an mpLP instance, whose
    // inactive rows come from Gamma in Lam; the error scales of those rows
    // then sum |Gamma_l|, not the multiplier rows' |Psi_l|)
    const T *LamL = lpm ? ws.Psi : Lam;
    T *G = out ? out : ws.G;
    const int ldg = out ? ldo : P1, hc = out ? hcol : p;
    T amax = T(0);
    T tmin = pos_inf<T>(), gmax = T(1);
    const bool want_t0 = t0_out != nullptr;
    T *labs = ws.Y;   // |Lambda_l|_1, Y is free once Lambda is known
    for (int a = lane; a < k; a += 32) {
        T rs = T(0);
        for (int cc = 0; cc < p; cc++) {
            const T v = LamL[a * P1 + cc];
            G[a * ldg + cc] = v;
            if (track) rs += xabs(v);
            if (want_t0 && xabs(v) > gmax) gmax = xabs(v);
        }
        const T h = -LamL[a * P1 + p];
        G[a * ldg + hc] = h;
        if (want_t0 && h < tmin) tmin = h;
        if (track) {
            rs += xabs(LamL[a * P1 + p]); if (rs > amax) amax = rs;
            if (lpm) {
                T gs = T(0);
                for (int cc = 0; cc <= p; cc++) gs += xabs(Lam[a * P1 + cc]);
                labs[a] = gs;
            } else {
                labs[a] = rs;
            }
            if (out) G[a * ldg + kRowScaleCol] = rs;
        }
    }
    if (track) __syncwarp();
    // inactive rows: g_c = -Wh_ic + sum_l Wm_i,S_l Lambda_lc (c < p) and
    // h = wc_i - sum_l Wm_i,S_l Lambda_lp, each summed in ascending l; the
    // columns go in register blocks of 8 so that Wm_i,S_l is read once per block
    constexpr int CB = 8;
    for (int i = lane; i < m; i += 32) {
        if (mask_has(lo, hi, i)) continue;
        const int pos = k + i - mask_rank(lo, hi, i);
        const T *wmi = D.Wm + (size_t)i * m;
        T rs = T(0);
        for (int c0 = 0; c0 < P1; c0 += CB) {
            T acc[CB];
#pragma unroll
            for (int j = 0; j < CB; j++) {
                const int cc = c0 + j;
                acc[j] = cc < p ? -D.Wh[(size_t)i * p + cc] : (cc == p ? D.wc[i] : T(0));
                if (track && cc <= p) rs += xabs(acc[j]);
            }
            for (int l = 0; l < k; l++) {
                const T w = wmi[S[l]];
                const T *lam = Lam + l * P1;
                if (track && c0 == 0) rs = xfma(xabs(w), labs[l], rs);
#pragma unroll
                for (int j = 0; j < CB; j++) {
                    const int cc = c0 + j;
                    if (cc < p) acc[j] = xfma(w, lam[cc], acc[j]);
                    else if (cc == p) acc[j] = xfma(-w, lam[cc], acc[j]);
                }
            }
#pragma unroll
            for (int j = 0; j < CB; j++) {
                if (c0 + j < p) {
                    G[pos * ldg + c0 + j] = acc[j];
                    if (want_t0 && xabs(acc[j]) > gmax) gmax = xabs(acc[j]);
                } else if (c0 + j == p) {
                    G[pos * ldg + hc] = acc[j];
                    if (want_t0 && acc[j] < tmin) tmin = acc[j];
                }
            }
        }
        if (track && rs > amax) amax = rs;
        if (track && out) G[pos * ldg + kRowScaleCol] = rs;
    }
    for (int ii = lane; ii < ncp; ii += 32) {
        for (int cc = 0; cc < p; cc++) {
            const T v = D.At[ii * p + cc];
            G[(m + ii) * ldg + cc] = v;
            if (want_t0 && xabs(v) > gmax) gmax = xabs(v);
        }
        G[(m + ii) * ldg + hc] = D.bt[ii];
        if (track && out) G[(m + ii) * ldg + kRowScaleCol] = T(0);   // the box rows are exact
    }
    if (want_t0) {
#pragma unroll
        for (int off = 16; off; off >>= 1) {
            const T o = __shfl_xor_sync(FULLMASK, tmin, off); if (o < tmin) tmin = o;
            const T g = __shfl_xor_sync(FULLMASK, gmax, off); if (g > gmax) gmax = g;
        }
        *t0_out = tmin;
        *g0_out = gmax;
    }
    if (track) {
#pragma unroll
        for (int off = 16; off; off >>= 1) { const T o = __shfl_xor_sync(FULLMASK, amax, off); if (o > amax) amax = o; }
    }
    __syncwarp();
    return amax;
}

// mpLP (Q = 0) with |S| = k < n: x is not fixed by S, so LP2 keeps a
// direction u in the null space of A_S (x = A_S^T Gamma(theta) + P u, P the
// projector onto that null space) and the stationarity residual
// (c + H theta) - A_S^T Psi(theta) = r0 + E theta as rows
// |r0 + E theta| <= tol_feas, as the reference's LP2 keeps x and the
// stationarity equalities (main.py:107-108).  Two phases: min sigma over
// rows +-(r0 + E theta) - sigma <= tol_feas (sigma free); when sigma* <= 0
// the row -sigma >= 0 is appended and max t solved from that basis.
// Columns theta (p), u (n), t, sigma; rows: the m margin rows (G, reference
// order, with A_i P in the u columns of the inactive rows), the ncp
// parameter rows, 2n residual rows.  The set is never a region.  Same
// operations as the oracle's lp2_short_mplp.
__device__ void lp2_short_mplp(const DevBuffers &B, const Tol &tol, const InstDesc &I, uint64_t lo, uint64_t hi,
                               int k, OptWs<double> &ws, OptResult &res)
{
    const int lane = lane_id();
    const int m = I.m, n = I.n, p = I.p, ncp = I.ncp, P1 = p + 1, ld = I.ld2lp;
    const int ncols = p + n + 2, ct = p + n, cs = p + n + 1;
    const int nrows = m + ncp + 2 * n;
    // Phi = Wm[S,S]^-1 A_S (x = A_S^T Gamma + P u, P = I - A_S^T Phi)
    for (int idx = lane; idx < k * n; idx += 32) {
        const int a = idx / n, j = idx - a * n;
        ws.Phi[idx] = B.dpool[I.o_QiAT + (size_t)j * m + ws.S[a]];
    }
    __syncwarp();
    chol_solve_inplace<double>(ws.R, k, ws.Phi, n, n);
    const double *G = ws.G, *Phi = ws.Phi, *Psi = ws.Psi;
    const double *At = B.dpool + I.o_QiAT, *Wm = B.dpool + I.o_Wm;
    const double *Hm = B.dpool + I.o_Hm, *cv = B.dpool + I.o_cv;
    const double *Ab = B.dpool + I.o_At, *bb = B.dpool + I.o_bt;
    const int *S = ws.S;
    double *T = ws.Tb;
    uint8_t *bid = ws.ids, *nid = ws.ids + nrows + 1;
    double t0 = pos_inf<double>();
    for (int r = lane; r < m; r += 32) { const double h = G[r * P1 + p]; if (h < t0) t0 = h; }
#pragma unroll
    for (int off = 16; off; off >>= 1) { const double o = __shfl_xor_sync(FULLMASK, t0, off); if (o < t0) t0 = o; }
    for (int idx = lane; idx < (nrows + 2) * ld; idx += 32) T[idx] = 0.0;
    __syncwarp();
    for (int r = lane; r < m; r += 32) {
        double *Tr = T + (size_t)r * ld;
        for (int cc = 0; cc < p; cc++) Tr[cc] = G[r * P1 + cc];
        Tr[ct] = 1.0;
        double beta = xfma(-1.0, t0, G[r * P1 + p]);
        if (!(beta > 0.0)) beta = 0.0;
        Tr[ncols] = beta;
    }
    for (int i = lane; i < m; i += 32) {
        if (mask_has(lo, hi, i)) continue;
        double *Tr = T + (size_t)(k + i - mask_rank(lo, hi, i)) * ld;
        for (int j = 0; j < n; j++) {
            double acc = At[(size_t)j * m + i];
            for (int l = 0; l < k; l++) acc = xfma(-Wm[(size_t)i * m + S[l]], Phi[l * n + j], acc);
            Tr[p + j] = acc;
        }
    }
    for (int ii = lane; ii < ncp; ii += 32) {
        double *Tr = T + (size_t)(m + ii) * ld;
        for (int cc = 0; cc < p; cc++) Tr[cc] = Ab[ii * p + cc];
        Tr[ncols] = bb[ii];
    }
    const double eps = tol.tol_feas;
    double rmax = 0.0;
    for (int i = lane; i < n; i += 32) {
        double *Tp = T + (size_t)(m + ncp + 2 * i) * ld, *Tn = Tp + ld;
        for (int cc = 0; cc < p; cc++) {
            double acc = Hm[i * p + cc];
            for (int l = 0; l < k; l++) acc = xfma(-At[(size_t)i * m + S[l]], Psi[l * P1 + cc], acc);
            Tp[cc] = acc;
            Tn[cc] = -acc;
        }
        double acc = cv[i];
        for (int l = 0; l < k; l++) acc = xfma(-At[(size_t)i * m + S[l]], Psi[l * P1 + p], acc);
        Tp[cs] = -1.0;
        Tn[cs] = -1.0;
        Tp[ncols] = xadd(eps, -acc);
        Tn[ncols] = xadd(eps, acc);
        if (fabs(acc) > rmax) rmax = fabs(acc);
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) { const double o = __shfl_xor_sync(FULLMASK, rmax, off); if (o > rmax) rmax = o; }
    const double s0 = xadd(rmax, -eps);
    __syncwarp();
    for (int r = m + ncp + lane; r < nrows; r += 32) {
        double beta = xadd(T[(size_t)r * ld + ncols], s0);
        if (!(beta > 0.0)) beta = 0.0;
        T[(size_t)r * ld + ncols] = beta;
    }
    for (int r = lane; r < nrows; r += 32) bid[r] = (uint8_t)(ncols + r);
    for (int cc = lane; cc < ncols; cc += 32) nid[cc] = (uint8_t)cc;
    double *obj = T + (size_t)nrows * ld;
    if (lane == 0) { obj[cs] = -1.0; obj[ncols] = s0; }
    __syncwarp();
    const double tpiv = tol.tol_piv, tdj = tol.tol_dj;
    int piv1 = 0, piv2 = 0;
    int st;
    {
        Lp<double> L{T, ld, nrows, ncols, ncols, bid, nid};
        st = warp_simplex<double>(L, tpiv, tdj, tol.max_pivots, tol.degen_switch, &piv1);
    }
    res.lp2_piv = piv1;
    if (st != LP_OPTIMAL) { res.lp2_status = st; return; }
    const double sig = obj[ncols];
    if (sig > 0.0) { res.lp2_status = LP_INFEASIBLE; res.t = -pos_inf<double>(); return; }
    // row nrows: s = -sigma >= 0 in the current basis (sigma basic in row rs,
    // or nonbasic in column qs); row nrows + 1: the objective -t
    int rs = -1, rt = -1, qs = -1, qt = -1;
    for (int r0 = 0; r0 < nrows; r0 += 32) {
        const int r = r0 + lane;
        const unsigned bs = __ballot_sync(FULLMASK, r < nrows && bid[r] == cs);
        const unsigned bt = __ballot_sync(FULLMASK, r < nrows && bid[r] == ct);
        if (bs && rs < 0) rs = r0 + __ffs(bs) - 1;
        if (bt && rt < 0) rt = r0 + __ffs(bt) - 1;
    }
    for (int c0 = 0; c0 < ncols; c0 += 32) {
        const int cc = c0 + lane;
        const unsigned bs = __ballot_sync(FULLMASK, cc < ncols && nid[cc] == cs);
        const unsigned bt = __ballot_sync(FULLMASK, cc < ncols && nid[cc] == ct);
        if (bs && qs < 0) qs = c0 + __ffs(bs) - 1;
        if (bt && qt < 0) qt = c0 + __ffs(bt) - 1;
    }
    double *Ts = T + (size_t)nrows * ld, *ob = Ts + ld;
    for (int cc = lane; cc <= ncols; cc += 32) {
        double vs, vo;
        if (rs >= 0) {
            const double v = T[(size_t)rs * ld + cc];
            vs = cc < ncols ? -v : xadd(-s0, -v);
        } else {
            vs = cc == qs ? 1.0 : (cc == ncols ? -s0 : 0.0);
        }
        if (rt >= 0) {
            const double v = T[(size_t)rt * ld + cc];
            vo = cc < ncols ? -v : xadd(-t0, -v);
        } else {
            vo = cc == qt ? 1.0 : (cc == ncols ? -t0 : 0.0);
        }
        Ts[cc] = vs;
        ob[cc] = vo;
    }
    if (lane == 0) bid[nrows] = (uint8_t)(ncols + nrows);
    __syncwarp();
    {
        Lp<double> L{T, ld, nrows + 1, ncols, ncols, bid, nid};
        st = warp_simplex<double>(L, tpiv, tdj, tol.max_pivots, tol.degen_switch, &piv2);
    }
    res.lp2_piv = piv1 + piv2;
    res.lp2_status = st;
    if (st == LP_OPTIMAL) {
        res.t = -ob[ncols];
        res.optimal = res.t > tol.tol_opt;
    } else if (st == LP_UNBOUNDED) {
        res.t = pos_inf<double>();
    }
}

// Chebyshev ball of the region rows in ws.G (utils.py:39-86): the box rows
// and the rows with a nonzero theta part, each normalised, then max r over
// the ball; res.cheb_status / cheb_piv / r / region.  Uses ws.Tb and ws.ids.
template <typename T>
__device__ void chebyshev_ball(const Tol &tol, const InstDesc &I, OptWs<T> &ws, OptResult &res)
{
    const int lane = lane_id();
    const int m = I.m, p = I.p, ncp = I.ncp, P1 = p + 1, R2 = m + ncp;
    const int ld2 = sizeof(T) == 4 ? I.ld2 : I.ld2d;
    const T tpiv = (T)tol.tol_piv;
    const T tdj = (T)tol.tol_dj;
    const T *G = ws.G;
    T *Tb = ws.Tb;
    uint8_t *bid = ws.ids, *nid = ws.ids + R2;
    // Chebyshev ball: keep box rows and rows with a nonzero theta part
    int nc = 0;
    for (int r0 = 0; r0 < R2; r0 += 32) {
        const int r = r0 + lane;
        bool keep = false;
        if (r < R2) {
            if (r >= m) keep = true;
            else keep = nonzero_row<T>(G + (size_t)r * P1, p, tol.tol_zero_row);
        }
        const unsigned km = __ballot_sync(FULLMASK, keep);
        if (keep) {
            const int np = nc + __popc(km & ((1u << lane) - 1u));
            const T *g = G + (size_t)r * P1;
            T acc = T(0);
            for (int cc = 0; cc < p; cc++) acc = xfma(g[cc], g[cc], acc);
            const T inv = xdiv(T(1), xsqrt(acc));
            T *tr = Tb + (size_t)np * ld2;
            T nn = T(0);
            for (int cc = 0; cc < p; cc++) { const T v = xmul(g[cc], inv); tr[cc] = v; nn = xfma(v, v, nn); }
            tr[p] = xsqrt(nn);
            tr[p + 1] = xmul(g[p], inv);
            bid[np] = (uint8_t)(P1 + np);
        }
        nc += __popc(km);
    }
    __syncwarp();
    T r0v = pos_inf<T>();
    for (int r = lane; r < nc; r += 32) {
        const T v = xdiv(Tb[(size_t)r * ld2 + p + 1], Tb[(size_t)r * ld2 + p]);
        if (v < r0v) r0v = v;
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) { const T o = __shfl_xor_sync(FULLMASK, r0v, off); if (o < r0v) r0v = o; }
    for (int r = lane; r < nc; r += 32) {
        T *tr = Tb + (size_t)r * ld2;
        T beta = xfma(-tr[p], r0v, tr[p + 1]);
        if (!(beta > T(0))) beta = T(0);
        tr[p + 1] = beta;
    }
    for (int cc = lane; cc <= P1; cc += 32) {
        T *ob = Tb + (size_t)nc * ld2;
        ob[cc] = (cc == p) ? T(1) : (cc == P1 ? -r0v : T(0));
        if (cc < P1) nid[cc] = (uint8_t)cc;
    }
    __syncwarp();
    {
        Lp<T> L{Tb, ld2, nc, P1, P1, bid, nid};
        int piv = 0;
        res.cheb_status = warp_simplex<T>(L, tpiv, tdj, tol.max_pivots, tol.degen_switch, &piv);
        res.cheb_piv = piv;
    }
    if (res.cheb_status == LP_OPTIMAL) {
        res.r = (double)(-Tb[(size_t)nc * ld2 + P1]);
        res.region = res.r >= tol.r_min;
    } else if (res.cheb_status == LP_UNBOUNDED) {
        res.r = pos_inf<double>();
    }
}

// FP64 check of a "not optimal" that the FP32 dual screen found but could not
// accept under its error margin (ill-conditioned KKT factors), run by the FP64
// kernel right after its KKT factor.  `basis` holds the p + 1 rows (numbered
// as region_rows orders them, one byte each) of the screen's final dual basis.
// Only those rows are formed in FP64 (region_rows' operations in its order,
// into Gb, (p + 1) x (p + 1) doubles); y solves [g_B | c_B]^T y = e_t in FP32
// (Gauss-Jordan with partial pivoting, equation e in lane e: any y serves),
// and for y+ = max(y, 0) and every feasible (theta, t) of LP2 with theta in
// the box
//     t <= (h_B.y+ + sum_c |(g_B^T y+)_c| reach_c) / (c_B.y+),
// evaluated in FP64 (the weak duality of lp2_dual_screen).  A bound below
// min(0, tol_opt) by more than 1e-7 of the magnitude of its terms leaves the
// FP64 LP2 optimum of the same rows below tol_opt, so the set is not optimal
// without the LP.  Returns 1 when proven; *bound_out the bound (NaN: none).
__device__ __noinline__ int lp2_cert64(const KktData<double> &D, const InstDesc &I, const int *S, const double *LamM,
                                       const double *Lam, int k, unsigned long long basis, double tol_opt,
                                       double *Gb, double *bound_out)
{
    constexpr int MP = kDualMaxP;
    const int lane = lane_id();
    const int m = I.m, p = I.p, P1 = p + 1;
    *bound_out = __longlong_as_double(0x7ff8000000000000LL);
    int b = -1;
    if (lane < P1) {
        const unsigned v = (unsigned)(basis >> (8 * lane)) & 0xffu;
        b = v == 0xffu ? -1 : (int)v;
    }
    if (!__all_sync(FULLMASK, lane >= P1 || (b >= 0 && b < m + I.ncp))) return 0;
    // the basic rows [g | h]: entry (i, c) in lane i * P1 + c (two rounds)
    for (int e = lane; e < P1 * P1; e += 32) {
        const int i = e / P1, c = e - i * P1;
        const int r = (int)((basis >> (8 * i)) & 0xffu);
        double v;
        if (r < k) {
            v = c < p ? LamM[r * P1 + c] : -LamM[r * P1 + p];
        } else if (r < m) {
            int ci = r - k;                                  // the (r - k)-th constraint outside S
            for (int l = 0; l < k; l++) if (S[l] <= ci) ci++;
            const double *wmi = D.Wm + (size_t)ci * m;
            double acc = c < p ? -D.Wh[(size_t)ci * p + c] : D.wc[ci];
            for (int l = 0; l < k; l++) {
                const double w = wmi[S[l]];
                acc = c < p ? xfma(w, Lam[l * P1 + c], acc) : xfma(-w, Lam[l * P1 + p], acc);
            }
            v = acc;
        } else {
            v = c < p ? D.At[(size_t)(r - m) * p + c] : D.bt[r - m];
        }
        Gb[e] = v;
    }
    __syncwarp();
    // y in FP32: lane e < P1 holds equation e over the unknowns y_0..y_p
    float a[MP + 2];
#pragma unroll
    for (int i = 0; i <= MP; i++) {
        const int bi = __shfl_sync(FULLMASK, b, i < P1 ? i : 0);
        a[i] = (i < P1 && lane < P1) ? (lane < p ? (float)Gb[i * P1 + lane] : (bi < m ? 1.0f : 0.0f)) : 0.0f;
    }
    a[MP + 1] = lane == p ? 1.0f : 0.0f;
    bool used = lane >= P1;
    int src = 0;
#pragma unroll
    for (int i = 0; i <= MP; i++) {
        if (i < P1) {
            float best = used ? -1.0f : fabsf(a[i]);
            int bl = lane;
#pragma unroll
            for (int off = 16; off; off >>= 1) {
                const float ob = __shfl_xor_sync(FULLMASK, best, off);
                const int ol = __shfl_xor_sync(FULLMASK, bl, off);
                if (ob > best || (ob == best && ol < bl)) { best = ob; bl = ol; }
            }
            if (!(best > 0.0f)) return 0;                   // singular basis
            const float inv = 1.0f / __shfl_sync(FULLMASK, a[i], bl);
            const float f = lane == bl ? 0.0f : a[i] * inv;
#pragma unroll
            for (int c = 0; c <= MP + 1; c++) {
                const float rb = __shfl_sync(FULLMASK, a[c], bl);
                a[c] = lane == bl ? rb * inv : __fmaf_rn(-f, rb, a[c]);
            }
            if (lane == bl) used = true;
            if (lane == i) src = bl;
        }
    }
    const float yv = __shfl_sync(FULLMASK, a[MP + 1], src);
    const double yp = lane < P1 ? (double)fmaxf(yv, 0.0f) : 0.0;   // fmaxf maps NaN to 0: still y >= 0
    // FP64: lane c < p (g_B^T y+)_c and sum y+ |g|; lane p c_B.y+; lane p + 1 h_B.y+ and sum y+ |h|
    double acc = 0.0, aab = 0.0;
#pragma unroll
    for (int i = 0; i <= MP; i++) {
        if (i < P1) {
            const double yi = __shfl_sync(FULLMASK, yp, i);
            const int bi = __shfl_sync(FULLMASK, b, i);
            if (lane < p) {
                const double g = Gb[i * P1 + lane];
                acc = fma(yi, g, acc);
                aab = fma(yi, fabs(g), aab);
            } else if (lane == p) {
                if (bi < m) acc += yi;
            } else if (lane == P1) {
                const double h = Gb[i * P1 + p];
                acc = fma(yi, h, acc);
                aab = fma(yi, fabs(h), aab);
            }
        }
    }
    // |theta_c| <= reach_c inside the box (rows c: s theta_c <= bt_c, p + c: -s' theta_c <= bt_{p+c}),
    // widened by 1e-12 for the rounding of the two quotients
    double reach = 0.0;
    if (lane < p) {
        const double hi = D.bt[lane] / D.At[(size_t)lane * p + lane];
        const double lo = D.bt[p + lane] / D.At[(size_t)(p + lane) * p + lane];
        reach = fmax(fabs(lo), fabs(hi)) * (1.0 + 1e-12);
    }
    const double cy = __shfl_sync(FULLMASK, acc, p);
    double num = lane < p ? fabs(acc) * reach : (lane == P1 ? acc : 0.0);
    double mag = lane < p ? aab * reach : (lane == P1 ? aab : 0.0);
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        num += __shfl_xor_sync(FULLMASK, num, off);
        mag += __shfl_xor_sync(FULLMASK, mag, off);
    }
    if (!(cy > 0.0)) return 0;
    const double bound = num / cy;
    *bound_out = bound;
    return bound < fmin(0.0, tol_opt) - 1e-7 * (mag / cy) ? 1 : 0;
}

// Optimality and region verdict of one feasible set (the FP64 path; the FP32
// screen of the mixed path is k_opt_screen).  LP: the instance is an mpLP.
// basis (mixed precision, mpQP over a box): the FP32 dual screen's final
// basis, checked by lp2_cert64 before the LP2 (~0: none).
template <typename T, bool LP = false>
__device__ OptResult eval_optimality(const DevBuffers &B, const Tol &tol, const InstDesc &I, uint64_t lo, uint64_t hi,
                                     OptWs<T> &ws, unsigned long long basis = ~0ull)
{
    const int lane = lane_id();
    const int m = I.m, p = I.p, ncp = I.ncp, P1 = p + 1, R2 = m + ncp;
    const int ld2 = sizeof(T) == 4 ? I.ld2 : I.ld2d;
    const KktData<T> D = kkt_data<T>(B, I);
    OptResult res;
    res.licq = 1; res.lp2_status = LP_SKIPPED; res.lp2_piv = 0; res.cheb_status = LP_SKIPPED; res.cheb_piv = 0;
    res.optimal = 0; res.region = 0; res.cert = 0;
    res.t = __longlong_as_double(0x7ff8000000000000LL); res.r = res.t; res.err = res.t;
    res.decided = true;
    const T tpiv = (T)tol.tol_piv;
    const T tdj = (T)tol.tol_dj;
    int k = 0;
    if (kkt_factor<T>(D, I, lo, hi, (T)tol.tol_licq, ws, &k)) {
        res.licq = 0; res.lp2_status = LP_LICQ_FAIL;
        return res;
    }
    if constexpr (LP) {
        static_assert(sizeof(T) == 8, "mpLP instances are evaluated in FP64");
        mplp_multipliers(B, I, k, ws);
    }
    // mpQP, and mpLP with |S| = n (the same LP2 rows, multipliers -Psi)
    if constexpr (sizeof(T) == 8) {
        if (basis != ~0ull && (!LP || k == I.n)) {
            double bound;
            if (lp2_cert64(D, I, ws.S, LP ? ws.Psi : ws.Lam, ws.Lam, k, basis, tol.tol_opt, ws.Tb, &bound)) {
                res.lp2_status = LP_BOUND;
                res.t = bound;
                res.cert = 1;
                return res;
            }
            __syncwarp();
        }
    }
    region_rows<T, false, LP>(D, I, lo, hi, k, ws);
    if constexpr (LP) {
        if (k < I.n) {
            // no unique law x(theta): LP2 keeps a null-space direction of A_S
            lp2_short_mplp(B, tol, I, lo, hi, k, ws, res);
            return res;
        }
    }
    const T *G = ws.G;
    // LP2: max t  s.t.  g theta + t <= h (constraint rows), At theta <= bt
    T t0 = pos_inf<T>();
    for (int r = lane; r < m; r += 32) { const T h = G[r * P1 + p]; if (h < t0) t0 = h; }
#pragma unroll
    for (int off = 16; off; off >>= 1) { const T o = __shfl_xor_sync(FULLMASK, t0, off); if (o < t0) t0 = o; }
    T *Tb = ws.Tb;
    uint8_t *bid = ws.ids, *nid = ws.ids + R2;
    for (int r = lane; r < R2; r += 32) {
        T *tr = Tb + (size_t)r * ld2;
        const T *g = G + (size_t)r * P1;
        for (int cc = 0; cc < p; cc++) tr[cc] = g[cc];
        const T cf = (r < m) ? T(1) : T(0);
        tr[p] = cf;
        T beta = xfma(-cf, t0, g[p]);
        if (!(beta > T(0))) beta = T(0);
        tr[p + 1] = beta;
        bid[r] = (uint8_t)(P1 + r);
    }
    for (int cc = lane; cc <= P1; cc += 32) {
        T *ob = Tb + (size_t)R2 * ld2;
        ob[cc] = (cc == p) ? T(1) : (cc == P1 ? -t0 : T(0));
        if (cc < P1) nid[cc] = (uint8_t)cc;
    }
    __syncwarp();
    {
        Lp<T> L{Tb, ld2, R2, P1, P1, bid, nid};
        int piv = 0;
        res.lp2_status = warp_simplex<T>(L, tpiv, tdj, tol.max_pivots, tol.degen_switch, &piv);
        res.lp2_piv = piv;
    }
    if (res.lp2_status == LP_OPTIMAL) {
        const T t = -Tb[(size_t)R2 * ld2 + P1];
        res.t = (double)t;
        res.optimal = res.t > tol.tol_opt;
    } else {
        if (res.lp2_status == LP_UNBOUNDED) res.t = pos_inf<double>();
    }
    if (!res.optimal) return res;
    chebyshev_ball<T>(tol, I, ws, res);
    if constexpr (sizeof(T) == 8) res.err = law_error(B, I, k, ws);
    return res;
}

__device__ void write_opt(const DevBuffers &B, const Node &nd, int level, const OptResult &res, bool fp64)
{
    Ctl *ctl = B.ctl;
    if (res.optimal) atomicAdd(&B.ictl[nd.inst].opt_digest, mask_digest(nd.lo, nd.hi));
    if (res.region) atomicAdd(&B.ictl[nd.inst].reg_digest, mask_digest(nd.lo, nd.hi));
    if (res.optimal) {
        const long long oi = (long long)atomicAdd((unsigned long long *)&ctl->n_opt, 1ull);
        if (oi < B.opt_cap) {
            OptRec o;
            o.lo = nd.lo; o.hi = nd.hi; o.inst = nd.inst; o.level = level; o.t = res.t; o.r = res.r;
            o.region = res.region; o.fp64 = fp64; o.rec = nd.rec; o.err = res.err;
            B.opt[oi] = o;
        } else {
            atomicOr(&ctl->overflow, OV_OPT);
        }
    }
    if (nd.rec >= 0 && B.rec) {
        CandRec &R = B.rec[nd.rec];
        R.licq = res.licq; R.optimal = res.optimal; R.region = res.region;
        R.lp2_status = res.lp2_status; R.lp2_pivots = res.lp2_piv;
        R.cheb_status = res.cheb_status; R.cheb_pivots = res.cheb_piv;
        R.t = res.t; R.r = res.r;
        if (fp64) R.fp64 |= 2;
        if (res.cert) R.fp64 |= 8;
    }
}

// Final FP64 verdicts of every feasible set of a level (the FP64 path;
// instantiated for T = double only).  LP = false takes the sets of mpQP
// instances, LP = true those of mpLP instances (launched only when a batch
// has one), so that the mpQP kernel carries no mpLP code.
template <typename T, bool LP>
__global__ void __launch_bounds__(128) k_optimality(DevBuffers B, Tol tol, SlotDims sd, int level)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const size_t slot = opt_slot_bytes<T>(sd);
    OptWs<T> ws(smem + wib * slot, sd);
    const int side = level & 1;
    Ctl *ctl = B.ctl;
    const long long nn = ctl->n_node[side] < B.node_cap ? ctl->n_node[side] : B.node_cap;
    static_assert(sizeof(T) == 8, "the FP32 screen is k_opt_screen");
    LocalInstCounters lc;
    lc.reset(-1);
    for (;;) {
        long long x;
        if (lane == 0) x = (long long)atomicAdd(&ctl->ctr[LP ? 6 : 3], 1ull);
        x = __shfl_sync(FULLMASK, x, 0);
        if (x >= nn) break;
        const Node nd = B.node[side][x];
        if ((nd.flags & (NODE_VALID | NODE_FEASIBLE)) != (NODE_VALID | NODE_FEASIBLE)) continue;
        const InstDesc &I = B.inst[nd.inst];
        if (level < I.k_min || (I.lp != 0) != LP) continue;
        if (nd.inst != lc.inst) {
            if (lc.inst >= 0 && lane == 0) {
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].optimal, (unsigned long long)lc.a);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].region, (unsigned long long)lc.b);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp2_piv, (unsigned long long)lc.c);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].cheb_piv, (unsigned long long)lc.d);
            }
            lc.reset(nd.inst);
        }
        const OptResult res = eval_optimality<T, LP>(B, tol, I, nd.lo, nd.hi, ws);
        lc.c += res.lp2_piv;
        lc.d += res.cheb_piv;
        lc.a += res.optimal;
        lc.b += res.region;
        if (lane == 0) write_opt(B, nd, level, res, true);
        __syncwarp();
    }
    if (lc.inst >= 0 && lane == 0) {
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].optimal, (unsigned long long)lc.a);
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].region, (unsigned long long)lc.b);
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp2_piv, (unsigned long long)lc.c);
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].cheb_piv, (unsigned long long)lc.d);
    }
}

template <bool LP>
__global__ void __launch_bounds__(128) k_optimality_fp64(DevBuffers B, Tol tol, SlotDims sd, int level)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const size_t slot = opt_slot_bytes<double>(sd);
    OptWs<double> ws(smem + wib * slot, sd);
    const int side = level & 1;
    Ctl *ctl = B.ctl;
    // the FP64 queue, then the sets queued with an FP32 dual basis to check first
    const long long nq = ctl->n_q_opt < B.q_cap ? ctl->n_q_opt : B.q_cap;
    const long long nc = ctl->n_q_c2 < B.q_c2_cap ? ctl->n_q_c2 : B.q_c2_cap;
    for (;;) {
        long long x;
        if (lane == 0) x = (long long)atomicAdd(&ctl->ctr[LP ? 7 : 4], 1ull);
        x = __shfl_sync(FULLMASK, x, 0);
        if (x >= nq + nc) break;
        unsigned long long basis = ~0ull;
        int xn;
        if (x < nq) xn = B.q_opt[x];
        else { xn = B.q_c2[x - nq]; basis = B.q_c2b[x - nq]; }
        const Node nd = B.node[side][xn];
        const InstDesc &I = B.inst[nd.inst];
        if ((I.lp != 0) != LP) continue;
        const OptResult res = eval_optimality<double, LP>(B, tol, I, nd.lo, nd.hi, ws, basis);
        if (lane == 0) {
            InstCtl *ic = &B.ictl[nd.inst];
            atomicAdd((unsigned long long *)&ic->fb_opt, 1ull);
            if (res.cert) atomicAdd((unsigned long long *)&ic->cert_lp2, 1ull);
            atomicAdd((unsigned long long *)&ic->lp2_piv, (unsigned long long)res.lp2_piv);
            atomicAdd((unsigned long long *)&ic->cheb_piv, (unsigned long long)res.cheb_piv);
            if (res.optimal) atomicAdd((unsigned long long *)&ic->optimal, 1ull);
            if (res.region) atomicAdd((unsigned long long *)&ic->region, 1ull);
            write_opt(B, nd, level, res, true);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------
// level 0, finalisation and reset
// ---------------------------------------------------------------------
// One warp per instance: the empty set with the root LP1 tableau.
// ---------------------------------------------------------------------
// FP32 LP2 screen of the mixed path
// ---------------------------------------------------------------------

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) { const float o = __shfl_xor_sync(FULLMASK, v, off); if (o > v) v = o; }
    return v;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(FULLMASK, v, off);
    return v;
}


// Dual bound of LP2 for an instance whose parameter set is a box
// lo <= theta <= hi (constraint rows m..m+2p-1: theta_c <= hi_c scaled, then
// -theta_c <= -lo_c scaled).  LP2 is
//     max t  s.t.  g_r theta + c_r t <= h_r   (c_r = 1 for r < m, 0 for box rows).
// For every y >= 0 with c.y > 0 and every feasible (theta, t),
//     t <= (h.y + sum_c |(G^T y)_c| reach_c) / (c.y),   reach_c = max(|lo_c|, |hi_c|),
// so a y whose bound is below -thr proves "not optimal".  The y are the basic
// solutions of a revised primal simplex on the dual LP
//     min h.y  s.t.  G^T y = 0,  c.y = 1,  y >= 0,
// started at the best single-row bound (row i* and, per parameter, the box
// row that cancels g_{i*,c}) and stopped as soon as its objective is below
// -thr; the bound is then recomputed from max(y, 0) and the rows, so FP32
// drift in the basis inverse cannot make a "not optimal" verdict unsound.
// Lanes 0..p hold one basic variable each (row index, value, row of B^-1:
// binv[0..p-1] for the theta equations, binvp for c.y = 1); every lane holds
// the prices (pi[0..p-1]: a vertex theta; pip: the objective).
// Row layout (stride kDualLd): columns 0..5 g_r (zero beyond p), 6 c_r, 7 h_r.
// Returns 1 when "not optimal" is proven; *it_out iterations, *bound_out the
// last verified bound (+inf when none was computed).
// thr: the threshold from the largest row error scale (when to try the
// bound); ethr: threshold per unit of error scale -- a bound is final when it
// is below -ethr * sum_r y_r e_r / (c.y), e_r the error scale of row r
// (column kRowScaleCol), which is at most thr
__device__ int lp2_dual_screen(const float *T, int m, int R2, int p, const float *blo, const float *bhi, float thr,
                               float ethr, float tol_piv, float tol_dj, int max_it, int degen_switch, int *it_out,
                               float *bound_out, unsigned long long *basis_out = nullptr)
{
    constexpr int NR = kDualMaxRows / 32;
    constexpr int MP = kDualMaxP;
    constexpr int LD = kDualLd;
    const int lane = lane_id();
    const int P1 = p + 1;
    auto row8 = [&](int r, float *a) {
        const float4 v0 = reinterpret_cast<const float4 *>(T + r * LD)[0];
        const float4 v1 = reinterpret_cast<const float4 *>(T + r * LD)[1];
        a[0] = v0.x; a[1] = v0.y; a[2] = v0.z; a[3] = v0.w; a[4] = v1.x; a[5] = v1.y; a[6] = v1.z; a[7] = v1.w;
    };
    float lo[MP], hi[MP];
#pragma unroll
    for (int c = 0; c < MP; c++) { lo[c] = c < p ? blo[c] : 0.0f; hi[c] = c < p ? bhi[c] : 0.0f; }
    // best single-row bound b_r = h_r - min over the box of g_r theta (r < m)
    unsigned bkey = 0xffffffffu;
    int bi = -1;
    for (int r = lane; r < m; r += 32) {
        float a[8];
        row8(r, a);
        float b = a[7];
#pragma unroll
        for (int c = 0; c < MP; c++) b -= a[c] > 0.0f ? a[c] * lo[c] : a[c] * hi[c];
        const unsigned k = key_signed(b);
        if (bi < 0 || k < bkey) { bkey = k; bi = r; }
    }
    const int istar = warp_argmin(bkey, (unsigned)bi, bi);
    // start basis: lane 0 row i*, lane 1+c the box row of parameter c that
    // cancels g_{i*,c} (the upper row when g <= 0); pi = (box corner, b*)
    float gi[8];
    row8(istar, gi);
    float binv[MP], pi[MP], binvp = 0.0f, y = 0.0f;
    float pip = gi[7];
    int bidx = -1;
#pragma unroll
    for (int c = 0; c < MP; c++) {
        binv[c] = 0.0f;
        pi[c] = 0.0f;
        if (c < p) {
            const bool upper = !(gi[c] > 0.0f);
            const int row = m + (upper ? c : p + c);
            const float sc = T[row * LD + c];                 // the box row's coefficient
            pi[c] = upper ? hi[c] : lo[c];
            const float yc = __fdividef(-gi[c], sc);          // >= 0
            pip = __fmaf_rn(yc, T[row * LD + 7], pip);
            if (lane == 1 + c) { bidx = row; y = yc; binv[c] = __fdividef(1.0f, sc); binvp = yc; }
        }
    }
    if (lane == 0) { bidx = istar; y = 1.0f; binvp = 1.0f; }
    // basic flags of the own rows lane, lane+32, lane+64
    unsigned basic = 0;
#pragma unroll
    for (int s = 0; s < NR; s++) {
        const int r = lane + 32 * s;
        bool b = r == istar;
        if (r >= m && r < m + p) b = !(T[istar * LD + (r - m)] > 0.0f);
        else if (r >= m + p && r < m + 2 * p) b = T[istar * LD + (r - m - p)] > 0.0f;
        if (b) basic |= 1u << s;
    }
    float reach = 0.0f;
#pragma unroll
    for (int c = 0; c < MP; c++) if (lane == c) reach = fmaxf(fabsf(lo[c]), fabsf(hi[c]));
    // verified bound from max(y, 0): lane c < p sums (G^T y)_c, lane p c.y, lane p+1 h.y
    const int vcol = lane < p ? lane : (lane == p ? 6 : 7);
    float thr_row = thr;   // the per-row threshold of the last verified y
    auto verify = [&]() -> float {
        float acc = 0.0f, ey = 0.0f;
#pragma unroll
        for (int i = 0; i <= MP; i++) {
            if (i < P1) {
                const float yi = __shfl_sync(FULLMASK, fmaxf(y, 0.0f), i);
                const int ri = __shfl_sync(FULLMASK, bidx, i);
                if (lane <= P1) acc = __fmaf_rn(yi, T[ri * LD + vcol], acc);
                ey = __fmaf_rn(yi, T[ri * LD + kRowScaleCol], ey);
            }
        }
        const float cy = __shfl_sync(FULLMASK, acc, p);
        const float num = warp_sum(lane < p ? fabsf(acc) * reach : (lane == P1 ? acc : 0.0f));
        thr_row = cy > 0.0f ? fminf(thr, ethr * __fdividef(ey, cy)) : thr;
        return cy > 0.0f ? __fdividef(num, cy) : pos_inf<float>();
    };

    int it = 0, degen = 0, proven = 0;
    bool bland = false;
    float bound = pos_inf<float>();
    for (;;) {
        if (pip < -thr) {
            bound = verify();
            if (bound < -thr_row) { proven = 1; break; }
        }
        if (it >= max_it) break;
        // pricing: most negative reduced cost d_r = h_r - pi.a_r (Bland: smallest r)
        unsigned key = 0xffffffffu, kid = 0xffffffffu;
        int kq = -1;
        float dbest = 0.0f;
        // not unrolled: the kernel is bound by instruction fetch (the code of
        // the three row slots would be three copies of this body)
#pragma unroll 1
        for (int s = 0; s < NR; s++) {
            const int r = lane + 32 * s;
            if (r < R2 && !((basic >> s) & 1u)) {
                float a[8];
                row8(r, a);
                float d = __fmaf_rn(-pip, a[6], a[7]);
#pragma unroll
                for (int c = 0; c < MP; c++) d = __fmaf_rn(-pi[c], a[c], d);
                if (d < -tol_dj) {
                    const unsigned k = bland ? 0u : ~key_of(-d);
                    if (kq < 0 || k < key || (k == key && (unsigned)r < kid)) { key = k; kid = r; kq = r; dbest = d; }
                }
            }
        }
        const int q = warp_argmin(key, kid, kq);
        if (q < 0) {                       // dual optimum: pip is the LP2 optimum t*
            bound = verify();
            proven = bound < -thr_row;
            break;
        }
        const float dq = __shfl_sync(FULLMASK, dbest, q & 31);
        // entering column u = B^-1 a_q; ratio test over the basic positions
        float aq[8];
        row8(q, aq);
        float u = binvp * aq[6];
#pragma unroll
        for (int c = 0; c < MP; c++) u = __fmaf_rn(binv[c], aq[c], u);
        unsigned rk = 0xffffffffu, rid = 0xffffffffu;
        int rl = -1;
        if (lane < P1 && u > tol_piv) { rk = key_of(__fdividef(fmaxf(y, 0.0f), u)); rid = (unsigned)bidx; rl = lane; }
        const int l = warp_argmin(rk, rid, rl);
        if (l < 0) break;                  // unbounded dual: not possible for LP2 in exact arithmetic
        const float ul = __shfl_sync(FULLMASK, u, l);
        const float yl = __shfl_sync(FULLMASK, fmaxf(y, 0.0f), l);
        const int oldb = __shfl_sync(FULLMASK, bidx, l);
        const float inv = __fdividef(1.0f, ul);
        const float theta = yl * inv;
        const float f = u * inv, fp = dq * inv;
        // the pivot on row l of B^-1 (its old values, one element at a time)
        const bool own = lane == l, other = lane < P1 && lane != l;
#pragma unroll
        for (int c = 0; c < MP; c++) {
            const float rj = __shfl_sync(FULLMASK, binv[c], l);
            binv[c] = own ? rj * inv : (other ? __fmaf_rn(-f, rj, binv[c]) : binv[c]);
            pi[c] = __fmaf_rn(fp, rj, pi[c]);
        }
        {
            const float rj = __shfl_sync(FULLMASK, binvp, l);
            binvp = own ? rj * inv : (other ? __fmaf_rn(-f, rj, binvp) : binvp);
            pip = __fmaf_rn(fp, rj, pip);
        }
        if (own) { y = theta; bidx = q; }
        else if (other) y = __fmaf_rn(-theta, u, y);
        if (lane == (q & 31)) basic |= 1u << (q >> 5);
        if (lane == (oldb & 31)) basic &= ~(1u << (oldb >> 5));
        it++;
        degen = (theta == 0.0f) ? degen + 1 : 0;
        bland = degen >= degen_switch;
    }
    *it_out = it;
    *bound_out = bound;
    if (basis_out) {
        // the final basis, row numbers of lanes 0..p (0xff past p)
        unsigned long long word = ~0ull;
#pragma unroll
        for (int i = 0; i <= MP; i++) {
            const int bi = __shfl_sync(FULLMASK, bidx, i);
            if (i < P1) word = (word & ~(0xffull << (8 * i))) | ((unsigned long long)(bi & 0xff) << (8 * i));
        }
        *basis_out = word;
    }
    return proven;
}

// per-warp shared memory of the screen: KKT workspace (R, Y, Lambda, S),
// the LP2 tableau (R2+1) x ld2 and its basis ids (R2 + P1)
// (the primal route also keeps the unpivoted region rows G, R2 x (p+1))
__host__ __device__ inline size_t screen_warp_bytes(const SlotDims &sd, int route)
{
    return align16((size_t)sd.maxK * sd.maxK * 4) + 2 * align16((size_t)sd.maxK * sd.maxP1 * 4) +
           align16((size_t)sd.maxK * sizeof(int)) + align16((size_t)(sd.maxR2 + 1) * sd.maxLD2 * 4) +
           align16((size_t)sd.maxR2 + sd.maxP1) + (route == 1 ? align16((size_t)sd.maxR2 * sd.maxP1 * 4) : 0) +
           (route != 1 && sd.maxN ? align16((size_t)sd.maxK * sd.maxP1 * 4) : 0);
}

// The FP32 screen of every feasible set of a level, one warp per set.  Only a
// clear "not optimal" is final; every other set is queued for
// k_optimality_fp64.  mode 0: the dual bound where the parameter set is a box
// (p <= 6, at most 96 rows), the primal tableau screen elsewhere; mode 1:
// the primal tableau screen everywhere.  The two routes are two kernels
// (ROUTE 0 dual, ROUTE 1 primal), each taking only its own sets, so that
// each carries only its own code.
__host__ __device__ __forceinline__ bool dual_route(int mode, const InstDesc &I, const SlotDims &sd)
{
    return mode == 0 && I.box && !I.lp && I.p <= kDualMaxP && I.m + I.ncp <= kDualMaxRows && sd.maxLD2 >= kDualLd;
}

// The instances whose sets the first stage of the dual screen takes (one set
// per thread at the levels |S| <= kLaneMaxK, one per tile above them): the
// dual route's, and the mpLP instances whose parameter set is a box (their
// multiplier law is -Psi(theta); the sets it leaves go to FP64, which also
// decides the mpLP's stationarity rows)
__host__ __device__ __forceinline__ bool lanes_route(int mode, const InstDesc &I, const SlotDims &sd)
{
    return I.lp ? (mode == 0 && I.box && I.p <= kDualMaxP) : dual_route(mode, I, sd);
}

// mpLP in the FP32 screen: Lam holds Gamma = (A_S A_S^T)^-1 [F_S | b_S] after
// kkt_factor<float>; the multiplier law Psi = (A_S A_S^T)^-1 [A_S H | A_S c]
// (FP32 copies of A H, A c) from the same factor, reciprocal pivots on R's
// diagonal, in place per column (lane per column).  Out of line, so that the
// mpQP sets' path keeps its registers.
__device__ __noinline__ void mplp_multipliers_f(const float *WhL, const float *wcL, int p, int k, OptWs<float> &ws)
{
    const int P1 = p + 1;
    for (int cc = lane_id(); cc < P1; cc += 32) {
        for (int a = 0; a < k; a++) {
            float acc = cc < p ? WhL[(size_t)ws.S[a] * p + cc] : wcL[ws.S[a]];
            for (int l = 0; l < a; l++) acc = __fmaf_rn(-ws.R[l * k + a], ws.Psi[l * P1 + cc], acc);
            ws.Psi[a * P1 + cc] = acc * ws.R[a * k + a];
        }
        for (int a = k - 1; a >= 0; a--) {
            float acc = ws.Psi[a * P1 + cc];
            for (int l = a + 1; l < k; l++) acc = __fmaf_rn(-ws.R[a * k + l], ws.Psi[l * P1 + cc], acc);
            ws.Psi[a * P1 + cc] = acc * ws.R[a * k + a];
        }
    }
    __syncwarp();
}

// mpLP sets with |S| = n over a box also take the dual route's second stage:
// their LP2 rows are the mpQP ones with Gamma for Lambda in the inactive rows
// and multiplier rows from Psi
__host__ __device__ __forceinline__ bool rows_route_lp(int mode, const InstDesc &I, const SlotDims &sd, int k)
{
    return I.lp && k == I.n && mode == 0 && I.box && I.p <= kDualMaxP && I.m + I.ncp <= kDualMaxRows &&
           sd.maxLD2 >= kDualLd;
}

// The FP32 data of the multiplier law: Wm and the right-hand sides [Wh | wc]
// (mpQP: Lambda), or for an mpLP [A H | A c] (Psi = (A_S A_S^T)^-1 [A_S H |
// A_S c], its multipliers -Psi)
__device__ __forceinline__ KktData<float> multiplier_data(const DevBuffers &B, const InstDesc &I)
{
    KktData<float> D = kkt_data<float>(B, I);
    if (I.lp) { D.Wh = B.fpool + I.f_WhL; D.wc = B.fpool + I.f_wcL; }
    return D;
}

// ---------------------------------------------------------------------
// Screen stage 0 on tiles of a warp
// ---------------------------------------------------------------------
// Stage 0 of the dual route works on small LPs -- the k multiplier rows and
// the 2p box rows (k + 2p <= 44), a basis of p + 1 <= 7 -- so a full warp
// left half of its lanes idle.  Here each W-thread tile of a warp screens its
// own set (32 / W per warp; W = 8, 16 or 32 is a plan setting the autotuner
// picks -- on the m = 62 batch 8 was fastest, 111 against 124 ms for 16):
// the same operations as kkt_factor<float> and lp2_dual_screen, with
// tile-wide shuffles and reductions.  W >= p + 1 (the basis rows sit in
// lanes 0..p).
namespace cgx = cooperative_groups;

// A slot of a device queue for each thread that calls this together with
// others: one atomic per group of threads that arrive converged.
__device__ __forceinline__ long long queue_slot(long long *counter)
{
    const cgx::coalesced_group g = cgx::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd((unsigned long long *)counter, (unsigned long long)g.size());
    base = g.shfl(base, 0);
    return (long long)base + g.thread_rank();
}
constexpr int kTileRows = 48;                  // k + 2p rows, ceil(48 / W) slots per lane
template <int W>
using ScreenTile = cgx::thread_block_tile<W, cgx::thread_block>;

template <int W>
__device__ __forceinline__ int tile_argmin(const ScreenTile<W> &t, unsigned key, unsigned id, int idx)
{
    const unsigned kmin = cgx::reduce(t, key, cgx::less<unsigned>());
    if (kmin == 0xffffffffu) return -1;
    const bool m = key == kmin;
    const unsigned idm = cgx::reduce(t, m ? id : 0xffffffffu, cgx::less<unsigned>());
    const unsigned win = t.ballot(m && id == idm);
    return t.shfl(idx, __ffs(win) - 1);
}

template <int W>
__device__ __forceinline__ float tile_max(const ScreenTile<W> &t, float v)
{
#pragma unroll
    for (int off = W / 2; off; off >>= 1) v = fmaxf(v, t.shfl_xor(v, off));
    return v;
}

template <int W>
__device__ __forceinline__ float tile_sum(const ScreenTile<W> &t, float v)
{
#pragma unroll
    for (int off = W / 2; off; off >>= 1) v += t.shfl_xor(v, off);
    return v;
}

// Stage-0 slot of one tile: R (maxK^2), Y and Lambda (maxK x P1), S, the
// dual-layout rows (k + 2p, and 2n more for an mpLP, of kDualLd floats)
__host__ __device__ inline int tile_rows(const SlotDims &sd)
{
    // an mpLP set with |S| < n adds 2n stationarity residual rows
    const int r = sd.maxK + 2 * kDualMaxP + 2 * sd.maxN;
    return r < kTileRows ? r : kTileRows;
}
__host__ __device__ inline size_t tile_slot_bytes(const SlotDims &sd)
{
    return align16((size_t)sd.maxK * sd.maxK * 4) + 2 * align16((size_t)sd.maxK * sd.maxP1 * 4) +
           align16((size_t)sd.maxK * sizeof(int)) + align16((size_t)tile_rows(sd) * kDualLd * 4);
}

// kkt_factor<float> with the lanes of a tile (the same operations in the same
// order; R keeps the reciprocal pivot on its diagonal).  Returns 0, or 1 when
// a pivot ratio fails thr.
template <int W>
__device__ int kkt_factor_tile(const ScreenTile<W> &t, const KktData<float> &D, const InstDesc &I, uint64_t lo,
                               uint64_t hi, float thr, float *R, float *Y, float *Lam, int *S, int *k_out,
                               float *rho_out)
{
    const int tl = t.thread_rank();
    const int m = I.m, p = I.p, P1 = p + 1;
    const int k = mask_pop(lo, hi);
    *k_out = k;
    for (int i = tl; i < m; i += W)
        if (mask_has(lo, hi, i)) S[mask_rank(lo, hi, i)] = i;
    t.sync();
    float rho = 1.0f;
    for (int a = 0; a < k; a++) {
        int fail = 0;
        if (tl == 0) {
            const float d0 = D.Wm[(size_t)S[a] * m + S[a]];
            float acc = d0;
            for (int l = 0; l < a; l++) acc = __fmaf_rn(-R[l * k + a], R[l * k + a], acc);
            if (!(acc > thr * d0)) fail = 1;
            else {
                R[a * k + a] = __frcp_rn(__fsqrt_rn(acc));
                const float rr = __fdividef(acc, d0);
                if (rr < rho) rho = rr;
            }
        }
        fail = t.shfl(fail, 0);
        if (fail) return 1;
        t.sync();
        for (int b = a + 1 + tl; b < k; b += W) {
            float acc = D.Wm[(size_t)S[a] * m + S[b]];
            for (int l = 0; l < a; l++) acc = __fmaf_rn(-R[l * k + a], R[l * k + b], acc);
            R[a * k + b] = acc * R[a * k + a];
        }
        t.sync();
    }
    for (int cc = tl; cc < P1; cc += W) {
        for (int a = 0; a < k; a++) {
            float acc = (cc < p) ? D.Wh[(size_t)S[a] * p + cc] : D.wc[S[a]];
            for (int l = 0; l < a; l++) acc = __fmaf_rn(-R[l * k + a], Y[l * P1 + cc], acc);
            Y[a * P1 + cc] = acc * R[a * k + a];
        }
        for (int a = k - 1; a >= 0; a--) {
            float acc = Y[a * P1 + cc];
            for (int l = a + 1; l < k; l++) acc = __fmaf_rn(-R[a * k + l], Lam[l * P1 + cc], acc);
            Lam[a * P1 + cc] = acc * R[a * k + a];
        }
    }
    t.sync();
    *rho_out = t.shfl(rho, 0);
    return 0;
}

// lp2_dual_screen with the lanes of a tile: rows r = lane + W s, basis rows
// in lanes 0..p.  Same pricing, ratio test, pivot and verified bound.
// WARM: the LP may start from the final basis of the parent set's LP
// (`warm`, p + 1 row numbers of the parent's layout, 0xff = none), the
// reference's basis sharing between sets at Hamming distance one
// (batched_simplex.cu:525-590).  The set S u {j} has j above every element
// of S, so the parent's multiplier rows keep their numbers and its box rows
// move down one.  The basis matrix is inverted in the tile (Gauss-Jordan with
// partial pivoting); a singular or primal-infeasible basis falls back to the
// single-row start, as the reference resets to its initial basis.  *warm_out:
// 0 no basis offered, 1 offered and rejected, 2 started from it; *basis_out:
// this LP's final basis (8 bytes, 0xff past p + 1).
constexpr float kWarmPivMin = 1e-7f;

template <int W, bool WARM = false>
__device__ int lp2_dual_screen_tile(const ScreenTile<W> &t, const float *T, int m, int R2, int p, const float *blo,
                                    const float *bhi, float thr, float ethr, float tol_piv, float tol_dj, int max_it,
                                    int degen_switch, int *it_out, float *bound_out, const uint8_t *warm = nullptr,
                                    unsigned long long *basis_out = nullptr, int *warm_out = nullptr)
{
    constexpr int NR = (kTileRows + W - 1) / W;
    constexpr int MP = kDualMaxP;
    constexpr int LD = kDualLd;
    const int lane = t.thread_rank();
    const int P1 = p + 1;
    auto row8 = [&](int r, float *a) {
        const float4 v0 = reinterpret_cast<const float4 *>(T + r * LD)[0];
        const float4 v1 = reinterpret_cast<const float4 *>(T + r * LD)[1];
        a[0] = v0.x; a[1] = v0.y; a[2] = v0.z; a[3] = v0.w; a[4] = v1.x; a[5] = v1.y; a[6] = v1.z; a[7] = v1.w;
    };
    float lo[MP], hi[MP];
#pragma unroll
    for (int c = 0; c < MP; c++) { lo[c] = c < p ? blo[c] : 0.0f; hi[c] = c < p ? bhi[c] : 0.0f; }
    float binv[MP], pi[MP], binvp = 0.0f, y = 0.0f, pip = 0.0f;
    int bidx = -1;
    unsigned basic = 0;
    bool warm_ok = false;
    if constexpr (WARM) {
        int wb = -1;
        if (warm && lane < P1) {
            const int r = warm[lane];
            wb = r == 0xff ? -1 : (r < m - 1 ? r : r + 1);
        }
        bool ok = t.all(lane >= P1 || (wb >= 0 && wb < R2));
        if (warm_out) *warm_out = warm ? (ok ? 1 : 0) : 0;
        if (warm && ok) {
            // lane e < P1: equation e of [B | I] (e < p: the g column e of the
            // basic rows, e = p: their c column)
            const int col = lane < p ? lane : 6;
            float Bv[MP + 1], Iv[MP + 1];
#pragma unroll
            for (int i = 0; i <= MP; i++) {
                const int bi = t.shfl(wb, i < P1 ? i : 0);
                Bv[i] = (i < P1 && lane < P1) ? T[bi * LD + col] : 0.0f;
                Iv[i] = i == lane ? 1.0f : 0.0f;
            }
            bool used = lane >= P1;
            int src = 0;
#pragma unroll
            for (int i = 0; i <= MP; i++) {
                if (i < P1 && ok) {
                    const unsigned key = used ? 0xffffffffu : ~__float_as_uint(fabsf(Bv[i]));
                    const int pl = tile_argmin<W>(t, key, (unsigned)lane, lane);   // -1: column i all zero
                    const float pv = t.shfl(Bv[i], pl < 0 ? 0 : pl);
                    if (pl < 0 || !(fabsf(pv) > kWarmPivMin)) ok = false;
                    else {
                        const float inv = __fdividef(1.0f, pv);
                        const float f = lane == pl ? 0.0f : Bv[i] * inv;
#pragma unroll
                        for (int c = 0; c <= MP; c++) {
                            const float rb = t.shfl(Bv[c], pl), ri = t.shfl(Iv[c], pl);
                            Bv[c] = lane == pl ? rb * inv : __fmaf_rn(-f, rb, Bv[c]);
                            Iv[c] = lane == pl ? ri * inv : __fmaf_rn(-f, ri, Iv[c]);
                        }
                        if (lane == pl) used = true;
                        if (lane == i) src = pl;
                    }
                }
            }
            if (ok) {
                // lane i: row i of B^-1 (the row of the lane that pivoted column i)
#pragma unroll
                for (int c = 0; c < MP; c++) {
                    const float v = t.shfl(Iv[c], src);
                    binv[c] = (lane < P1 && c < p) ? v : 0.0f;
                }
                float vp = 0.0f;
#pragma unroll
                for (int c = 0; c <= MP; c++) { const float v = t.shfl(Iv[c], src); if (c == p) vp = v; }
                binvp = lane < P1 ? vp : 0.0f;
                y = binvp;
                ok = t.all(lane >= P1 || y >= 0.0f);
            }
            if (ok) {
                bidx = lane < P1 ? wb : -1;
                const float hb = lane < P1 ? T[wb * LD + 7] : 0.0f;
#pragma unroll
                for (int c = 0; c < MP; c++) pi[c] = tile_sum<W>(t, hb * binv[c]);
                pip = tile_sum<W>(t, hb * binvp);
#pragma unroll
                for (int i = 0; i <= MP; i++) {
                    const int bi = t.shfl(wb, i < P1 ? i : 0);
                    if (i < P1 && lane == (bi & (W - 1))) basic |= 1u << (bi / W);
                }
                warm_ok = true;
                if (warm_out) *warm_out = 2;
            } else {
                binvp = 0.0f; y = 0.0f;
#pragma unroll
                for (int c = 0; c < MP; c++) binv[c] = 0.0f;
            }
        }
    }
    if (!warm_ok) {
    unsigned bkey = 0xffffffffu;
    int bi = -1;
    for (int r = lane; r < m; r += W) {
        float a[8];
        row8(r, a);
        float b = a[7];
#pragma unroll
        for (int c = 0; c < MP; c++) b -= a[c] > 0.0f ? a[c] * lo[c] : a[c] * hi[c];
        const unsigned k = key_signed(b);
        if (bi < 0 || k < bkey) { bkey = k; bi = r; }
    }
    const int istar = tile_argmin<W>(t, bkey, (unsigned)bi, bi);
    float gi[8];
    row8(istar, gi);
    pip = gi[7];
#pragma unroll
    for (int c = 0; c < MP; c++) {
        binv[c] = 0.0f;
        pi[c] = 0.0f;
        if (c < p) {
            const bool upper = !(gi[c] > 0.0f);
            const int row = m + (upper ? c : p + c);
            const float sc = T[row * LD + c];
            pi[c] = upper ? hi[c] : lo[c];
            const float yc = __fdividef(-gi[c], sc);
            pip = __fmaf_rn(yc, T[row * LD + 7], pip);
            if (lane == 1 + c) { bidx = row; y = yc; binv[c] = __fdividef(1.0f, sc); binvp = yc; }
        }
    }
    if (lane == 0) { bidx = istar; y = 1.0f; binvp = 1.0f; }
#pragma unroll 1
    for (int s = 0; s < NR; s++) {
        const int r = lane + W * s;
        bool b = r == istar;
        if (r >= m && r < m + p) b = !(T[istar * LD + (r - m)] > 0.0f);
        else if (r >= m + p && r < m + 2 * p) b = T[istar * LD + (r - m - p)] > 0.0f;
        if (b) basic |= 1u << s;
    }
    }
    float reach = 0.0f;
#pragma unroll
    for (int c = 0; c < MP; c++) if (lane == c) reach = fmaxf(fabsf(lo[c]), fabsf(hi[c]));
    const int vcol = lane < p ? lane : (lane == p ? 6 : 7);
    float thr_row = thr;   // the per-row threshold of the last verified y
    auto verify = [&]() -> float {
        float acc = 0.0f, ey = 0.0f;
#pragma unroll
        for (int i = 0; i <= MP; i++) {
            if (i < P1) {
                const float yi = t.shfl(fmaxf(y, 0.0f), i);
                const int ri = t.shfl(bidx, i);
                if (lane <= P1) acc = __fmaf_rn(yi, T[ri * LD + vcol], acc);
                ey = __fmaf_rn(yi, T[ri * LD + kRowScaleCol], ey);
            }
        }
        const float cy = t.shfl(acc, p);
        const float num = tile_sum<W>(t, lane < p ? fabsf(acc) * reach : (lane == P1 ? acc : 0.0f));
        thr_row = cy > 0.0f ? fminf(thr, ethr * __fdividef(ey, cy)) : thr;
        return cy > 0.0f ? __fdividef(num, cy) : pos_inf<float>();
    };
    int it = 0, degen = 0, proven = 0;
    bool bland = false;
    float bound = pos_inf<float>();
    for (;;) {
        if (pip < -thr) {
            bound = verify();
            if (bound < -thr_row) { proven = 1; break; }
        }
        if (it >= max_it) break;
        unsigned key = 0xffffffffu, kid = 0xffffffffu;
        int kq = -1;
        float dbest = 0.0f;
#pragma unroll 1
        for (int s = 0; s < NR; s++) {
            const int r = lane + W * s;
            if (r < R2 && !((basic >> s) & 1u)) {
                float a[8];
                row8(r, a);
                float d = __fmaf_rn(-pip, a[6], a[7]);
#pragma unroll
                for (int c = 0; c < MP; c++) d = __fmaf_rn(-pi[c], a[c], d);
                if (d < -tol_dj) {
                    const unsigned k = bland ? 0u : ~key_of(-d);
                    if (kq < 0 || k < key || (k == key && (unsigned)r < kid)) { key = k; kid = r; kq = r; dbest = d; }
                }
            }
        }
        const int q = tile_argmin<W>(t, key, kid, kq);
        if (q < 0) {
            bound = verify();
            proven = bound < -thr_row;
            break;
        }
        const float dq = t.shfl(dbest, q & (W - 1));
        float aq[8];
        row8(q, aq);
        float u = binvp * aq[6];
#pragma unroll
        for (int c = 0; c < MP; c++) u = __fmaf_rn(binv[c], aq[c], u);
        unsigned rk = 0xffffffffu, rid = 0xffffffffu;
        int rl = -1;
        if (lane < P1 && u > tol_piv) { rk = key_of(__fdividef(fmaxf(y, 0.0f), u)); rid = (unsigned)bidx; rl = lane; }
        const int l = tile_argmin<W>(t, rk, rid, rl);
        if (l < 0) break;
        const float ul = t.shfl(u, l);
        const float yl = t.shfl(fmaxf(y, 0.0f), l);
        const int oldb = t.shfl(bidx, l);
        const float inv = __fdividef(1.0f, ul);
        const float theta = yl * inv;
        const float f = u * inv, fp = dq * inv;
        const bool own = lane == l, other = lane < P1 && lane != l;
#pragma unroll
        for (int c = 0; c < MP; c++) {
            const float rj = t.shfl(binv[c], l);
            binv[c] = own ? rj * inv : (other ? __fmaf_rn(-f, rj, binv[c]) : binv[c]);
            pi[c] = __fmaf_rn(fp, rj, pi[c]);
        }
        {
            const float rj = t.shfl(binvp, l);
            binvp = own ? rj * inv : (other ? __fmaf_rn(-f, rj, binvp) : binvp);
            pip = __fmaf_rn(fp, rj, pip);
        }
        if (own) { y = theta; bidx = q; }
        else if (other) y = __fmaf_rn(-theta, u, y);
        if (lane == (q & (W - 1))) basic |= 1u << (q / W);
        if (lane == (oldb & (W - 1))) basic &= ~(1u << (oldb / W));
        it++;
        degen = (theta == 0.0f) ? degen + 1 : 0;
        bland = degen >= degen_switch;
    }
    *it_out = it;
    *bound_out = bound;
    if constexpr (WARM) {
        unsigned long long word = ~0ull;
#pragma unroll
        for (int i = 0; i <= MP; i++) {
            const int b = t.shfl(bidx, i);
            if (i < P1) word = (word & ~(0xffull << (8 * i))) | ((unsigned long long)(b & 0xff) << (8 * i));
        }
        if (basis_out) *basis_out = word;
    }
    return proven;
}

// The stationarity residual rows of an mpLP set with |S| = k < n, in the dual
// layout at T: the residual of x's stationarity (c + H theta) - A_S^T
// Psi(theta) = r0 + E theta must stay within tol_feas in every component
// (the reference's LP2 equalities, main.py:107-108), so the rows
//   (r0 + E theta)_i + t <= tol_feas,   -(r0 + E theta)_i + t <= tol_feas
// (2n rows, a t coefficient of 1) hold at t = 0 wherever the set can be
// optimal, and a verified bound below zero over them, the multiplier rows
// and the box proves "not optimal".  E_i = H_i - sum_l A_{S_l,i} Psi_l and
// r0_i = c_i - sum_l A_{S_l,i} Psi_l,p from the FP32 Psi in Lam; each row's
// error scale is sum_l |A_{S_l,i}| (the l-th multiplier row's magnitude) plus
// |H_i| + |c_i|.  Returns this lane's largest error scale.
template <int W>
__device__ float mplp_residual_rows(const ScreenTile<W> &t, const DevBuffers &B, const InstDesc &I, const int *S,
                                    const float *Lam, int k, float tol_feas, float *T)
{
    const int n = I.n, m = I.m, p = I.p, P1 = p + 1;
    const float *AT = B.fpool + I.f_AT, *Hm = B.fpool + I.f_Hm, *cv = B.fpool + I.f_cv;
    float amax = 0.0f;
    for (int i = t.thread_rank(); i < n; i += W) {
        float e[kDualMaxP];
        float r0 = cv[i], rs = fabsf(cv[i]);
#pragma unroll
        for (int c = 0; c < kDualMaxP; c++) {
            e[c] = c < p ? Hm[i * p + c] : 0.0f;
            rs += fabsf(e[c]);
        }
        for (int l = 0; l < k; l++) {
            const float a = AT[(size_t)i * m + S[l]];
            const float *lam = Lam + l * P1;
            float ls = fabsf(lam[p]);
#pragma unroll
            for (int c = 0; c < kDualMaxP; c++)
                if (c < p) { e[c] = __fmaf_rn(-a, lam[c], e[c]); ls += fabsf(lam[c]); }
            r0 = __fmaf_rn(-a, lam[p], r0);
            rs = __fmaf_rn(fabsf(a), ls, rs);
        }
        float *tp = T + (size_t)(2 * i) * kDualLd, *tn = tp + kDualLd;
#pragma unroll
        for (int c = 0; c < kDualMaxP; c++) { tp[c] = e[c]; tn[c] = -e[c]; }
        tp[6] = 1.0f; tn[6] = 1.0f;
        tp[7] = tol_feas - r0; tn[7] = tol_feas + r0;
        tp[kRowScaleCol] = rs; tn[kRowScaleCol] = rs;
        amax = fmaxf(amax, rs);
    }
    return amax;
}

// Stage 0 of the dual route, one set per tile (32 / W per warp): KKT factor,
// the multiplier rows and the box, dual bound; the sets it cannot settle go
// to stage 1 (k_opt_screen<0, 1>), a failed KKT margin to the FP64 queue.
// An mpLP set with |S| < n also takes its stationarity residual rows into
// the LP (mplp_residual_rows), so that a set whose residual cannot vanish
// inside the box is settled here.
// WARM: the dual LP starts from the parent set's final basis when that basis
// is valid for this set (B.lp2b; the parent of node x is candidate x's).
// src 0: every node of the level; src 1: the mpLP sets with |S| < n that the
// one-set-per-thread stage left (its queue in q_lp1, shared with stage 1,
// which takes only the mpQP sets), their LPs counted as pivots only.
template <int W, bool WARM = false>
__global__ void __launch_bounds__(32, 24) k_opt_screen_tiles(DevBuffers B, Tol tol, SlotDims sd, int level, int mode,
                                                                         int src)
{
    static_assert(W >= kDualMaxP + 1 && W <= 32 && (W & (W - 1)) == 0, "tile width");
    extern __shared__ __align__(16) unsigned char smem[];
    const ScreenTile<W> t = cgx::tiled_partition<W>(cgx::this_thread_block());
    const int lane = t.thread_rank();
    float *R, *Y, *Lam, *Tb;
    int *S;
    {
        unsigned char *base = smem + (threadIdx.x / W) * tile_slot_bytes(sd);
        size_t o = 0;
        R = (float *)(base + o); o += align16((size_t)sd.maxK * sd.maxK * 4);
        Y = (float *)(base + o); o += align16((size_t)sd.maxK * sd.maxP1 * 4);
        Lam = (float *)(base + o); o += align16((size_t)sd.maxK * sd.maxP1 * 4);
        S = (int *)(base + o); o += align16((size_t)sd.maxK * sizeof(int));
        Tb = (float *)(base + o);
    }
    const int side = level & 1;
    Ctl *ctl = B.ctl;
    const long long nn = src == 0 ? (ctl->n_node[side] < B.node_cap ? ctl->n_node[side] : B.node_cap)
                                  : (ctl->n_q_scr < B.q_cap ? ctl->n_q_scr : B.q_cap);
    LocalInstCounters lc;
    lc.reset(-1);
    auto flush = [&]() {
        if (lc.inst >= 0 && lane == 0) {
            atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp2_piv, (unsigned long long)lc.c);
            if (src == 0) {
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].s0_lps, (unsigned long long)lc.d);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].s0_piv, (unsigned long long)lc.c);
            }
            if (WARM) {
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].warm_try, (unsigned long long)lc.f);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].warm_used, (unsigned long long)lc.g);
            }
        }
    };
    for (;;) {
        long long x;
        if (lane == 0) x = (long long)atomicAdd(&ctl->ctr[src == 0 ? 3 : 10], 1ull);
        x = t.shfl(x, 0);
        if (x >= nn) break;
        if (src != 0) x = B.q_lp1[x];
        if (WARM && src == 0 && lane == 0) B.lp2b[side][x] = ~0ull;   // no basis unless this set's LP runs
        const Node nd = B.node[side][x];
        if ((nd.flags & (NODE_VALID | NODE_FEASIBLE)) != (NODE_VALID | NODE_FEASIBLE)) continue;
        const InstDesc &I = B.inst[nd.inst];
        if (level < I.k_min) continue;
        if (!lanes_route(mode, I, sd) || (src != 0 && (!I.lp || level >= I.n))) continue;
        if (nd.inst != lc.inst) { flush(); lc.reset(nd.inst); }
        const KktData<float> D = multiplier_data(B, I);
        const int p = I.p, ncp = I.ncp, P1 = p + 1;
        int k = 0, piv = 0, nres = 0;
        float rho = 1.0f, bound = 0.0f;
        bool proven = false, to_rows = false;
        if (!kkt_factor_tile<W>(t, D, I, nd.lo, nd.hi, tol.margin_licq32, R, Y, Lam, S, &k, &rho)) {
            to_rows = true;
            if (k > 0 && k + ncp <= tile_rows(sd)) {
                float bmax = 0.0f;
                for (int ii = lane; ii < ncp; ii += W) bmax = fmaxf(bmax, fabsf(D.bt[ii]));
                bmax = tile_max<W>(t, bmax);
                float amaxA = 0.0f;
                for (int a = lane; a < k; a += W) {
                    float *tr = Tb + (size_t)a * kDualLd;
                    const float *lam = Lam + a * P1;
                    float rs = 0.0f;
                    for (int cc = 0; cc < p; cc++) { tr[cc] = lam[cc]; rs += fabsf(lam[cc]); }
                    for (int cc = p; cc < kDualMaxP; cc++) tr[cc] = 0.0f;
                    tr[6] = 1.0f;
                    tr[7] = -lam[p];
                    rs += fabsf(lam[p]);
                    tr[kRowScaleCol] = rs;
                    amaxA = fmaxf(amaxA, rs);
                }
                for (int ii = lane; ii < ncp; ii += W) {
                    float *tr = Tb + (size_t)(k + ii) * kDualLd;
                    for (int cc = 0; cc < kDualMaxP; cc++) tr[cc] = cc < p ? D.At[ii * p + cc] : 0.0f;
                    tr[6] = 0.0f;
                    tr[7] = D.bt[ii];
                    tr[kRowScaleCol] = 0.0f;
                }
                if (I.lp && k < I.n && k + ncp + 2 * I.n <= tile_rows(sd)) {
                    amaxA = fmaxf(amaxA, mplp_residual_rows<W>(t, B, I, S, Lam, k, (float)tol.tol_feas,
                                                               Tb + (size_t)(k + ncp) * kDualLd));
                    nres = 2 * I.n;
                }
                amaxA = tile_max<W>(t, amaxA);
                // error scale per unit of row magnitude: 1 / smallest pivot ratio
                // times the reach of theta inside the box
                const float escale = __fdividef(1.0f + (float)p * bmax, rho);
                t.sync();
                const uint8_t *warm = nullptr;
                if (WARM && src == 0 && level >= 1) {
                    const int par = B.cand[x].parent;
                    if (par >= 0) warm = reinterpret_cast<const uint8_t *>(B.lp2b[side ^ 1] + par);
                }
                unsigned long long bword = ~0ull;
                int wst = 0;
                proven = lp2_dual_screen_tile<W, WARM>(t, Tb, k, k + ncp + nres, p, B.fpool + I.f_blo,
                                                    B.fpool + I.f_bhi, tol.margin_t32 * escale * amaxA,
                                                    tol.margin_t32 * escale, tol.tol_piv32, tol.tol_dj32,
                                                    tol.max_pivots, tol.degen_switch, &piv, &bound, warm, &bword,
                                                    &wst);
                to_rows = !proven;
                lc.d++;
                if (WARM && src == 0) {
                    if (lane == 0) B.lp2b[side][x] = bword;
                    lc.f += wst >= 1;
                    lc.g += wst == 2;
                }
                t.sync();
            }
        }
        lc.c += piv;
        if (!proven) {
            // stage 1 takes the sets with a KKT factor (of an mpLP only those with
            // |S| = n); a failed KKT margin, and every other mpLP set, goes to FP64
            if (lane == 0) {
                if (to_rows && (!I.lp || (src == 0 && rows_route_lp(mode, I, sd, k)))) {
                    const long long qi = (long long)atomicAdd((unsigned long long *)&ctl->n_q_scr, 1ull);
                    if (qi < B.q_cap) B.q_lp1[qi] = (int)x; else atomicOr(&ctl->overflow, OV_QUEUE);
                } else {
                    const long long qi = (long long)atomicAdd((unsigned long long *)&ctl->n_q_opt, 1ull);
                    if (qi < B.q_cap) B.q_opt[qi] = (int)x; else atomicOr(&ctl->overflow, OV_QUEUE);
                }
            }
            t.sync();
            continue;
        }
        // a final "not optimal" only leaves a diagnostic record
        if (lane == 0 && nd.rec >= 0 && B.rec) {
            OptResult res;
            res.licq = 1; res.lp2_status = LP_BOUND; res.lp2_piv = piv;
            res.cheb_status = LP_SKIPPED; res.cheb_piv = 0; res.optimal = 0; res.region = 0;
            res.t = (double)bound; res.r = __longlong_as_double(0x7ff8000000000000LL);
            res.decided = true;
            write_opt(B, nd, level, res, false);
        }
        t.sync();
    }
    flush();
}

// Stage 0 of the dual route with one set per thread, for the levels with
// |S| <= kLaneMaxK: the operations of k_opt_screen_tiles -- the KKT factor
// with its LICQ margin, the multiplier rows and the box, lp2_dual_screen from
// the best single-row start, the bound verified from max(y, 0) -- run
// serially by one thread per set, 32 consecutive sets per warp.  A tile of 8
// lanes spends most of its instructions on shuffles, syncs and lanes left
// idle by k, p + 1 <= 7; here every lane works on its own set.  Each thread
// keeps its arrays in its own column of the warp's shared memory (element e
// at e * 32 + lane: no bank conflicts, whatever the threads' positions).
// The only differences from the tile: the R stride (kLaneMaxK) and the order
// of one sum in the verified bound (a few ulps, inside its error margin).
constexpr int kLaneP1 = kDualMaxP + 1;
// words per thread: Lambda, B^-1 rows (p columns and the c column), y, the
// multiplier rows' error scales, S, the basic rows (R and Y live in registers)
constexpr int kLaneWords = kLaneMaxK * kLaneP1 + kLaneP1 * kDualMaxP + 3 * kLaneP1 + 2 * kLaneMaxK;

// pass 0 runs over the level's nodes, pass 1 over B.q_s0, pass 2 over B.q_s1.
// cap > 0: an LP still running after cap pivots stops, and its set goes to the
// next pass's queue (q_s0 after pass 0, q_s1 after pass 1); cap = 0: the LP
// runs to the end.  Each pass runs an LP again from the same start, so the
// result is that of one uncapped pass.  The 32 sets of a warp then mostly
// share a pivot count, instead of all waiting for the slowest (a fifth of the
// sets need 4 to 25 pivots).
__global__ void __launch_bounds__(32) k_opt_screen_lanes(DevBuffers B, Tol tol, SlotDims sd, int level, int mode,
                                                         int pass, int cap)
{
    extern __shared__ __align__(16) float lsm[];
    constexpr int KM = kLaneMaxK, P7 = kLaneP1, MP = kDualMaxP;
    const int lane = lane_id();
    float *Lm = lsm + lane;                // Lambda: [a][cc] at (a P7 + cc) 32
    float *Bi = Lm + KM * P7 * 32;         // B^-1 row i, column c < p: (i MP + c) 32
    float *Bp = Bi + P7 * MP * 32;         // B^-1 row i, the c column
    float *Yv = Bp + P7 * 32;              // y_i
    float *Sc = Yv + P7 * 32;              // error scale of multiplier row a
    int *Sx = (int *)(Sc + KM * 32);       // S[a]
    int *Bx = Sx + KM * 32;                // basic row of basic variable i
    const int side = level & 1;
    Ctl *ctl = B.ctl;
    const long long nn = pass == 0 ? (ctl->n_node[side] < B.node_cap ? ctl->n_node[side] : B.node_cap)
                       : pass == 1 ? (ctl->n_q_s0 < B.q_s0_cap ? ctl->n_q_s0 : B.q_s0_cap)
                                   : (ctl->n_q_s1 < B.q_s1_cap ? ctl->n_q_s1 : B.q_s1_cap);
    LocalInstCounters lc;
    lc.reset(-1);
    auto flush = [&]() {
        if (lc.inst >= 0) {
            atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp2_piv, (unsigned long long)lc.c);
            atomicAdd((unsigned long long *)&B.ictl[lc.inst].s0_lps, (unsigned long long)lc.d);
            atomicAdd((unsigned long long *)&B.ictl[lc.inst].s0_piv, (unsigned long long)lc.c);
        }
    };
    const int max_it = cap > 0 ? cap : tol.max_pivots;
    for (;;) {
        long long x0;
        if (lane == 0) x0 = (long long)atomicAdd(&ctl->ctr[pass == 0 ? 3 : (pass == 1 ? 9 : 11)], 32ull);
        x0 = __shfl_sync(FULLMASK, x0, 0);
        if (x0 >= nn) break;
        if (x0 + lane >= nn) continue;
        const long long x = pass == 0 ? x0 + lane : (long long)(pass == 1 ? B.q_s0 : B.q_s1)[x0 + lane];
        const Node nd = B.node[side][x];
        if ((nd.flags & (NODE_VALID | NODE_FEASIBLE)) != (NODE_VALID | NODE_FEASIBLE)) continue;
        const InstDesc &I = B.inst[nd.inst];
        if (level < I.k_min) continue;
        if (!lanes_route(mode, I, sd)) continue;
        if (nd.inst != lc.inst) { flush(); lc.reset(nd.inst); }
        const KktData<float> D = multiplier_data(B, I);
        const int m = I.m, p = I.p, ncp = I.ncp, P1 = p + 1;
        const float *WhX = D.Wh, *wcX = D.wc;
        int k = 0;
        {
            uint64_t lo = nd.lo, hi = nd.hi;
            while ((lo | hi) && k < KM) {
                int i;
                if (lo) { i = __ffsll((long long)lo) - 1; lo &= lo - 1; }
                else { i = 64 + __ffsll((long long)hi) - 1; hi &= hi - 1; }
                Sx[k * 32] = i;
                k++;
            }
            if (lo | hi) k = KM + 1;   // larger than this kernel takes: FP64 decides
        }
        // KKT factor (kkt_factor's operations in the same order, R keeping the
        // reciprocal pivots), unrolled over k <= KM so that R, Y and Lambda
        // stay in registers; Lambda then goes to shared memory for the LP,
        // which reads its rows by index
        float rho = 1.0f;
        bool fail = k > KM;
        const float thr = tol.margin_licq32;
        int Sr[KM];
        float Rr[KM][KM];
#pragma unroll
        for (int a = 0; a < KM; a++) {
            Sr[a] = a < k ? Sx[a * 32] : 0;
#pragma unroll
            for (int b = 0; b < KM; b++) Rr[a][b] = 0.0f;
        }
#pragma unroll
        for (int a = 0; a < KM; a++) {
            if (a < k && !fail) {
                const float d0 = D.Wm[(size_t)Sr[a] * m + Sr[a]];
                float acc = d0;
#pragma unroll
                for (int l = 0; l < a; l++) acc = __fmaf_rn(-Rr[l][a], Rr[l][a], acc);
                if (!(acc > thr * d0)) fail = true;
                else {
                    const float ra = __frcp_rn(__fsqrt_rn(acc));
                    Rr[a][a] = ra;
                    const float rr = __fdividef(acc, d0);
                    if (rr < rho) rho = rr;
#pragma unroll
                    for (int b = a + 1; b < KM; b++) {
                        if (b < k) {
                            float acc2 = D.Wm[(size_t)Sr[a] * m + Sr[b]];
#pragma unroll
                            for (int l = 0; l < a; l++) acc2 = __fmaf_rn(-Rr[l][a], Rr[l][b], acc2);
                            Rr[a][b] = acc2 * ra;
                        }
                    }
                }
            }
        }
        int piv = 0;
        bool proven = false, to_rows = !fail;
        if (!fail && k > 0) {
            float Lr[KM][P7];
#pragma unroll
            for (int cc = 0; cc < P7; cc++) {
#pragma unroll
                for (int a = 0; a < KM; a++) Lr[a][cc] = 0.0f;
                if (cc < P1) {
#pragma unroll
                    for (int a = 0; a < KM; a++) {
                        if (a < k) {
                            float acc = (cc < p) ? WhX[(size_t)Sr[a] * p + cc] : wcX[Sr[a]];
#pragma unroll
                            for (int l = 0; l < a; l++) acc = __fmaf_rn(-Rr[l][a], Lr[l][cc], acc);
                            Lr[a][cc] = acc * Rr[a][a];
                        }
                    }
#pragma unroll
                    for (int a = KM - 1; a >= 0; a--) {
                        if (a < k) {
                            float acc = Lr[a][cc];
#pragma unroll
                            for (int l = a + 1; l < KM; l++)
                                if (l < k) acc = __fmaf_rn(-Rr[a][l], Lr[l][cc], acc);
                            Lr[a][cc] = acc * Rr[a][a];
                        }
                    }
                }
            }
            // Lambda to shared memory; the multiplier rows' error scales, the box's reach
            float amaxA = 0.0f, bmax = 0.0f;
#pragma unroll
            for (int a = 0; a < KM; a++) {
                if (a < k) {
                    float rs = 0.0f, rl = 0.0f;
#pragma unroll
                    for (int cc = 0; cc < P7; cc++) {
                        if (cc < P1) Lm[(a * P7 + cc) * 32] = Lr[a][cc];
                        if (cc < p) rs += fabsf(Lr[a][cc]);
                        if (cc == p) rl = Lr[a][cc];
                    }
                    rs += fabsf(rl);
                    Sc[a * 32] = rs;
                    amaxA = fmaxf(amaxA, rs);
                }
            }
            for (int ii = 0; ii < ncp; ii++) bmax = fmaxf(bmax, fabsf(D.bt[ii]));
            const float escale = __fdividef(1.0f + (float)p * bmax, rho);
            const float thr_lp = tol.margin_t32 * escale * amaxA, ethr = tol.margin_t32 * escale;
            const float *blo = B.fpool + I.f_blo, *bhi = B.fpool + I.f_bhi;
            const int R2 = k + ncp;
            // row r of the dual layout: g (p columns), c, h
            auto row8 = [&](int r, float *a8) {
                if (r < k) {
#pragma unroll
                    for (int c = 0; c < MP; c++) a8[c] = c < p ? Lm[(r * P7 + c) * 32] : 0.0f;
                    a8[6] = 1.0f;
                    a8[7] = -Lm[(r * P7 + p) * 32];
                } else {
                    const int ii = r - k;
#pragma unroll
                    for (int c = 0; c < MP; c++) a8[c] = c < p ? D.At[ii * p + c] : 0.0f;
                    a8[6] = 0.0f;
                    a8[7] = D.bt[ii];
                }
            };
            // best single-row bound over the multiplier rows
            int istar = -1;
            unsigned bkey = 0xffffffffu;
            for (int r = 0; r < k; r++) {
                float a8[8];
                row8(r, a8);
                float b = a8[7];
#pragma unroll
                for (int c = 0; c < MP; c++) {
                    const float lc_ = c < p ? blo[c] : 0.0f, hc_ = c < p ? bhi[c] : 0.0f;
                    b -= a8[c] > 0.0f ? a8[c] * lc_ : a8[c] * hc_;
                }
                const unsigned kk = key_signed(b);
                if (istar < 0 || kk < bkey) { bkey = kk; istar = r; }
            }
            float gi[8];
            row8(istar, gi);
            float pi[MP];
            float pip = gi[7];
            unsigned basic = 1u << istar;
            for (int i = 0; i < P1; i++) {
                for (int c = 0; c < MP; c++) Bi[(i * MP + c) * 32] = 0.0f;
                Bp[i * 32] = 0.0f;
                Yv[i * 32] = 0.0f;
            }
#pragma unroll
            for (int c = 0; c < MP; c++) {
                pi[c] = 0.0f;
                if (c < p) {
                    const bool upper = !(gi[c] > 0.0f);
                    const int row = k + (upper ? c : p + c);
                    const float sc = D.At[(row - k) * p + c];
                    pi[c] = upper ? bhi[c] : blo[c];
                    const float yc = __fdividef(-gi[c], sc);
                    pip = __fmaf_rn(yc, D.bt[row - k], pip);
                    Bx[(1 + c) * 32] = row;
                    Yv[(1 + c) * 32] = yc;
                    Bi[((1 + c) * MP + c) * 32] = __fdividef(1.0f, sc);
                    Bp[(1 + c) * 32] = yc;
                    basic |= 1u << row;
                }
            }
            Bx[0] = istar;
            Yv[0] = 1.0f;
            Bp[0] = 1.0f;
            float thr_row = thr_lp;
            auto verify = [&]() -> float {
                float acc[MP + 2], ey = 0.0f;
#pragma unroll
                for (int v = 0; v < MP + 2; v++) acc[v] = 0.0f;
                for (int i = 0; i < P1; i++) {
                    const float yi = fmaxf(Yv[i * 32], 0.0f);
                    const int ri = Bx[i * 32];
                    float a8[8];
                    row8(ri, a8);
#pragma unroll
                    for (int v = 0; v < MP + 2; v++) {
                        // v < p: column v; v == p: c (6); v == p + 1: h (7)
                        if (v <= P1) acc[v] = __fmaf_rn(yi, v < p ? a8[v] : (v == p ? a8[6] : a8[7]), acc[v]);
                    }
                    ey = __fmaf_rn(yi, ri < k ? Sc[ri * 32] : 0.0f, ey);
                }
                float cy = 0.0f, num = 0.0f;
#pragma unroll
                for (int v = 0; v < MP + 2; v++) {
                    if (v < p) num += fabsf(acc[v]) * fmaxf(fabsf(blo[v]), fabsf(bhi[v]));
                    else if (v == p) cy = acc[v];
                    else if (v == P1) num += acc[v];
                }
                thr_row = cy > 0.0f ? fminf(thr_lp, ethr * __fdividef(ey, cy)) : thr_lp;
                return cy > 0.0f ? __fdividef(num, cy) : pos_inf<float>();
            };
            int it = 0, degen = 0;
            bool bland = false, capped = false;
            float bound = pos_inf<float>();
            for (;;) {
                if (pip < -thr_lp) {
                    bound = verify();
                    if (bound < -thr_row) { proven = true; break; }
                }
                if (it >= max_it) { capped = cap > 0; break; }
                // pricing: the most negative reduced cost, smallest row on ties
                int q = -1;
                unsigned key = 0xffffffffu;
                float dq = 0.0f;
                for (int r = 0; r < k; r++) {
                    if ((basic >> r) & 1u) continue;
                    float a8[8];
                    row8(r, a8);
                    float d = __fmaf_rn(-pip, a8[6], a8[7]);
#pragma unroll
                    for (int c = 0; c < MP; c++) d = __fmaf_rn(-pi[c], a8[c], d);
                    if (d < -tol.tol_dj32) {
                        const unsigned kk = bland ? 0u : ~key_of(-d);
                        if (q < 0 || kk < key) { key = kk; q = r; dq = d; }
                    }
                }
                // a box row has one nonzero g (column c) and c = 0: its reduced
                // cost h - pi_c g_c is the general sum's value (the other terms
                // add exact zeros)
                for (int ii = 0; ii < ncp; ii++) {
                    const int r = k + ii;
                    if ((basic >> r) & 1u) continue;
                    const int cb = ii < p ? ii : ii - p;
                    float pc = 0.0f;
#pragma unroll
                    for (int c = 0; c < MP; c++) if (c == cb) pc = pi[c];
                    const float d = __fmaf_rn(-pc, D.At[ii * p + cb], D.bt[ii]);
                    if (d < -tol.tol_dj32) {
                        const unsigned kk = bland ? 0u : ~key_of(-d);
                        if (q < 0 || kk < key) { key = kk; q = r; dq = d; }
                    }
                }
                if (q < 0) {
                    bound = verify();
                    proven = bound < -thr_row;
                    break;
                }
                float aq[8];
                row8(q, aq);
                // ratio test over the basic variables: smallest max(y, 0) / u, smallest row on ties
                float u[P7];
                int l = -1, lrow = 0x7fffffff;
                unsigned rk = 0xffffffffu;
#pragma unroll
                for (int i = 0; i < P7; i++) {
                    u[i] = 0.0f;
                    if (i < P1) {
                        float ui = Bp[i * 32] * aq[6];
#pragma unroll
                        for (int c = 0; c < MP; c++) ui = __fmaf_rn(Bi[(i * MP + c) * 32], aq[c], ui);
                        u[i] = ui;
                        if (ui > tol.tol_piv32) {
                            const unsigned kk = key_of(__fdividef(fmaxf(Yv[i * 32], 0.0f), ui));
                            const int bi = Bx[i * 32];
                            if (l < 0 || kk < rk || (kk == rk && bi < lrow)) { rk = kk; l = i; lrow = bi; }
                        }
                    }
                }
                if (l < 0) break;
                float ul = 0.0f;
#pragma unroll
                for (int i = 0; i < P7; i++) if (i == l) ul = u[i];
                const float yl = fmaxf(Yv[l * 32], 0.0f);
                const int oldb = Bx[l * 32];
                const float inv = __fdividef(1.0f, ul);
                const float theta = yl * inv;
                const float fp = dq * inv;
#pragma unroll
                for (int c = 0; c < MP; c++) {
                    const float rj = Bi[(l * MP + c) * 32];
#pragma unroll
                    for (int i = 0; i < P7; i++) {
                        if (i < P1) {
                            float &bic = Bi[(i * MP + c) * 32];
                            bic = i == l ? rj * inv : __fmaf_rn(-(u[i] * inv), rj, bic);
                        }
                    }
                    pi[c] = __fmaf_rn(fp, rj, pi[c]);
                }
                {
                    const float rj = Bp[l * 32];
#pragma unroll
                    for (int i = 0; i < P7; i++) {
                        if (i < P1) {
                            float &bp = Bp[i * 32];
                            bp = i == l ? rj * inv : __fmaf_rn(-(u[i] * inv), rj, bp);
                        }
                    }
                    pip = __fmaf_rn(fp, rj, pip);
                }
#pragma unroll
                for (int i = 0; i < P7; i++) {
                    if (i < P1) {
                        if (i == l) { Yv[i * 32] = theta; Bx[i * 32] = q; }
                        else Yv[i * 32] = __fmaf_rn(-theta, u[i], Yv[i * 32]);
                    }
                }
                basic |= 1u << q;
                basic &= ~(1u << oldb);
                it++;
                degen = (theta == 0.0f) ? degen + 1 : 0;
                bland = degen >= tol.degen_switch;
            }
            if (capped) {
                // the next pass runs this set again from the start (a full
                // queue sends it to the second stage)
                if (pass == 0) {
                    const long long qi = queue_slot(&ctl->n_q_s0);
                    if (qi < B.q_s0_cap) { B.q_s0[qi] = (int)x; continue; }
                } else {
                    const long long qi = queue_slot(&ctl->n_q_s1);
                    if (qi < B.q_s1_cap) { B.q_s1[qi] = (int)x; continue; }
                }
            }
            piv = it;
            to_rows = !proven;
            lc.d++;
            if (proven && nd.rec >= 0 && B.rec) {
                OptResult res;
                res.licq = 1; res.lp2_status = LP_BOUND; res.lp2_piv = piv;
                res.cheb_status = LP_SKIPPED; res.cheb_piv = 0; res.optimal = 0; res.region = 0;
                res.t = (double)bound; res.r = __longlong_as_double(0x7ff8000000000000LL);
                res.decided = true;
                write_opt(B, nd, level, res, false);
            }
        }
        lc.c += piv;
        if (!proven) {
            // stage 1 takes the sets with a KKT factor (of an mpLP those with |S|
            // = n), the tile stage with the stationarity rows the mpLP sets with
            // |S| < n; a failed KKT margin, and every other mpLP set, goes to FP64
            if (to_rows && (!I.lp || (k < I.n && k + ncp + 2 * I.n <= tile_rows(sd)) || rows_route_lp(mode, I, sd, k))) {
                const long long qi = queue_slot(&ctl->n_q_scr);
                if (qi < B.q_cap) B.q_lp1[qi] = (int)x; else atomicOr(&ctl->overflow, OV_QUEUE);
            } else {
                const long long qi = queue_slot(&ctl->n_q_opt);
                if (qi < B.q_cap) B.q_opt[qi] = (int)x; else atomicOr(&ctl->overflow, OV_QUEUE);
            }
        }
    }
    flush();
}

size_t screen_lanes_smem() { return (size_t)kLaneWords * 32 * sizeof(float); }

cudaError_t launch_opt_screen_lanes(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int mode,
                                    int grid, size_t smem, cudaStream_t s, int pass, int cap)
{
    k_opt_screen_lanes<<<grid, 32, smem, s>>>(B, tol, sd, level, mode, pass, cap);
    return cudaGetLastError();
}

// ROUTE 1: the primal route, every set of the level.  ROUTE 0 with STAGE 1:
// the dual route's second stage -- the sets its first stage
// (k_opt_screen_tiles) could not settle from the multiplier rows and the
// box, through all region rows.  Separate kernels, so that each instruction
// stream stays small (the one-kernel screen was bound by instruction fetch).
template <int ROUTE, int STAGE = 0>
__global__ void __launch_bounds__(32, 32) k_opt_screen(DevBuffers B, Tol tol, SlotDims sd, int level, int mode)
{
    static_assert((ROUTE == 0) == (STAGE >= 1), "the dual route's first stage is k_opt_screen_tiles");
    // STAGE 2: the second stage for the mpLP sets with |S| = n (multiplier
    // rows from Psi), its own instance so that the mpQP one keeps its registers
    constexpr bool LPR = STAGE == 2;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id();
    OptWs<float> ws;
    float *Tb;
    uint8_t *ids;
    {
        size_t o = 0;
        ws.R = (float *)(smem + o); o += align16((size_t)sd.maxK * sd.maxK * 4);
        ws.Y = (float *)(smem + o); o += align16((size_t)sd.maxK * sd.maxP1 * 4);
        ws.Lam = (float *)(smem + o); o += align16((size_t)sd.maxK * sd.maxP1 * 4);
        ws.S = (int *)(smem + o); o += align16((size_t)sd.maxK * sizeof(int));
        Tb = (float *)(smem + o); o += align16((size_t)(sd.maxR2 + 1) * sd.maxLD2 * 4);
        ids = smem + o; o += align16((size_t)sd.maxR2 + sd.maxP1);
        ws.G = ROUTE == 1 ? (float *)(smem + o) : nullptr;
        ws.Tb = nullptr; ws.ids = nullptr;
        ws.Psi = ws.Phi = nullptr;
        if (ROUTE == 0 && sd.maxN) ws.Psi = (float *)(smem + o);   // mpLP multiplier law (second stage)
    }
    const int side = level & 1;
    Ctl *ctl = B.ctl;
    const long long nn = STAGE == 0 ? (ctl->n_node[side] < B.node_cap ? ctl->n_node[side] : B.node_cap)
                                    : (ctl->n_q_scr < B.q_cap ? ctl->n_q_scr : B.q_cap);
    LocalInstCounters lc;
    lc.reset(-1);
    for (;;) {
        long long x;
        if (lane == 0) x = (long long)atomicAdd(&ctl->ctr[STAGE == 2 ? 12 : (STAGE == 1 ? 6 : (ROUTE == 0 ? 3 : 5))], 1ull);
        x = __shfl_sync(FULLMASK, x, 0);
        if (x >= nn) break;
        // stage 1 reads the queue of stage 0 (kept in q_lp1: the LP1 queue is
        // consumed before the screen runs)
        if (STAGE >= 1) x = B.q_lp1[x];
        const Node nd = B.node[side][x];
        if ((nd.flags & (NODE_VALID | NODE_FEASIBLE)) != (NODE_VALID | NODE_FEASIBLE)) continue;
        const InstDesc &I = B.inst[nd.inst];
        if (level < I.k_min) continue;
        if (LPR ? !rows_route_lp(mode, I, sd, level) : dual_route(mode, I, sd) != (ROUTE == 0)) continue;
        constexpr bool lp_rows = LPR;
        // mpLP sets the first stage of the dual screen takes (one set per
        // thread at |S| <= kLaneMaxK, tiles above or with basis sharing)
        if (ROUTE == 1 && I.lp && lanes_route(mode, I, sd)) continue;
        if (nd.inst != lc.inst) {
            if (lc.inst >= 0 && lane == 0) {
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].optimal, (unsigned long long)lc.a);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].region, (unsigned long long)lc.b);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp2_piv, (unsigned long long)lc.c);
                atomicAdd((unsigned long long *)&B.ictl[lc.inst].cheb_piv, (unsigned long long)lc.d);
            }
            lc.reset(nd.inst);
        }
        const KktData<float> D = kkt_data<float>(B, I);
        const int m = I.m, p = I.p, ncp = I.ncp, P1 = p + 1, R2 = m + ncp, ld2 = I.ld2;
        int k = 0;
        float rho = 1.0f;
        bool decided = false;
        int status = LP_SKIPPED, piv = 0;
        float t = 0.0f;
        unsigned long long dbasis = ~0ull;
        // mpLP instances (Q = 0) take the primal route and are not screened:
        // every set goes to FP64 (dual_route excludes them)
        if (!(ROUTE == 1 && I.lp) && !kkt_factor<float>(D, I, nd.lo, nd.hi, tol.margin_licq32, ws, &k, &rho)) {
            // LP2: max t  s.t.  g theta + t <= h (constraint rows), At theta <= bt
            // the dual screen (mode 0, a box, p <= 6, at most 96 rows; its layout
            // needs rows of kDualLd floats in the slot) or the primal tableau
            constexpr bool dual = ROUTE == 0;
            float bmax = 0.0f;
            for (int ii = lane; ii < ncp; ii += 32) { const float v = fabsf(D.bt[ii]); if (v > bmax) bmax = v; }
            bmax = warp_max(bmax);
            {
            float t0, g0;
            if constexpr (lp_rows) mplp_multipliers_f(B.fpool + I.f_WhL, B.fpool + I.f_wcL, p, k, ws);
            // dual: rows straight into the dual layout; primal: rows into G,
            // kept unpivoted for the bound that verifies the verdict
            const float amax = dual ? region_rows<float, true, LPR>(D, I, nd.lo, nd.hi, k, ws, Tb, kDualLd, 7, &t0, &g0)
                                    : region_rows<float, true>(D, I, nd.lo, nd.hi, k, ws, nullptr, 0, 0, &t0, &g0);
            // error scale of the FP32 rows: row magnitude / smallest Cholesky
            // pivot ratio, times the reach of theta inside the box (rho >
            // margin_licq, so the quotient is tame)
            const float scale = __fdividef(amax, rho) * (1.0f + (float)p * bmax);
            __syncwarp();
            if constexpr (dual) {
                // dual layout: g beyond p zero, column 6 c_r (h is in column 7)
                for (int r = lane; r < R2; r += 32) {
                    float *tr = Tb + (size_t)r * kDualLd;
                    for (int cc = p; cc < kDualMaxP; cc++) tr[cc] = 0.0f;
                    tr[6] = (r < m) ? 1.0f : 0.0f;
                }
                __syncwarp();
                float bound;
                int pivB = 0;
                decided = lp2_dual_screen(Tb, m, R2, p, B.fpool + I.f_blo, B.fpool + I.f_bhi, tol.margin_t32 * scale,
                                          tol.margin_t32 * __fdividef(1.0f + (float)p * bmax, rho), tol.tol_piv32,
                                          tol.tol_dj32, tol.max_pivots, tol.degen_switch, &pivB, &bound, &dbasis);
                piv += pivB;
                status = LP_BOUND;
                t = bound;
            } else {
                uint8_t *bid = ids, *nid = ids + R2;
                const float *G = ws.G;
                for (int r = lane; r < R2; r += 32) {
                    float *tr = Tb + (size_t)r * ld2;
                    const float *g = G + (size_t)r * P1;
                    for (int cc = 0; cc < p; cc++) tr[cc] = g[cc];
                    const float cf = (r < m) ? 1.0f : 0.0f;
                    float beta = __fmaf_rn(-cf, t0, g[p]);
                    if (!(beta > 0.0f)) beta = 0.0f;
                    tr[p] = cf;
                    tr[P1] = beta;
                    bid[r] = (uint8_t)(P1 + r);
                }
                for (int cc = lane; cc <= P1; cc += 32) {
                    float *ob = Tb + (size_t)R2 * ld2;
                    ob[cc] = (cc == p) ? 1.0f : (cc == P1 ? -t0 : 0.0f);
                    if (cc < P1) nid[cc] = (uint8_t)cc;
                }
                __syncwarp();
                Lp<float> L{Tb, ld2, R2, P1, P1, bid, nid};
                status = warp_simplex_f32<2>(L, tol.tol_piv32, tol.tol_dj32, tol.max_pivots, tol.degen_switch, &piv);
                t = -Tb[(size_t)R2 * ld2 + P1];
                // The FP32 primal optimum t is only a lower bound on t* when the
                // FP32 basis is not truly optimal (degenerate, badly
                // conditioned LPs), so it never decides alone: the duals y of
                // the final tableau (y_r = -reduced cost of slack r, 0 when
                // basic) give the upper bound (h.y + sum_c |(G^T y)_c| reach_c)
                // / (c.y) of lp2_dual_screen, evaluated on the unpivoted rows;
                // it needs a box (reach), so other parameter sets go to FP64.
                if (status == LP_OPTIMAL && t < -tol.margin_t32 * scale && I.box) {
                    const float *ob = Tb + (size_t)R2 * ld2;
                    int ry = -1;
                    float yv = 0.0f;
                    if (lane < P1 && nid[lane] >= P1) { ry = nid[lane] - P1; yv = fmaxf(-ob[lane], 0.0f); }
                    // lane c < p: (G^T y)_c, lane p: c.y, lane p+1: h.y
                    float acc = 0.0f;
                    for (int i = 0; i < P1; i++) {
                        const int ri = __shfl_sync(FULLMASK, ry, i);
                        const float yi = __shfl_sync(FULLMASK, yv, i);
                        if (ri >= 0 && lane <= P1) {
                            const float v = lane < p ? G[(size_t)ri * P1 + lane]
                                                     : (lane == p ? (ri < m ? 1.0f : 0.0f) : G[(size_t)ri * P1 + p]);
                            acc = __fmaf_rn(yi, v, acc);
                        }
                    }
                    float reach = 0.0f;
                    if (lane < p) {
                        const float lo_c = B.fpool[I.f_blo + lane], hi_c = B.fpool[I.f_bhi + lane];
                        reach = fmaxf(fabsf(lo_c), fabsf(hi_c));
                    }
                    const float cy = __shfl_sync(FULLMASK, acc, p);
                    const float num = warp_sum(lane < p ? fabsf(acc) * reach : (lane == P1 ? acc : 0.0f));
                    const float bound = cy > 0.0f ? __fdividef(num, cy) : pos_inf<float>();
                    decided = bound < -tol.margin_t32 * scale;
                    t = bound;
                }
            }
            }
        }
        lc.c += piv;
        if (!decided) {
            if (lane == 0) {
                // a negative FP32 dual bound that the margin did not accept: the
                // FP64 kernel checks its basis first (lp2_cert64)
                bool queued = false;
                if (ROUTE == 0 && status == LP_BOUND && t < 0.0f && dbasis != ~0ull) {
                    const long long qi = (long long)atomicAdd((unsigned long long *)&ctl->n_q_c2, 1ull);
                    if (qi < B.q_c2_cap) { B.q_c2[qi] = (int)x; B.q_c2b[qi] = dbasis; queued = true; }
                }
                if (!queued) {
                    const long long qi = (long long)atomicAdd((unsigned long long *)&ctl->n_q_opt, 1ull);
                    if (qi < B.q_cap) B.q_opt[qi] = (int)x; else atomicOr(&ctl->overflow, OV_QUEUE);
                }
            }
            __syncwarp();
            continue;
        }
        // a final "not optimal" only leaves a diagnostic record
        if (lane == 0 && nd.rec >= 0 && B.rec) {
            OptResult res;
            res.licq = 1; res.lp2_status = status; res.lp2_piv = piv;
            res.cheb_status = LP_SKIPPED; res.cheb_piv = 0; res.optimal = 0; res.region = 0;
            res.t = (double)t; res.r = __longlong_as_double(0x7ff8000000000000LL);
            res.decided = true;
            write_opt(B, nd, level, res, false);
        }
        __syncwarp();
    }
    if (lc.inst >= 0 && lane == 0) {
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].optimal, (unsigned long long)lc.a);
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].region, (unsigned long long)lc.b);
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].lp2_piv, (unsigned long long)lc.c);
        atomicAdd((unsigned long long *)&B.ictl[lc.inst].cheb_piv, (unsigned long long)lc.d);
    }
}

// ---------------------------------------------------------------------
// Constraint reduction: one FP64 LP per row (redundancy test)
// ---------------------------------------------------------------------
// The LP rows are M u <= d (u = (x, theta) free, nv columns, row-major M).
// For each row i of `check`: max a_i u over all rows, with row i relaxed to
// d_i + 1 so that the maximum stays finite; row i is redundant when that
// maximum is at most d_i + tol.  One warp per row, the FP64 warp simplex from
// the slack basis (u = 0 is feasible: d >= 0).  out[c] = 1 redundant, 0 not
// (an iteration limit keeps the row).
__global__ void __launch_bounds__(32) k_redundancy(const double *M, const double *d, int nrows, int nv, int ld,
                                                   const int *check, int n_check, double tol, Tol lt, int max_piv,
                                                   int *out)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id();
    double *T = (double *)smem;
    uint8_t *bid = smem + align16((size_t)(nrows + 1) * ld * sizeof(double));
    uint8_t *nid = bid + nrows;
    for (int c = blockIdx.x; c < n_check; c += gridDim.x) {
        const int i = check[c];
        for (int e = lane; e < nrows * nv; e += 32) {
            const int r = e / nv, j = e - r * nv;
            T[(size_t)r * ld + j] = M[e];
        }
        for (int r = lane; r < nrows; r += 32) {
            T[(size_t)r * ld + nv] = d[r] + (r == i ? 1.0 : 0.0);
            bid[r] = (uint8_t)(nv + r);
        }
        // objective: minimise -a_i u  (z = 0 - sum_j a_ij u_j)
        for (int j = lane; j <= nv; j += 32) {
            T[(size_t)nrows * ld + j] = j < nv ? M[(size_t)i * nv + j] : 0.0;
            if (j < nv) nid[j] = (uint8_t)j;
        }
        __syncwarp();
        Lp<double> L{T, ld, nrows, nv, nv, bid, nid};
        int piv = 0;
        const int st = warp_simplex<double>(L, lt.tol_piv, lt.tol_dj, max_piv, lt.degen_switch, &piv);
        const double maxval = -T[(size_t)nrows * ld + nv];
        if (lane == 0) out[c] = (st == LP_OPTIMAL && maxval <= d[i] + tol) ? 1 : 0;
        __syncwarp();
    }
}

template <typename T>
__global__ void k_level0(DevBuffers B)
{
    const int lane = lane_id();
    const int inst = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (inst >= B.n_inst) return;
    const InstDesc &I = B.inst[inst];
    Ctl *ctl = B.ctl;
    long long toff = 0, ioff = 0;
    for (int i = 0; i < inst; i++) { toff += B.inst[i].tab_elems; ioff += B.inst[i].ids_bytes; }
    T *dst = (T *)B.tab[0] + toff;
    const T *src = pool_of<T>(B) + root_off<T>(I);
    warp_copy_v<T>(dst, src, I.tab_elems);
    uint8_t *ids = B.ids[0] + ioff;
    if constexpr (sizeof(T) == 4) {
        // the FP32 root has its free variables basic (their rows dropped);
        // its basis ids follow the tableau in the pool
        const float *rid = B.fpool + I.f_root + I.tab_elems;
        for (int i = lane; i < I.M1 + I.nv; i += 32) ids[i] = (uint8_t)(int)rid[i];
    } else {
        for (int i = lane; i < I.M1; i += 32) ids[i] = (uint8_t)(I.nv + i);
        for (int j = lane; j < I.nv; j += 32) ids[I.M1 + j] = (uint8_t)j;
    }
    if (lane == 0) {
        Node nd;
        nd.lo = 0; nd.hi = 0; nd.inst = inst; nd.tab_off = toff; nd.ids_off = ioff;
        nd.flags = NODE_VALID | NODE_FEASIBLE | (sizeof(T) == 4 ? (I.root_rows + 1) << kNodeRowsShift : 0);
        nd.rec = (B.rec && inst < B.rec_cap) ? inst : -1;
        B.node[0][inst] = nd;
        if (!B.exhaustive) {
            hash_insert(B.hash[0], hash_cap_for(B, B.n_inst), hash_tag(ctl->epoch, 0), inst, 0, 0);
        }
        if (nd.rec >= 0) {
            CandRec &R = B.rec[nd.rec];
            R.mask_lo = 0; R.mask_hi = 0; R.level = 0; R.parent = -1;
            R.lp1_status = LP_OPTIMAL; R.lp1_pivots = 0; R.z = 0.0;
            R.feasible = 1; R.licq = 0; R.optimal = 0; R.region = 0;
            R.lp2_status = LP_SKIPPED; R.lp2_pivots = 0; R.cheb_status = LP_SKIPPED; R.cheb_pivots = 0;
            R.t = __longlong_as_double(0x7ff8000000000000LL); R.r = R.t;
            R.inst = inst; R.fp64 = 1;
            R.lp1_growth = 0.0f; R.lp1_minbeta = 0.0f; R.lp1_bound = R.t;
        }
        InstCtl *ic = &B.ictl[inst];
        ic->lvl_cand = 1;
        ic->feasible = 1;
        ic->feas_digest = mask_digest(0, 0);
        if (inst == 0) {
            long long tt = 0, it = 0;
            for (int i = 0; i < B.n_inst; i++) { tt += B.inst[i].tab_elems; it += B.inst[i].ids_bytes; }
            ctl->n_node[0] = B.n_inst;
            ctl->n_cand = B.n_inst;
            ctl->tab_used[0] = tt;
            ctl->ids_used[0] = it;
        }
    }
}

// Reset all counters (first node of every run).
__global__ void k_reset(DevBuffers B)
{
    const int t = threadIdx.x;
    for (int i = t; i < B.n_inst; i += blockDim.x) {
        InstCtl z = {};
        B.ictl[i] = z;
    }
    if (t == 0) {
        Ctl z = {};
        *B.ctl = z;
        B.ctl->epoch = (int)(atomicAdd(&g_hash_epoch, 1u) & 0x7fffffffu);
    }
}

// After each level: budget bookkeeping and counter resets.
__global__ void k_finalize(DevBuffers B, int level)
{
    const int t = threadIdx.x;
    Ctl *ctl = B.ctl;
    for (int i = t; i < B.n_inst; i += blockDim.x) {
        InstCtl *ic = &B.ictl[i];
        const InstDesc &I = B.inst[i];
        if (!ic->stopped) {
            if (I.budget > 0 && ic->cum_cand + ic->lvl_cand > I.budget) {
                ic->stopped = 1;
                ic->truncated = 1;
            } else {
                ic->cum_cand += ic->lvl_cand;
                ic->parents += ic->lvl_parents;
                ic->par_bytes += ic->lvl_par_bytes;
                if (ic->lvl_cand > 0) ic->last_level = level;
                if (level >= I.k_max || ic->lvl_cand == 0) ic->stopped = 1;
            }
        }
        ic->lvl_cand = 0;
        ic->lvl_parents = 0;
        ic->lvl_par_bytes = 0;
    }
    __syncthreads();
    if (t == 0) {
        const int pside = (level & 1) ^ 1;
        if (B.rec) ctl->rec_base += ctl->n_cand;
        ctl->hcap[level & 1] = hash_cap_for(B, ctl->n_cand);   // what this level's inserts used
        ctl->n_cand = 0;
        if (ctl->tab_full[level & 1]) ctl->split_levels++;   // this level's children partly without a tableau
        if (level > 0) {
            ctl->n_node[pside] = 0;
            ctl->tab_used[pside] = 0;
            ctl->ids_used[pside] = 0;
            ctl->tab_full[pside] = 0;
        }
        for (int c = 0; c < kCtlCounters; c++) ctl->ctr[c] = 0;
        ctl->n_q_lp1 = 0;
        ctl->n_q_cert = 0;
        ctl->n_q_opt = 0;
        ctl->n_q_scr = 0;
        ctl->n_q_s0 = 0;
        ctl->n_q_s1 = 0;
        ctl->n_q_c2 = 0;
        ctl->level = level;
    }
}

// ---------------------------------------------------------------------
// K4: region laws of given active sets (FP64)
// ---------------------------------------------------------------------
// Output per set (stride doubles): lagrange rows [lagrange_A | lagrange_b]
// (k x (p+1)), then parameter rows [parameter_A | parameter_b] (n x (p+1)),
// then the normalised region rows [CR_As | CR_bs] (n_cr x (p+1)).
// sizes = {k, n, p, n_cr}; k = -1 when the KKT factor fails (LICQ), k = -2
// for an mpLP set with |S| < n (x(theta) is not unique; nothing written).
__global__ void __launch_bounds__(128) k_region_laws(DevBuffers B, Tol tol, SlotDims sd, const uint64_t *masks,
                                                     long long n_sets, double *laws, int *sizes, long long stride,
                                                     double *radius, double *err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const size_t slot = opt_slot_bytes<double>(sd);
    OptWs<double> ws(smem + wib * slot, sd);
    const InstDesc &I = B.inst[0];
    const KktData<double> D = kkt_data<double>(B, I);
    const int m = I.m, n = I.n, p = I.p, ncp = I.ncp, P1 = p + 1, R2 = m + ncp;
    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long x = gw; x < n_sets; x += nw) {
        const uint64_t lo = masks[2 * x], hi = masks[2 * x + 1];
        double *out = laws + x * stride;
        int *sz = sizes + 4 * x;
        int k = 0;
        if (radius && lane == 0) radius[x] = __longlong_as_double(0x7ff8000000000000LL);
        if (err && lane == 0) err[x] = __longlong_as_double(0x7ff8000000000000LL);
        if (kkt_factor<double>(D, I, lo, hi, tol.tol_licq, ws, &k)) {
            if (lane == 0) { sz[0] = -1; sz[1] = n; sz[2] = p; sz[3] = 0; }
            continue;
        }
        if (I.lp && k < n) {   // mpLP with |S| < n: no unique law x(theta)
            if (lane == 0) { sz[0] = -2; sz[1] = n; sz[2] = p; sz[3] = 0; }
            __syncwarp();
            continue;
        }
        if (I.lp) {
            mplp_multipliers(B, I, k, ws);
            region_rows<double, false, true>(D, I, lo, hi, k, ws);
        } else {
            region_rows<double>(D, I, lo, hi, k, ws);
        }
        const double *Lam = ws.Lam;
        const double *LamL = I.lp ? ws.Psi : Lam;
        const double *QiAT = B.dpool + I.o_QiAT, *QiH = B.dpool + I.o_QiH, *Qic = B.dpool + I.o_Qic;
        for (int a = lane; a < k; a += 32)
            for (int cc = 0; cc < P1; cc++) out[a * P1 + cc] = -LamL[a * P1 + cc];
        double *par = out + (long long)m * P1;
        for (int r = lane; r < n; r += 32) {
            for (int cc = 0; cc < P1; cc++) {
                double acc = (cc < p) ? -QiH[r * p + cc] : -Qic[r];
                for (int l = 0; l < k; l++) acc = xfma(QiAT[(size_t)r * m + ws.S[l]], Lam[l * P1 + cc], acc);
                par[r * P1 + cc] = acc;
            }
        }
        double *cr = par + (long long)n * P1;
        const double *G = ws.G;
        int nc = 0;
        for (int r0 = 0; r0 < R2; r0 += 32) {
            const int r = r0 + lane;
            bool keep = false;
            if (r < R2) {
                if (r >= m) keep = true;
                else keep = nonzero_row<double>(G + (size_t)r * P1, p, tol.tol_zero_row);
            }
            const unsigned km = __ballot_sync(FULLMASK, keep);
            if (keep) {
                const int np = nc + __popc(km & ((1u << lane) - 1u));
                const double *g = G + (size_t)r * P1;
                double acc = 0.0;
                for (int cc = 0; cc < p; cc++) acc = xfma(g[cc], g[cc], acc);
                const double inv = xdiv(1.0, xsqrt(acc));
                for (int cc = 0; cc < p; cc++) cr[np * P1 + cc] = xmul(g[cc], inv);
                cr[np * P1 + p] = xmul(g[p], inv);
            }
            nc += __popc(km);
        }
        if (lane == 0) { sz[0] = k; sz[1] = n; sz[2] = p; sz[3] = nc; }
        __syncwarp();
        if (radius) {
            // the Chebyshev radius of the same rows (region when >= r_min)
            OptResult res;
            res.r = __longlong_as_double(0x7ff8000000000000LL); res.region = 0;
            chebyshev_ball<double>(tol, I, ws, res);
            if (lane == 0) radius[x] = res.r;
            __syncwarp();
        }
        if (err) {
            const double e = law_error(B, I, k, ws);
            if (lane == 0) err[x] = e;
            __syncwarp();
        }
    }
}

size_t laws_smem_per_warp(const SlotDims &sd) { return opt_slot_bytes<double>(sd); }

cudaError_t launch_region_laws(const DevBuffers &B, const Tol &tol, const SlotDims &sd, const uint64_t *masks,
                               long long n_sets, double *laws, int *sizes, long long stride, int grid, size_t smem,
                               cudaStream_t s)
{
    k_region_laws<<<grid, 128, smem, s>>>(B, tol, sd, masks, n_sets, laws, sizes, stride, nullptr, nullptr);
    return cudaGetLastError();
}

// the same with each set's Chebyshev radius and law error (n_sets doubles
// each, either may be null)
cudaError_t launch_region_laws_r(const DevBuffers &B, const Tol &tol, const SlotDims &sd, const uint64_t *masks,
                                 long long n_sets, double *laws, int *sizes, long long stride, double *radius,
                                 double *err, int grid, size_t smem, cudaStream_t s)
{
    k_region_laws<<<grid, 128, smem, s>>>(B, tol, sd, masks, n_sets, laws, sizes, stride, radius, err);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------
// explicit instantiations / host-visible launch wrappers
// ---------------------------------------------------------------------
size_t feas_smem_per_warp(int prec_bytes, const SlotDims &sd)
{
    return prec_bytes == 8 ? feas_slot_bytes<double>(sd.maxM1, sd.maxLD1d, sd.maxNv)
                           : feas_slot_bytes<float>(sd.maxM1, sd.maxLD1, sd.maxNv);
}

size_t cert_smem_per_warp(const SlotDims &sd) { return cert_slot_bytes(sd.maxNv); }

size_t lp1_smem_per_warp(int prec_bytes, const SlotDims &sd)
{
    return prec_bytes == 8 ? lp1_slot_bytes<double>(sd.maxM1, sd.maxLD1d, sd.maxNv)
                           : lp1_slot_bytes<float>(sd.maxM1, sd.maxLD1, sd.maxNv);
}

size_t screen_smem_per_warp(const SlotDims &sd, int route) { return screen_warp_bytes(sd, route); }
size_t screen_tiles_smem(const SlotDims &sd, int tile_w) { return (32 / tile_w) * tile_slot_bytes(sd); }   // a 32-thread block
bool screen_dual_route(int mode, const InstDesc &I, const SlotDims &sd) { return dual_route(mode, I, sd); }
bool screen_lanes_route(int mode, const InstDesc &I, const SlotDims &sd) { return lanes_route(mode, I, sd); }

size_t opt_smem_per_warp(int prec_bytes, const SlotDims &sd)
{
    return prec_bytes == 8 ? opt_slot_bytes<double>(sd) : opt_slot_bytes<float>(sd);
}

}  // namespace mq

using namespace mq;

// Launch wrappers (plain C++ linkage inside the library)
namespace mq {

const void *kernel_ptr(const char *name)
{
    struct E { const char *n; const void *f; };
    static const E tab[] = {
        {"enumerate", (const void *)k_enumerate},
        {"feas64", (const void *)k_feasibility<double>},
        {"feas32", (const void *)k_feasibility<float>},
        {"lp1_fp64", (const void *)k_lp1_fp64},
        {"lp1_cert", (const void *)k_lp1_cert},
        {"opt64", (const void *)k_optimality<double, false>},
        {"opt64_lp", (const void *)k_optimality<double, true>},
        {"opt_fp64", (const void *)k_optimality_fp64<false>},
        {"opt_fp64_lp", (const void *)k_optimality_fp64<true>},
        {"screen_dual_rows", (const void *)k_opt_screen<0, 1>},
        {"screen_dual_rows_lp", (const void *)k_opt_screen<0, 2>},
        {"screen_dual_tiles8", (const void *)k_opt_screen_tiles<8>},
        {"screen_dual_tiles16", (const void *)k_opt_screen_tiles<16>},
        {"screen_dual_tiles32", (const void *)k_opt_screen_tiles<32>},
        {"screen_dual_lanes", (const void *)k_opt_screen_lanes},
        {"screen_dual_tiles8w", (const void *)k_opt_screen_tiles<8, true>},
        {"screen_dual_tiles16w", (const void *)k_opt_screen_tiles<16, true>},
        {"screen_dual_tiles32w", (const void *)k_opt_screen_tiles<32, true>},
        {"screen_primal", (const void *)k_opt_screen<1>},
        {"level0_64", (const void *)k_level0<double>},
        {"level0_32", (const void *)k_level0<float>},
        {"reset", (const void *)k_reset},
        {"finalize", (const void *)k_finalize},
        {"laws", (const void *)k_region_laws},
    };
    for (const E &e : tab) {
        const char *a = e.n, *b = name;
        while (*a && *a == *b) { a++; b++; }
        if (*a == 0 && *b == 0) return e.f;
    }
    return nullptr;
}

cudaError_t launch_enumerate(const DevBuffers &B, int level, int grid, cudaStream_t s)
{
    k_enumerate<<<grid, 128, 0, s>>>(B, level);
    return cudaGetLastError();
}

// warps: warps per block (1..4, smem = warps x the slot); chunk: candidates
// a warp claims at a time (1..32)
cudaError_t launch_feasibility(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int prec,
                               int grid, size_t smem, cudaStream_t s, int warps, int chunk)
{
    if (warps < 1 || warps > 4 || chunk < 1 || chunk > kFeasChunkMax) return cudaErrorInvalidValue;
    if (prec == PREC_FP64) k_feasibility<double><<<grid, 32 * warps, smem, s>>>(B, tol, sd, level, chunk);
    else k_feasibility<float><<<grid, 32 * warps, smem, s>>>(B, tol, sd, level, chunk);
    return cudaGetLastError();
}

cudaError_t launch_lp1_fp64(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int grid,
                            size_t smem, cudaStream_t s)
{
    k_lp1_fp64<<<grid, 128, smem, s>>>(B, tol, sd, level);
    return cudaGetLastError();
}

cudaError_t launch_lp1_cert(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int grid,
                            size_t smem, cudaStream_t s)
{
    k_lp1_cert<<<grid, 128, smem, s>>>(B, tol, sd, level);
    return cudaGetLastError();
}

cudaError_t launch_optimality(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, bool lp,
                              int grid, size_t smem, cudaStream_t s)
{
    // the FP32 screen of the mixed path is launch_opt_screen
    if (lp) k_optimality<double, true><<<grid, 128, smem, s>>>(B, tol, sd, level);
    else k_optimality<double, false><<<grid, 128, smem, s>>>(B, tol, sd, level);
    return cudaGetLastError();
}

cudaError_t launch_opt_screen(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, int mode, int route,
                              int grid, size_t smem, cudaStream_t s, int tile_w)
{
    // route 0: the dual route's first stage (tiles of tile_w threads), 2: its
    // second stage, 1: the primal route, 3: the tile stage over the mpLP sets
    // the one-set-per-thread stage queued (their stationarity rows)
    const int src = route == 3 ? 1 : 0;
    if (route == 0 && B.lp2b[0]) {
        if (tile_w == 8) k_opt_screen_tiles<8, true><<<grid, 32, smem, s>>>(B, tol, sd, level, mode, 0);
        else if (tile_w == 16) k_opt_screen_tiles<16, true><<<grid, 32, smem, s>>>(B, tol, sd, level, mode, 0);
        else if (tile_w == 32) k_opt_screen_tiles<32, true><<<grid, 32, smem, s>>>(B, tol, sd, level, mode, 0);
        else return cudaErrorInvalidValue;
    } else if (route == 0 || route == 3) {
        if (tile_w == 8) k_opt_screen_tiles<8><<<grid, 32, smem, s>>>(B, tol, sd, level, mode, src);
        else if (tile_w == 16) k_opt_screen_tiles<16><<<grid, 32, smem, s>>>(B, tol, sd, level, mode, src);
        else if (tile_w == 32) k_opt_screen_tiles<32><<<grid, 32, smem, s>>>(B, tol, sd, level, mode, src);
        else return cudaErrorInvalidValue;
    }
    else if (route == 2) k_opt_screen<0, 1><<<grid, 32, smem, s>>>(B, tol, sd, level, mode);
    else if (route == 6) k_opt_screen<0, 2><<<grid, 32, smem, s>>>(B, tol, sd, level, mode);
    else k_opt_screen<1><<<grid, 32, smem, s>>>(B, tol, sd, level, mode);
    return cudaGetLastError();
}

size_t redundancy_smem_bytes(int nrows, int ld)
{
    return align16((size_t)(nrows + 1) * ld * sizeof(double)) + align16((size_t)nrows + 64);
}

cudaError_t launch_redundancy(const double *M, const double *d, int nrows, int nv, int ld, const int *check, int n_check,
                              double tol, const Tol &lt, int max_piv, int *out, int grid, size_t smem, cudaStream_t s)
{
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_redundancy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_redundancy<<<grid, 32, smem, s>>>(M, d, nrows, nv, ld, check, n_check, tol, lt, max_piv, out);
    return cudaGetLastError();
}

cudaError_t launch_optimality_fp64(const DevBuffers &B, const Tol &tol, const SlotDims &sd, int level, bool lp,
                                   int grid, size_t smem, cudaStream_t s)
{
    if (lp) k_optimality_fp64<true><<<grid, 128, smem, s>>>(B, tol, sd, level);
    else k_optimality_fp64<false><<<grid, 128, smem, s>>>(B, tol, sd, level);
    return cudaGetLastError();
}

cudaError_t launch_level0(const DevBuffers &B, int prec, cudaStream_t s)
{
    const int warps = 4;
    const int grid = (B.n_inst + warps - 1) / warps;
    if (prec == PREC_FP64) k_level0<double><<<grid, 32 * warps, 0, s>>>(B);
    else k_level0<float><<<grid, 32 * warps, 0, s>>>(B);
    return cudaGetLastError();
}

cudaError_t launch_reset(const DevBuffers &B, cudaStream_t s)
{
    k_reset<<<1, 256, 0, s>>>(B);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const DevBuffers &B, int level, cudaStream_t s)
{
    k_finalize<<<1, 256, 0, s>>>(B, level);
    return cudaGetLastError();
}

}  // namespace mq
