/*
 * CPU oracle for the combinatorial mpQP active-set check -- TEST
 * INFRASTRUCTURE ONLY (see mpqp_oracle.h).
 *
 * Floating-point contract: every multiply-add is an explicit fma(), every
 * sum runs in ascending index order from the stated initial value, and the
 * file is compiled with -ffp-contract=off.  The FP64 device kernels follow
 * the same operation order, so the two produce bit-identical LP values and
 * verdicts on the same input.
 */
#include "mpqp_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* problem data                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
    int n, m, p, ncp;
    int M1;      /* LP1 rows: m + ncp                                  */
    int nv;      /* LP1 free variables: n + p                          */
    int ld1;     /* LP1 tableau row stride: nv + 1                     */
    int ld2;     /* LP2 / Chebyshev tableau row stride: p + 2          */
    int lp;      /* 1: Q = 0 (mpLP); the blocks below change meaning    */
    int ld2lp;   /* mpLP, |S| < n: LP2 row stride p + n + 3             */
    double *Wm;  /* m x m   A Q^-1 A^T          (mpLP: A A^T)          */
    double *Wh;  /* m x p   A Q^-1 H + F        (mpLP: F)              */
    double *wc;  /* m       b + A Q^-1 c        (mpLP: b)              */
    double *QiAT;/* n x m   Q^-1 A^T            (mpLP: A^T)            */
    double *QiH; /* n x p   Q^-1 H              (mpLP: 0)              */
    double *Qic; /* n       Q^-1 c              (mpLP: 0)              */
    double *WhL; /* mpLP: m x p  A H                                   */
    double *wcL; /* mpLP: m      A c                                   */
    double *root;/* (M1+1) x ld1, LP1 tableau of the empty set         */
    const orc_problem *pr;
} orc_data;

void orc_default_tol(orc_tol *t)
{
    t->tol_feas = 1e-9;
    t->tol_opt = 1e-9;
    t->tol_licq = 1e-10;
    t->r_min = 1e-8;
    t->tol_piv = 1e-9;
    t->tol_dj = 1e-9;
    t->max_pivots = 256;
    t->degen_switch = 8;
    t->tol_zero_row = 1e-12;
}

static void free_data(orc_data *d)
{
    free(d->Wm); free(d->Wh); free(d->wc); free(d->QiAT); free(d->QiH); free(d->Qic); free(d->root);
    free(d->WhL); free(d->wcL);
    memset(d, 0, sizeof(*d));
}

/* L y = rhs (L lower, row-major n x n) */
static void fwd_sub(const double *L, int n, const double *rhs, int rs, double *y, int ys)
{
    for (int i = 0; i < n; i++) {
        double acc = rhs[i * rs];
        for (int l = 0; l < i; l++) acc = fma(-L[i * n + l], y[l * ys], acc);
        y[i * ys] = acc / L[i * n + i];
    }
}

/* L^T x = y */
static void bwd_sub(const double *L, int n, const double *y, int ysd, double *x, int xs)
{
    for (int i = n - 1; i >= 0; i--) {
        double acc = y[i * ysd];
        for (int l = i + 1; l < n; l++) acc = fma(-L[l * n + i], x[l * xs], acc);
        x[i * xs] = acc / L[i * n + i];
    }
}

static int prepare(const orc_problem *pr, orc_data *d)
{
    memset(d, 0, sizeof(*d));
    const int n = pr->n, m = pr->m, p = pr->p, ncp = pr->ncp;
    if (n < 1 || m < 1 || p < 1 || ncp < 1 || m > 128) return -1;
    if (m + ncp + n + p > 255 || m + ncp + p + 1 > 255) return -1;
    for (int i = 0; i < m; i++) if (!(pr->b[i] >= 0.0)) return -3;   /* origin must be feasible */
    for (int i = 0; i < ncp; i++) if (!(pr->bt[i] >= 0.0)) return -3;
    d->n = n; d->m = m; d->p = p; d->ncp = ncp;
    d->M1 = m + ncp; d->nv = n + p; d->ld1 = d->nv + 1; d->ld2 = p + 2;
    d->pr = pr;
    d->lp = 1;
    for (int i = 0; i < n * n && d->lp; i++) if (pr->Q[i] != 0.0) d->lp = 0;
    d->ld2lp = p + n + 3;
    /* mpLP, |S| < n: LP2 columns theta, u, t, sigma and rows m + ncp + 2n + 1 */
    if (d->lp && (p + n + 2) + (m + ncp + 2 * n + 1) > 255) return -1;
    double *L = calloc((size_t)n * n, sizeof(double));
    double *V = calloc((size_t)n * m, sizeof(double));
    double *U = calloc((size_t)n * p, sizeof(double));
    double *u = calloc((size_t)n, sizeof(double));
    d->Wm = calloc((size_t)m * m, sizeof(double));
    d->Wh = calloc((size_t)m * p, sizeof(double));
    d->wc = calloc((size_t)m, sizeof(double));
    d->QiAT = calloc((size_t)n * m, sizeof(double));
    d->QiH = calloc((size_t)n * p, sizeof(double));
    d->Qic = calloc((size_t)n, sizeof(double));
    d->root = calloc((size_t)(d->M1 + 1) * d->ld1, sizeof(double));
    int rc = 0;
    if (d->lp) {
        /* mpLP (Q = 0): Wm = A A^T, Wh = F, wc = b, QiAT = A^T, QiH = Qic = 0,
         * WhL = A H, wcL = A c; each entry sums over ascending i from 0 */
        d->WhL = calloc((size_t)m * p, sizeof(double));
        d->wcL = calloc((size_t)m, sizeof(double));
        for (int r = 0; r < m; r++) {
            for (int s = 0; s < m; s++) {
                double acc = 0.0;
                for (int i = 0; i < n; i++) acc = fma(pr->A[r * n + i], pr->A[s * n + i], acc);
                d->Wm[r * m + s] = acc;
            }
            for (int c = 0; c < p; c++) {
                d->Wh[r * p + c] = pr->F[r * p + c];
                double acc = 0.0;
                for (int i = 0; i < n; i++) acc = fma(pr->A[r * n + i], pr->H[i * p + c], acc);
                d->WhL[r * p + c] = acc;
            }
            d->wc[r] = pr->b[r];
            double acc = 0.0;
            for (int i = 0; i < n; i++) acc = fma(pr->A[r * n + i], pr->c[i], acc);
            d->wcL[r] = acc;
            for (int i = 0; i < n; i++) d->QiAT[i * m + r] = pr->A[r * n + i];
        }
    }
    /* Cholesky Q = L L^T */
    for (int j = 0; j < n && rc == 0 && !d->lp; j++) {
        for (int i = j; i < n; i++) {
            double acc = pr->Q[i * n + j];
            for (int l = 0; l < j; l++) acc = fma(-L[i * n + l], L[j * n + l], acc);
            if (i == j) {
                if (!(acc > 0.0)) { rc = -2; break; }
                L[j * n + j] = sqrt(acc);
            } else {
                L[i * n + j] = acc / L[j * n + j];
            }
        }
    }
    if (rc == 0 && !d->lp) {
        for (int r = 0; r < m; r++) fwd_sub(L, n, pr->A + (size_t)r * n, 1, V + r, m);
        for (int c = 0; c < p; c++) fwd_sub(L, n, pr->H + c, p, U + c, p);
        fwd_sub(L, n, pr->c, 1, u, 1);
        for (int r = 0; r < m; r++) {
            for (int s = 0; s < m; s++) {
                double acc = 0.0;
                for (int i = 0; i < n; i++) acc = fma(V[i * m + r], V[i * m + s], acc);
                d->Wm[r * m + s] = acc;
            }
            for (int c = 0; c < p; c++) {
                double acc = pr->F[r * p + c];
                for (int i = 0; i < n; i++) acc = fma(V[i * m + r], U[i * p + c], acc);
                d->Wh[r * p + c] = acc;
            }
            double acc = pr->b[r];
            for (int i = 0; i < n; i++) acc = fma(V[i * m + r], u[i], acc);
            d->wc[r] = acc;
        }
        for (int r = 0; r < m; r++) bwd_sub(L, n, V + r, m, d->QiAT + r, m);
        for (int c = 0; c < p; c++) bwd_sub(L, n, U + c, p, d->QiH + c, p);
        bwd_sub(L, n, u, 1, d->Qic, 1);
    }
    if (rc == 0) {
        /* LP1 root tableau: rows [A -F; 0 At], rhs [b; bt], objective row 0 */
        const int ld = d->ld1;
        for (int i = 0; i < m; i++) {
            for (int j = 0; j < n; j++) d->root[i * ld + j] = pr->A[i * n + j];
            for (int j = 0; j < p; j++) d->root[i * ld + n + j] = -pr->F[i * p + j];
            d->root[i * ld + d->nv] = pr->b[i];
        }
        for (int i = 0; i < ncp; i++) {
            for (int j = 0; j < p; j++) d->root[(m + i) * ld + n + j] = pr->At[i * p + j];
            d->root[(m + i) * ld + d->nv] = pr->bt[i];
        }
    }
    free(L); free(V); free(U); free(u);
    if (rc) free_data(d);
    return rc;
}

int orc_kkt_data(const orc_problem *pr, double *Wm, double *Wh, double *wc)
{
    orc_data d;
    int rc = prepare(pr, &d);
    if (rc) return rc;
    memcpy(Wm, d.Wm, sizeof(double) * pr->m * pr->m);
    memcpy(Wh, d.Wh, sizeof(double) * pr->m * pr->p);
    memcpy(wc, d.wc, sizeof(double) * pr->m);
    free_data(&d);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Tucker-tableau simplex                                               */
/* ------------------------------------------------------------------ */
/* Layout: rows 0..nrows-1 are basic variables, row nrows the objective;
 * columns 0..ncols-1 nonbasic variables, column ncols the right-hand side.
 * Each row reads  x_B = T[.,ncols] - sum_j T[.,j] x_N(j); the objective row
 * reads z = T[nrows,ncols] - sum_j T[nrows,j] x_N(j) and z is minimised.
 * Variables with id < nfree are free (never leave the basis), the others are
 * nonnegative.  Pricing: largest |reduced cost| with the smallest id on ties
 * (Bland's smallest-id rule after degen_switch consecutive degenerate
 * pivots); ratio test: smallest max(beta,0)/a over a > tol_piv, smallest id
 * on ties. */

static void tucker_pivot(double *T, int ld, int nrows_tot, int ncols_tot, int r, int q)
{
    double *R = T + (size_t)r * ld;
    const double inv = 1.0 / R[q];
    for (int j = 0; j < ncols_tot; j++)
        if (j != q) R[j] = R[j] * inv;
    R[q] = inv;
    for (int i = 0; i < nrows_tot; i++) {
        if (i == r) continue;
        double *Ti = T + (size_t)i * ld;
        const double f = Ti[q];
        for (int j = 0; j < ncols_tot; j++)
            if (j != q) Ti[j] = fma(-f, R[j], Ti[j]);
        Ti[q] = -f * inv;
    }
}

static int tucker_solve(double *T, int ld, int nrows, int ncols, uint8_t *bid, uint8_t *nid,
                        int nfree, const orc_tol *tol, int *pivots)
{
    int piv = 0, degen = 0, bland = 0, status;
    const double *obj = T + (size_t)nrows * ld;
    for (;;) {
        int q = -1, qid = 1 << 30;
        double qs = 0.0;
        for (int j = 0; j < ncols; j++) {
            const double g = obj[j];
            const int id = nid[j];
            const double s = (id < nfree) ? fabs(g) : g;
            if (!(s > tol->tol_dj)) continue;
            if (bland) {
                if (id < qid) { q = j; qid = id; qs = s; }
            } else if (s > qs || (s == qs && id < qid)) {
                q = j; qid = id; qs = s;
            }
        }
        if (q < 0) { status = ORC_OPTIMAL; break; }
        const double sg = obj[q] > 0.0 ? 1.0 : -1.0;
        int r = -1, rid = 1 << 30;
        double rr = 0.0;
        for (int i = 0; i < nrows; i++) {
            const int id = bid[i];
            if (id < nfree) continue;
            const double a = sg * T[(size_t)i * ld + q];
            if (!(a > tol->tol_piv)) continue;
            double beta = T[(size_t)i * ld + ncols];
            if (!(beta > 0.0)) beta = 0.0;
            const double ratio = beta / a;
            if (r < 0 || ratio < rr || (ratio == rr && id < rid)) { r = i; rr = ratio; rid = id; }
        }
        if (r < 0) { status = ORC_UNBOUNDED; break; }
        if (piv >= tol->max_pivots) { status = ORC_ITER_LIMIT; break; }
        tucker_pivot(T, ld, nrows + 1, ncols + 1, r, q);
        const uint8_t t = bid[r]; bid[r] = nid[q]; nid[q] = t;
        piv++;
        if (rr == 0.0) degen++; else degen = 0;
        bland = degen >= tol->degen_switch;
    }
    *pivots = piv;
    return status;
}

/* ------------------------------------------------------------------ */
/* LP1: feasibility of S = parent + {j}, warm-started from the parent   */
/* ------------------------------------------------------------------ */

typedef struct {
    double *T;      /* (M1+1) x ld1 */
    uint8_t *bid;   /* M1 */
    uint8_t *nid;   /* nv */
} lp1_state;

static void lp1_init_root(const orc_data *d, lp1_state *s)
{
    memcpy(s->T, d->root, sizeof(double) * (d->M1 + 1) * d->ld1);
    for (int i = 0; i < d->M1; i++) s->bid[i] = (uint8_t)(d->nv + i);
    for (int j = 0; j < d->nv; j++) s->nid[j] = (uint8_t)j;
}

static void lp1_child(const orc_data *d, const lp1_state *par, int j, lp1_state *s,
                      const orc_tol *tol, int *status, int *pivots, double *z)
{
    const int ld = d->ld1, M1 = d->M1, nv = d->nv;
    memcpy(s->T, par->T, sizeof(double) * (M1 + 1) * ld);
    memcpy(s->bid, par->bid, M1);
    memcpy(s->nid, par->nid, nv);
    const int wid = nv + j;
    double *obj = s->T + (size_t)M1 * ld;
    int rho = -1;
    for (int i = 0; i < M1; i++) if (s->bid[i] == wid) { rho = i; break; }
    if (rho >= 0) {
        const double *row = s->T + (size_t)rho * ld;
        for (int c = 0; c <= nv; c++) obj[c] = obj[c] + row[c];
    } else {
        for (int c = 0; c < nv; c++) if (s->nid[c] == wid) { obj[c] = obj[c] - 1.0; break; }
    }
    *status = tucker_solve(s->T, ld, M1, nv, s->bid, s->nid, nv, tol, pivots);
    *z = obj[nv];
}

/* ------------------------------------------------------------------ */
/* KKT factor, region rows, LP2 (optimality) and the Chebyshev LP        */
/* ------------------------------------------------------------------ */

typedef struct {
    double *R;     /* k x k upper Cholesky factor of Wm[S,S]  (kmax x kmax) */
    double *Y;     /* k x (p+1) */
    double *Lam;   /* k x (p+1): Lambda = Wm[S,S]^-1 [Wh_S | wc_S] */
    double *G;     /* (m+ncp) x (p+1) region rows [g | h] in reference order */
    double *T;     /* (m+ncp+1) x ld2 LP tableau (mpLP: (m+ncp+2n+2) x ld2lp) */
    uint8_t *bid, *nid;
    double *Psi;   /* mpLP: k x (p+1), Wm[S,S]^-1 [WhL_S | wcL_S] (multiplier law) */
    double *Phi;   /* mpLP: k x n,     Wm[S,S]^-1 A_S */
} opt_ws;

static void opt_ws_alloc(const orc_data *d, opt_ws *w)
{
    const int m = d->m, p = d->p, n = d->n, R = m + d->ncp;
    const size_t tq = (size_t)(R + 1) * d->ld2, tl = (size_t)(R + 2 * n + 2) * d->ld2lp;
    w->R = calloc((size_t)m * m, sizeof(double));
    w->Y = calloc((size_t)m * (p + 1), sizeof(double));
    w->Lam = calloc((size_t)m * (p + 1), sizeof(double));
    w->G = calloc((size_t)R * (p + 1), sizeof(double));
    w->T = calloc(d->lp && tl > tq ? tl : tq, sizeof(double));
    w->bid = calloc((size_t)R + 2 * n + 1, 1);
    w->nid = calloc((size_t)p + n + 2, 1);
    w->Psi = calloc((size_t)m * (p + 1), sizeof(double));
    w->Phi = calloc((size_t)m * n, sizeof(double));
}

static void opt_ws_free(opt_ws *w)
{
    free(w->R); free(w->Y); free(w->Lam); free(w->G); free(w->T); free(w->bid); free(w->nid);
    free(w->Psi); free(w->Phi);
}

/* X = Wm[S,S]^-1 B in place (R the upper Cholesky factor, k x k): X holds
 * B_S on entry (row stride ldx, ncols columns); per column a forward then a
 * backward substitution, each accumulating in ascending l */
static void chol_solve_inplace(const double *R, int k, double *X, int ldx, int ncols)
{
    for (int a = 0; a < k; a++)
        for (int c = 0; c < ncols; c++) {
            double acc = X[a * ldx + c];
            for (int l = 0; l < a; l++) acc = fma(-R[l * k + a], X[l * ldx + c], acc);
            X[a * ldx + c] = acc / R[a * k + a];
        }
    for (int a = k - 1; a >= 0; a--)
        for (int c = 0; c < ncols; c++) {
            double acc = X[a * ldx + c];
            for (int l = a + 1; l < k; l++) acc = fma(-R[a * k + l], X[l * ldx + c], acc);
            X[a * ldx + c] = acc / R[a * k + a];
        }
}

/* mpLP (Q = 0) with |S| = k < n: x is not fixed by S, so LP2 keeps a
 * direction u in the null space of A_S (x = A_S^T Gamma(theta) + P u, P the
 * projector onto that null space) and the stationarity residual
 * (c + H theta) - A_S^T Psi(theta) = r0 + E theta (zero when S can be
 * optimal) as rows |r0 + E theta| <= tol_feas -- the reference's LP2 keeps x
 * and the equalities of main.py:107-108 as they are.  Two phases: min sigma
 * over rows +-(r0 + E theta) - sigma <= tol_feas (sigma free), then, when
 * sigma* <= 0, the row -sigma >= 0 is appended and max t solved from that
 * basis.  Columns theta (p), u (n), t, sigma; rows: the m margin rows (G,
 * reference order, plus A_i P in the u columns of inactive rows), the ncp
 * parameter rows, 2n residual rows. */
static void lp2_short_mplp(const orc_data *d, const int *S, int k, const orc_tol *tol, opt_ws *w, orc_cand *rec)
{
    const int m = d->m, n = d->n, p = d->p, ncp = d->ncp, P1 = p + 1, ld = d->ld2lp;
    const int ncols = p + n + 2, ct = p + n, cs = p + n + 1;
    const int nrows = m + ncp + 2 * n;
    const double *G = w->G, *Phi = w->Phi, *Psi = w->Psi, *A = d->QiAT;
    double *T = w->T;
    double t0 = INFINITY;
    for (int r = 0; r < m; r++) if (G[r * P1 + p] < t0) t0 = G[r * P1 + p];
    memset(T, 0, sizeof(double) * (size_t)(nrows + 2) * ld);
    int si = 0, row = k;
    for (int r = 0; r < k; r++) {
        double *Tr = T + (size_t)r * ld;
        for (int c = 0; c < p; c++) Tr[c] = G[r * P1 + c];
        Tr[ct] = 1.0;
        double beta = fma(-1.0, t0, G[r * P1 + p]);
        if (!(beta > 0.0)) beta = 0.0;
        Tr[ncols] = beta;
    }
    for (int i = 0; i < m; i++) {
        if (si < k && S[si] == i) { si++; continue; }
        double *Tr = T + (size_t)row * ld;
        for (int c = 0; c < p; c++) Tr[c] = G[row * P1 + c];
        for (int j = 0; j < n; j++) {
            double acc = A[j * m + i];
            for (int l = 0; l < k; l++) acc = fma(-d->Wm[i * m + S[l]], Phi[l * n + j], acc);
            Tr[p + j] = acc;
        }
        Tr[ct] = 1.0;
        double beta = fma(-1.0, t0, G[row * P1 + p]);
        if (!(beta > 0.0)) beta = 0.0;
        Tr[ncols] = beta;
        row++;
    }
    for (int i = 0; i < ncp; i++) {
        double *Tr = T + (size_t)(m + i) * ld;
        for (int c = 0; c < p; c++) Tr[c] = d->pr->At[i * p + c];
        Tr[ncols] = d->pr->bt[i];
    }
    const double eps = tol->tol_feas;
    double rmax = 0.0;
    for (int i = 0; i < n; i++) {
        double *Tp = T + (size_t)(m + ncp + 2 * i) * ld, *Tn = Tp + ld;
        for (int c = 0; c < p; c++) {
            double acc = d->pr->H[i * p + c];
            for (int l = 0; l < k; l++) acc = fma(-A[i * m + S[l]], Psi[l * P1 + c], acc);
            Tp[c] = acc;
            Tn[c] = -acc;
        }
        double acc = d->pr->c[i];
        for (int l = 0; l < k; l++) acc = fma(-A[i * m + S[l]], Psi[l * P1 + p], acc);
        Tp[cs] = -1.0; Tn[cs] = -1.0;
        Tp[ncols] = eps - acc;   /* rhs before the sigma shift */
        Tn[ncols] = eps + acc;
        if (fabs(acc) > rmax) rmax = fabs(acc);
    }
    const double s0 = rmax - eps;
    for (int r = m + ncp; r < nrows; r++) {
        double beta = T[(size_t)r * ld + ncols] + s0;
        if (!(beta > 0.0)) beta = 0.0;
        T[(size_t)r * ld + ncols] = beta;
    }
    for (int r = 0; r < nrows; r++) w->bid[r] = (uint8_t)(ncols + r);
    for (int c = 0; c < ncols; c++) w->nid[c] = (uint8_t)c;
    /* phase 1: min sigma = s0 + sigma' */
    double *obj = T + (size_t)nrows * ld;
    obj[cs] = -1.0;
    obj[ncols] = s0;
    int piv1 = 0, piv2 = 0;
    int st = tucker_solve(T, ld, nrows, ncols, w->bid, w->nid, ncols, tol, &piv1);
    rec->lp2_pivots = piv1;
    if (st != ORC_OPTIMAL) { rec->lp2_status = st; return; }
    const double sig = obj[ncols];
    if (sig > 0.0) { rec->lp2_status = ORC_INFEASIBLE; rec->t = -INFINITY; return; }
    /* row nrows: s = -sigma >= 0 in the current basis (sigma basic in row rs,
     * or nonbasic in column qs); row nrows + 1: objective -t */
    int rs = -1, qs = -1, rt = -1, qt = -1;
    for (int r = 0; r < nrows; r++) { if (w->bid[r] == cs) rs = r; if (w->bid[r] == ct) rt = r; }
    for (int c = 0; c < ncols; c++) { if (w->nid[c] == cs) qs = c; if (w->nid[c] == ct) qt = c; }
    double *Ts = T + (size_t)nrows * ld, *ob = Ts + ld;
    for (int c = 0; c <= ncols; c++) { Ts[c] = 0.0; ob[c] = 0.0; }
    if (rs >= 0) {
        const double *Tr = T + (size_t)rs * ld;
        for (int c = 0; c < ncols; c++) Ts[c] = -Tr[c];
        Ts[ncols] = -s0 - Tr[ncols];
    } else {
        Ts[qs] = 1.0;
        Ts[ncols] = -s0;
    }
    w->bid[nrows] = (uint8_t)(ncols + nrows);
    if (rt >= 0) {
        const double *Tr = T + (size_t)rt * ld;
        for (int c = 0; c < ncols; c++) ob[c] = -Tr[c];
        ob[ncols] = -t0 - Tr[ncols];
    } else {
        ob[qt] = 1.0;
        ob[ncols] = -t0;
    }
    st = tucker_solve(T, ld, nrows + 1, ncols, w->bid, w->nid, ncols, tol, &piv2);
    rec->lp2_pivots = piv1 + piv2;
    rec->lp2_status = st;
    if (st == ORC_OPTIMAL) {
        rec->t = -ob[ncols];
        rec->optimal = rec->t > tol->tol_opt;
    } else if (st == ORC_UNBOUNDED) {
        rec->t = INFINITY;
    }
}

/* Tableau for max t (LP2) or max r (Chebyshev) over rows g theta + a_r * v <= h,
 * v free, shifted so that v = v0 + v' starts feasible at theta = 0. */
static void build_margin_lp(const orc_data *d, opt_ws *w, int nrows, const double *coef, double v0)
{
    const int p = d->p, ld = d->ld2;
    for (int r = 0; r < nrows; r++) {
        double *Tr = w->T + (size_t)r * ld;
        const double *g = w->G + (size_t)r * (p + 1);
        for (int c = 0; c < p; c++) Tr[c] = g[c];
        Tr[p] = coef[r];
        double beta = fma(-coef[r], v0, g[p]);
        if (!(beta > 0.0)) beta = 0.0;
        Tr[p + 1] = beta;
        w->bid[r] = (uint8_t)(p + 1 + r);
    }
    double *obj = w->T + (size_t)nrows * ld;
    for (int c = 0; c < p; c++) obj[c] = 0.0;
    obj[p] = 1.0;
    obj[p + 1] = -v0;
    for (int c = 0; c <= p; c++) w->nid[c] = (uint8_t)c;
}

/* Evaluate optimality and the region of S (sorted, |S| = k).  Fills the
 * LP2/Chebyshev fields of rec; optional outputs as in orc_check_set. */
static void optimality(const orc_data *d, const int *S, int k, const orc_tol *tol, opt_ws *w,
                       orc_cand *rec, double *laws, double *cr_rows, int *n_cr_rows)
{
    const int m = d->m, p = d->p, ncp = d->ncp, n = d->n;
    const int P1 = p + 1;
    double *R = w->R, *Y = w->Y, *Lam = w->Lam, *G = w->G;
    rec->licq = 1;
    rec->optimal = 0; rec->region = 0;
    rec->t = NAN; rec->r = NAN;
    rec->lp2_status = ORC_SKIPPED; rec->cheb_status = ORC_SKIPPED;
    rec->lp2_pivots = 0; rec->cheb_pivots = 0;
    if (n_cr_rows) *n_cr_rows = 0;
    /* Cholesky of Wm[S,S] with the LICQ test */
    for (int b = 0; b < k; b++) {
        for (int a = 0; a < b; a++) {
            double acc = d->Wm[S[a] * m + S[b]];
            for (int l = 0; l < a; l++) acc = fma(-R[l * k + a], R[l * k + b], acc);
            R[a * k + b] = acc / R[a * k + a];
        }
        double acc = d->Wm[S[b] * m + S[b]];
        const double diag0 = acc;
        for (int l = 0; l < b; l++) acc = fma(-R[l * k + b], R[l * k + b], acc);
        if (!(acc > tol->tol_licq * diag0)) {
            rec->licq = 0;
            rec->lp2_status = ORC_LICQ_FAIL;
            return;
        }
        R[b * k + b] = sqrt(acc);
    }
    /* Y = R^-T [Wh_S | wc_S];  Lambda = R^-1 Y */
    for (int a = 0; a < k; a++) {
        for (int c = 0; c < P1; c++) {
            double acc = (c < p) ? d->Wh[S[a] * p + c] : d->wc[S[a]];
            for (int l = 0; l < a; l++) acc = fma(-R[l * k + a], Y[l * P1 + c], acc);
            Y[a * P1 + c] = acc / R[a * k + a];
        }
    }
    for (int a = k - 1; a >= 0; a--) {
        for (int c = 0; c < P1; c++) {
            double acc = Y[a * P1 + c];
            for (int l = a + 1; l < k; l++) acc = fma(-R[a * k + l], Lam[l * P1 + c], acc);
            Lam[a * P1 + c] = acc / R[a * k + a];
        }
    }
    /* mpLP: Lam is Gamma = Wm[S,S]^-1 [F_S | b_S] (x = A_S^T Gamma(theta));
     * the multipliers are lambda(theta) = -Psi(theta), Psi = Wm[S,S]^-1 [A_S H | A_S c] */
    const double *LamL = Lam;
    if (d->lp) {
        for (int a = 0; a < k; a++)
            for (int c = 0; c < P1; c++) w->Psi[a * P1 + c] = (c < p) ? d->WhL[S[a] * p + c] : d->wcL[S[a]];
        chol_solve_inplace(R, k, w->Psi, P1, P1);
        LamL = w->Psi;
    }
    /* region rows, reference order: lambda rows (S order), inactive rows
     * (ascending), parameter box rows */
    int row = 0;
    for (int a = 0; a < k; a++, row++) {
        for (int c = 0; c < p; c++) G[row * P1 + c] = LamL[a * P1 + c];
        G[row * P1 + p] = -LamL[a * P1 + p];
    }
    int si = 0;
    for (int i = 0; i < m; i++) {
        if (si < k && S[si] == i) { si++; continue; }
        for (int c = 0; c < p; c++) {
            double acc = -d->Wh[i * p + c];
            for (int l = 0; l < k; l++) acc = fma(d->Wm[i * m + S[l]], Lam[l * P1 + c], acc);
            G[row * P1 + c] = acc;
        }
        double acc = d->wc[i];
        for (int l = 0; l < k; l++) acc = fma(-d->Wm[i * m + S[l]], Lam[l * P1 + p], acc);
        G[row * P1 + p] = acc;
        row++;
    }
    for (int i = 0; i < ncp; i++, row++) {
        for (int c = 0; c < p; c++) G[row * P1 + c] = d->pr->At[i * p + c];
        G[row * P1 + p] = d->pr->bt[i];
    }
    const int nrows = m + ncp;
    if (d->lp && k < n) {
        /* no unique law x(theta): LP2 with a null-space direction; never a region */
        for (int a = 0; a < k; a++)
            for (int j = 0; j < n; j++) w->Phi[a * n + j] = d->QiAT[j * m + S[a]];
        chol_solve_inplace(R, k, w->Phi, n, n);
        lp2_short_mplp(d, S, k, tol, w, rec);
        return;
    }
    /* LP2: max t s.t. g theta + t <= h (constraint rows), At theta <= bt */
    double coef[256];
    double t0 = INFINITY;
    for (int r = 0; r < m; r++) { coef[r] = 1.0; if (G[r * P1 + p] < t0) t0 = G[r * P1 + p]; }
    for (int r = m; r < nrows; r++) coef[r] = 0.0;
    build_margin_lp(d, w, nrows, coef, t0);
    int piv = 0;
    rec->lp2_status = tucker_solve(w->T, d->ld2, nrows, P1, w->bid, w->nid, P1, tol, &piv);
    rec->lp2_pivots = piv;
    if (rec->lp2_status == ORC_OPTIMAL) {
        rec->t = -w->T[(size_t)nrows * d->ld2 + P1];
        rec->optimal = rec->t > tol->tol_opt;
    } else if (rec->lp2_status == ORC_UNBOUNDED) {
        rec->t = INFINITY;
    }
    if (!rec->optimal) return;
    /* Chebyshev ball: drop all-zero theta rows of the lambda / inactive
     * blocks, normalise, max r s.t. g theta + |g| r <= h (utils.py:45-86) */
    int nc = 0;
    for (int r = 0; r < nrows; r++) {
        const double *g = G + (size_t)r * P1;
        if (r < m) {
            /* utils.py:46-47 drops rows whose theta part is exactly zero; rows
             * that are zero in exact arithmetic come out as rounding noise,
             * so the test is relative: max|g| <= tol_zero_row * max(1, |h|) */
            double gmax = 0.0;
            for (int c = 0; c < p; c++) if (fabs(g[c]) > gmax) gmax = fabs(g[c]);
            const double ah = fabs(g[p]);
            if (!(gmax > tol->tol_zero_row * (ah > 1.0 ? ah : 1.0))) continue;
        }
        double acc = 0.0;
        for (int c = 0; c < p; c++) acc = fma(g[c], g[c], acc);
        const double inv = 1.0 / sqrt(acc);
        double *o = G + (size_t)nc * P1;   /* compact in place (nc <= r) */
        double nn = 0.0;
        for (int c = 0; c < p; c++) { o[c] = g[c] * inv; nn = fma(o[c], o[c], nn); }
        o[p] = g[p] * inv;
        coef[nc] = sqrt(nn);
        nc++;
    }
    double r0 = INFINITY;
    for (int r = 0; r < nc; r++) { const double v = G[r * P1 + p] / coef[r]; if (v < r0) r0 = v; }
    if (cr_rows) {
        memcpy(cr_rows, G, sizeof(double) * nc * P1);
        *n_cr_rows = nc;
    }
    build_margin_lp(d, w, nc, coef, r0);
    rec->cheb_status = tucker_solve(w->T, d->ld2, nc, P1, w->bid, w->nid, P1, tol, &piv);
    rec->cheb_pivots = piv;
    if (rec->cheb_status == ORC_OPTIMAL) {
        rec->r = -w->T[(size_t)nc * d->ld2 + P1];
        rec->region = rec->r >= tol->r_min;
    } else if (rec->cheb_status == ORC_UNBOUNDED) {
        rec->r = INFINITY;
    }
    if (laws && rec->region) {
        double *lA = laws, *lb = laws + k * p, *pA = lb + k, *pb = pA + n * p;
        for (int a = 0; a < k; a++) {
            for (int c = 0; c < p; c++) lA[a * p + c] = -LamL[a * P1 + c];
            lb[a] = -LamL[a * P1 + p];
        }
        for (int r = 0; r < n; r++) {
            for (int c = 0; c < p; c++) {
                double acc = -d->QiH[r * p + c];
                for (int l = 0; l < k; l++) acc = fma(d->QiAT[r * m + S[l]], Lam[l * P1 + c], acc);
                pA[r * p + c] = acc;
            }
            double acc = -d->Qic[r];
            for (int l = 0; l < k; l++) acc = fma(d->QiAT[r * m + S[l]], Lam[l * P1 + p], acc);
            pb[r] = acc;
        }
    }
}

/* ------------------------------------------------------------------ */
/* masks and the feasible-set hash                                      */
/* ------------------------------------------------------------------ */

static inline void mask_set(uint64_t *lo, uint64_t *hi, int j)
{
    if (j < 64) *lo |= (uint64_t)1 << j; else *hi |= (uint64_t)1 << (j - 64);
}

static int mask_to_set(uint64_t lo, uint64_t hi, int *S)
{
    int k = 0;
    for (int j = 0; j < 64; j++) if (lo >> j & 1) S[k++] = j;
    for (int j = 0; j < 64; j++) if (hi >> j & 1) S[k++] = 64 + j;
    return k;
}

typedef struct { uint64_t *lo, *hi; int32_t *val; uint64_t cap; } mhash;

static inline uint64_t mix64(uint64_t x)
{
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

static int mh_init(mhash *h, int64_t n)
{
    uint64_t cap = 16;
    while (cap < (uint64_t)(2 * n + 1)) cap <<= 1;
    h->cap = cap;
    h->lo = calloc(cap, 8); h->hi = calloc(cap, 8); h->val = malloc(cap * 4);
    if (!h->lo || !h->hi || !h->val) return ORC_ENOMEM;
    for (uint64_t i = 0; i < cap; i++) h->val[i] = -1;
    return 0;
}

static void mh_free(mhash *h) { free(h->lo); free(h->hi); free(h->val); }

static void mh_insert(mhash *h, uint64_t lo, uint64_t hi, int32_t v)
{
    uint64_t i = mix64(lo ^ mix64(hi)) & (h->cap - 1);
    while (h->val[i] >= 0) i = (i + 1) & (h->cap - 1);
    h->lo[i] = lo; h->hi[i] = hi; h->val[i] = v;
}

static int32_t mh_find(const mhash *h, uint64_t lo, uint64_t hi)
{
    uint64_t i = mix64(lo ^ mix64(hi)) & (h->cap - 1);
    while (h->val[i] >= 0) {
        if (h->lo[i] == lo && h->hi[i] == hi) return h->val[i];
        i = (i + 1) & (h->cap - 1);
    }
    return -1;
}

/* ------------------------------------------------------------------ */
/* enumeration                                                          */
/* ------------------------------------------------------------------ */

typedef struct {
    const orc_data *d;
    const orc_tol *tol;
    int k, do_opt;
    /* LP1 phase */
    const double *parT; const uint8_t *parB, *parN;
    const int32_t *cpar, *cj;
    double *candT; uint8_t *candB, *candN;
    orc_cand *rec;
    int64_t ncand;
    /* optimality phase */
    const int64_t *feas_idx;
    int64_t nfeas;
    volatile int64_t next;
} job_t;

static void *lp1_worker(void *arg)
{
    job_t *jb = arg;
    const orc_data *d = jb->d;
    const size_t tsz = (size_t)(d->M1 + 1) * d->ld1;
    for (;;) {
        const int64_t i = __atomic_fetch_add(&jb->next, 1, __ATOMIC_RELAXED);
        if (i >= jb->ncand) break;
        lp1_state par = { (double *)jb->parT + (size_t)jb->cpar[i] * tsz,
                          (uint8_t *)jb->parB + (size_t)jb->cpar[i] * d->M1,
                          (uint8_t *)jb->parN + (size_t)jb->cpar[i] * d->nv };
        lp1_state s = { jb->candT + (size_t)i * tsz, jb->candB + (size_t)i * d->M1,
                        jb->candN + (size_t)i * d->nv };
        int st, pv; double z;
        lp1_child(d, &par, jb->cj[i], &s, jb->tol, &st, &pv, &z);
        orc_cand *r = &jb->rec[i];
        r->lp1_status = st; r->lp1_pivots = pv; r->z = z;
        r->feasible = (st == ORC_OPTIMAL) && (z <= jb->tol->tol_feas);
    }
    return NULL;
}

static void *opt_worker(void *arg)
{
    job_t *jb = arg;
    const orc_data *d = jb->d;
    opt_ws w;
    opt_ws_alloc(d, &w);
    int S[128];
    for (;;) {
        const int64_t i = __atomic_fetch_add(&jb->next, 1, __ATOMIC_RELAXED);
        if (i >= jb->nfeas) break;
        orc_cand *r = &jb->rec[jb->feas_idx[i]];
        const int k = mask_to_set(r->mask_lo, r->mask_hi, S);
        optimality(d, S, k, jb->tol, &w, r, NULL, NULL, NULL);
    }
    opt_ws_free(&w);
    return NULL;
}

static void run_pool(void *(*fn)(void *), job_t *jb, int nthreads)
{
    jb->next = 0;
    if (nthreads <= 1) { fn(jb); return; }
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, fn, jb);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

static void rec_init(orc_cand *r)
{
    memset(r, 0, sizeof(*r));
    r->t = NAN; r->r = NAN;
    r->lp2_status = ORC_SKIPPED; r->cheb_status = ORC_SKIPPED;
}

/* LP1 tableaus computed per pass of the level loop (candidates) */
#define ORC_CHUNK 65536

/* parents of one level: tableaus, basis ids and masks, grown on demand */
typedef struct {
    double *T; uint8_t *B, *N; uint64_t *lo, *hi;
    int64_t n, cap;
} parent_list;

static void pl_free(parent_list *l)
{
    free(l->T); free(l->B); free(l->N); free(l->lo); free(l->hi);
    memset(l, 0, sizeof(*l));
}

static int pl_reserve(parent_list *l, int64_t cap, size_t tsz, int M1, int nv)
{
    if (cap <= l->cap) return 0;
    double *T = realloc(l->T, (size_t)cap * tsz * sizeof(double));
    if (T) l->T = T;
    uint8_t *B = realloc(l->B, (size_t)cap * M1);
    if (B) l->B = B;
    uint8_t *N = realloc(l->N, (size_t)cap * nv);
    if (N) l->N = N;
    uint64_t *lo = realloc(l->lo, (size_t)cap * 8);
    if (lo) l->lo = lo;
    uint64_t *hi = realloc(l->hi, (size_t)cap * 8);
    if (hi) l->hi = hi;
    if (!T || !B || !N || !lo || !hi) return ORC_ENOMEM;
    l->cap = cap;
    return 0;
}

/* j_first > 0: only the sets whose elements are all >= j_first (a family
 * closed under subsets, so the subset test is the full enumeration's) */
static int enumerate_impl(const orc_problem *pr, const orc_tol *tol, int k_min, int k_max, int64_t budget,
                          int exhaustive, int nthreads, int keep_records, int j_first, orc_result *out)
{
    memset(out, 0, sizeof(*out));
    orc_data d;
    int rc = prepare(pr, &d);
    if (rc) return rc;
    if (k_max > d.m) k_max = d.m;
    if (k_min < 0) k_min = 0;
    const size_t tsz = (size_t)(d.M1 + 1) * d.ld1;
    /* everything the level loop owns, freed on every exit */
    parent_list F = {0}, NF = {0};
    int64_t cap_rec = 1024, n_rec = 0;
    orc_cand *recs = NULL, *crec = NULL;
    int32_t *cpar = NULL, *cj = NULL;
    double *CT = NULL;
    uint8_t *CB = NULL, *CN = NULL;
    int64_t *fidx = NULL;
    mhash h = {0};
    /* level 0: the empty set */
    if ((rc = pl_reserve(&F, 1, tsz, d.M1, d.nv))) goto done;
    {
        lp1_state s = { F.T, F.B, F.N };
        lp1_init_root(&d, &s);
        F.lo[0] = 0; F.hi[0] = 0; F.n = 1;
    }
    if (keep_records && !(recs = malloc(cap_rec * sizeof(orc_cand)))) { rc = ORC_ENOMEM; goto done; }
    {
        orc_cand r0;
        rec_init(&r0);
        r0.parent = -1;
        r0.feasible = 1;
        r0.lp1_status = ORC_OPTIMAL;
        if (k_min <= 0) {
            opt_ws w; opt_ws_alloc(&d, &w);
            optimality(&d, NULL, 0, tol, &w, &r0, NULL, NULL, NULL);
            opt_ws_free(&w);
        }
        out->n_cand = 1; out->n_feasible = 1;
        out->n_optimal += r0.optimal; out->n_region += r0.region;
        out->n_lp2_pivots += r0.lp2_pivots; out->n_cheb_pivots += r0.cheb_pivots;
        if (keep_records) recs[n_rec++] = r0;
    }
    out->n_levels = 1;
    int S[128];
    for (int k = 1; k <= k_max && F.n > 0; k++) {
        if ((rc = mh_init(&h, F.n))) goto done;
        for (int64_t i = 0; i < F.n; i++) mh_insert(&h, F.lo[i], F.hi[i], (int32_t)i);
        /* candidates */
        int64_t ccap = 1024, nc = 0;
        cpar = malloc(ccap * 4); cj = malloc(ccap * 4);
        if (!cpar || !cj) { rc = ORC_ENOMEM; goto done; }
        for (int64_t pi = 0; pi < F.n; pi++) {
            const int kp = mask_to_set(F.lo[pi], F.hi[pi], S);
            const int jmin = kp ? S[kp - 1] + 1 : (j_first > 0 ? j_first : 0);
            for (int j = jmin; j < d.m; j++) {
                int ok = 1;
                for (int a = 0; a < kp && ok && !exhaustive; a++) {
                    uint64_t lo = F.lo[pi], hi = F.hi[pi];
                    /* S + {j} - {S[a]} */
                    if (S[a] < 64) lo &= ~((uint64_t)1 << S[a]); else hi &= ~((uint64_t)1 << (S[a] - 64));
                    mask_set(&lo, &hi, j);
                    if (mh_find(&h, lo, hi) < 0) ok = 0;
                }
                if (!ok) { out->n_pruned++; continue; }
                if (nc == ccap) {
                    ccap *= 2;
                    int32_t *a = realloc(cpar, ccap * 4);
                    if (a) cpar = a;
                    int32_t *b = realloc(cj, ccap * 4);
                    if (b) cj = b;
                    if (!a || !b) { rc = ORC_ENOMEM; goto done; }
                }
                cpar[nc] = (int32_t)pi; cj[nc] = j; nc++;
            }
        }
        mh_free(&h);
        memset(&h, 0, sizeof(h));
        if (nc == 0) break;
        if (budget > 0 && out->n_cand + nc > budget) {
            out->truncated = 1;
            break;
        }
        out->n_levels = k + 1;
        /* children of the deepest level are nobody's parents */
        const int keep_children = exhaustive || k < k_max;
        const int64_t chunk = nc < ORC_CHUNK ? nc : ORC_CHUNK;
        crec = malloc(nc * sizeof(orc_cand));
        CT = malloc(chunk * tsz * sizeof(double));
        CB = malloc(chunk * d.M1); CN = malloc(chunk * d.nv);
        if (!crec || !CT || !CB || !CN) { rc = ORC_ENOMEM; goto done; }
        for (int64_t i = 0; i < nc; i++) {
            rec_init(&crec[i]);
            crec[i].mask_lo = F.lo[cpar[i]]; crec[i].mask_hi = F.hi[cpar[i]];
            mask_set(&crec[i].mask_lo, &crec[i].mask_hi, cj[i]);
            crec[i].level = k; crec[i].parent = cpar[i];
        }
        job_t jb;
        memset(&jb, 0, sizeof(jb));
        jb.d = &d; jb.tol = tol; jb.k = k;
        jb.parT = F.T; jb.parB = F.B; jb.parN = F.N;
        jb.candT = CT; jb.candB = CB; jb.candN = CN;
        /* LP1 chunk by chunk; the kept children in candidate (lexicographic) order */
        for (int64_t c0 = 0; c0 < nc; c0 += chunk) {
            const int64_t n = nc - c0 < chunk ? nc - c0 : chunk;
            jb.cpar = cpar + c0; jb.cj = cj + c0; jb.rec = crec + c0; jb.ncand = n;
            run_pool(lp1_worker, &jb, nthreads);
            if (!keep_children) continue;
            for (int64_t i = 0; i < n; i++) {
                const orc_cand *r = &crec[c0 + i];
                if (!r->feasible && !exhaustive) continue;
                if (NF.n == NF.cap && (rc = pl_reserve(&NF, NF.cap ? 2 * NF.cap : 1024, tsz, d.M1, d.nv))) goto done;
                memcpy(NF.T + NF.n * tsz, CT + i * tsz, tsz * sizeof(double));
                memcpy(NF.B + NF.n * d.M1, CB + i * d.M1, d.M1);
                memcpy(NF.N + NF.n * d.nv, CN + i * d.nv, d.nv);
                NF.lo[NF.n] = r->mask_lo; NF.hi[NF.n] = r->mask_hi;
                NF.n++;
            }
        }
        free(CT); free(CB); free(CN);
        CT = NULL; CB = NULL; CN = NULL;
        int64_t nfn = 0;
        for (int64_t i = 0; i < nc; i++) { nfn += crec[i].feasible; out->n_lp1_pivots += crec[i].lp1_pivots; }
        if (!(fidx = malloc((nfn ? nfn : 1) * sizeof(int64_t)))) { rc = ORC_ENOMEM; goto done; }
        for (int64_t i = 0, f = 0; i < nc; i++) if (crec[i].feasible) fidx[f++] = i;
        if (k >= k_min && nfn > 0) {
            jb.rec = crec; jb.feas_idx = fidx; jb.nfeas = nfn;
            run_pool(opt_worker, &jb, nthreads);
        }
        for (int64_t i = 0; i < nc; i++) {
            out->n_feasible += crec[i].feasible;
            out->n_optimal += crec[i].optimal;
            out->n_region += crec[i].region;
            out->n_lp2_pivots += crec[i].lp2_pivots;
            out->n_cheb_pivots += crec[i].cheb_pivots;
        }
        out->n_cand += nc;
        if (keep_records) {
            if (n_rec + nc > cap_rec) {
                while (n_rec + nc > cap_rec) cap_rec *= 2;
                orc_cand *rr = realloc(recs, cap_rec * sizeof(orc_cand));
                if (!rr) { rc = ORC_ENOMEM; goto done; }
                recs = rr;
            }
            memcpy(recs + n_rec, crec, nc * sizeof(orc_cand));
            n_rec += nc;
        }
        free(crec); free(cpar); free(cj); free(fidx);
        crec = NULL; cpar = NULL; cj = NULL; fidx = NULL;
        pl_free(&F);
        F = NF;
        memset(&NF, 0, sizeof(NF));
    }
done:
    mh_free(&h);
    free(crec); free(cpar); free(cj); free(fidx); free(CT); free(CB); free(CN);
    pl_free(&F); pl_free(&NF);
    free_data(&d);
    if (rc) {
        free(recs);
        memset(out, 0, sizeof(*out));
        return rc;
    }
    out->cand = recs;
    return 0;
}

int orc_enumerate(const orc_problem *pr, const orc_tol *tol, int k_min, int k_max,
                  int64_t budget, int exhaustive, int nthreads, int keep_records, orc_result *out)
{
    return enumerate_impl(pr, tol, k_min, k_max, budget, exhaustive, nthreads, keep_records, 0, out);
}

int orc_enumerate_tail(const orc_problem *pr, const orc_tol *tol, int k_min, int k_max, int64_t budget,
                       int nthreads, int j_first, orc_result *out)
{
    return enumerate_impl(pr, tol, k_min, k_max, budget, 0, nthreads, 0, j_first, out);
}

void orc_free_result(orc_result *res)
{
    free(res->cand);
    res->cand = NULL;
}

/* Dual certificate of LP1 infeasibility from a final basis.  LP1 of a set T
 * is  min c.w  s.t.  G u + w = beta, w >= 0, u free  (c = 1 on T, 0 elsewhere),
 * whose dual is  max beta.y  s.t.  G^T y = 0, y <= c; every such y gives
 * z*(T) >= beta.y.  The final basis fixes y_i = c_i on the rows whose slack is
 * basic; with every free variable basic, the duals of the nv nonbasic slacks
 * solve the square system  G_N^T y_N = -G_B^T c_B  (Gaussian elimination with
 * partial pivoting).  Returns 1 with *bound = beta.y when that y meets
 * y <= c + sign_tol, else 0.  (Not part of the reference's algorithm: the
 * checker for a certificate built from FP32 bases.) */
static int lp1_basis_bound(const orc_data *d, const lp1_state *s, const int *T, int k, double sign_tol,
                           double *bound)
{
    const int nv = d->nv, M1 = d->M1, ld = d->ld1;
    for (int c = 0; c < nv; c++) if (s->nid[c] < nv) return 0;     /* a free variable nonbasic */
    double *cost = calloc((size_t)M1, sizeof(double));
    double *y = calloc((size_t)M1, sizeof(double));
    double *M = malloc(sizeof(double) * (size_t)nv * (nv + 1));     /* [G_N^T | rhs] */
    for (int a = 0; a < k; a++) cost[T[a]] = 1.0;
    for (int r = 0; r < M1; r++) {
        const int i = s->bid[r] - nv;
        if (i >= 0) y[i] = cost[i];
    }
    for (int v = 0; v < nv; v++) {
        double rhs = 0.0;
        for (int r = 0; r < M1; r++) {
            const int i = s->bid[r] - nv;
            if (i >= 0 && cost[i] != 0.0) rhs -= d->root[(size_t)i * ld + v] * cost[i];
        }
        for (int c = 0; c < nv; c++) M[(size_t)v * (nv + 1) + c] = d->root[(size_t)(s->nid[c] - nv) * ld + v];
        M[(size_t)v * (nv + 1) + nv] = rhs;
    }
    int ok = 1;
    for (int col = 0; col < nv && ok; col++) {
        int piv = col;
        double best = fabs(M[(size_t)col * (nv + 1) + col]), scale = 0.0;
        for (int r = col; r < nv; r++) {
            const double a = fabs(M[(size_t)r * (nv + 1) + col]);
            if (a > best) { best = a; piv = r; }
            if (a > scale) scale = a;
        }
        if (!(best > 1e-13 * (scale > 1.0 ? scale : 1.0))) { ok = 0; break; }
        if (piv != col)
            for (int c = 0; c <= nv; c++) {
                const double t = M[(size_t)col * (nv + 1) + c];
                M[(size_t)col * (nv + 1) + c] = M[(size_t)piv * (nv + 1) + c];
                M[(size_t)piv * (nv + 1) + c] = t;
            }
        for (int r = col + 1; r < nv; r++) {
            const double f = M[(size_t)r * (nv + 1) + col] / M[(size_t)col * (nv + 1) + col];
            for (int c = col; c <= nv; c++) M[(size_t)r * (nv + 1) + c] -= f * M[(size_t)col * (nv + 1) + c];
        }
    }
    if (ok) {
        for (int r = nv - 1; r >= 0; r--) {
            double acc = M[(size_t)r * (nv + 1) + nv];
            for (int c = r + 1; c < nv; c++) acc -= M[(size_t)r * (nv + 1) + c] * y[s->nid[c] - nv];
            y[s->nid[r] - nv] = acc / M[(size_t)r * (nv + 1) + r];
        }
        double b = 0.0;
        for (int i = 0; i < M1 && ok; i++) {
            if (y[i] > cost[i] + sign_tol) ok = 0;
            b += d->root[(size_t)i * ld + nv] * y[i];
        }
        *bound = b;
    }
    free(cost); free(y); free(M);
    return ok;
}

int orc_lp1_dual_bound(const orc_problem *pr, const orc_tol *tol, const int *S, int k, double sign_tol,
                       double *bound, double *z_out, int *k_used)
{
    orc_data d;
    int rc = prepare(pr, &d);
    if (rc) return rc;
    for (int a = 1; a < k; a++) if (S[a] <= S[a - 1]) { free_data(&d); return -4; }
    if (k > 0 && (S[0] < 0 || S[k - 1] >= d.m)) { free_data(&d); return -4; }
    const size_t tsz = (size_t)(d.M1 + 1) * d.ld1;
    lp1_state a = { malloc(tsz * 8), malloc(d.M1), malloc(d.nv) };
    lp1_state b = { malloc(tsz * 8), malloc(d.M1), malloc(d.nv) };
    lp1_init_root(&d, &a);
    /* the warm-start chain of the prefixes, up to the first infeasible one
       (whose bound also bounds every superset) */
    int used = 0, status = ORC_OPTIMAL;
    double z = 0.0;
    for (int i = 0; i < k; i++) {
        int pv;
        lp1_child(&d, &a, S[i], &b, tol, &status, &pv, &z);
        lp1_state t = a; a = b; b = t;
        used = i + 1;
        if (!(status == ORC_OPTIMAL && z <= tol->tol_feas)) break;
    }
    int got = 0;
    *bound = 0.0;
    if (status == ORC_OPTIMAL) got = lp1_basis_bound(&d, &a, S, used, sign_tol, bound);
    *z_out = z;
    *k_used = used;
    free(a.T); free(a.bid); free(a.nid); free(b.T); free(b.bid); free(b.nid);
    free_data(&d);
    return got;
}

int orc_check_set(const orc_problem *pr, const orc_tol *tol, const int *S, int k,
                  orc_cand *rec, double *laws, double *cr_rows, int *n_cr_rows)
{
    orc_data d;
    int rc = prepare(pr, &d);
    if (rc) return rc;
    for (int a = 1; a < k; a++) if (S[a] <= S[a - 1]) { free_data(&d); return -4; }
    if (k > 0 && (S[0] < 0 || S[k - 1] >= d.m)) { free_data(&d); return -4; }
    const size_t tsz = (size_t)(d.M1 + 1) * d.ld1;
    lp1_state a = { malloc(tsz * 8), malloc(d.M1), malloc(d.nv) };
    lp1_state b = { malloc(tsz * 8), malloc(d.M1), malloc(d.nv) };
    lp1_init_root(&d, &a);
    rec_init(rec);
    rec->level = k;
    rec->parent = -1;
    rec->feasible = 1;
    rec->lp1_status = ORC_OPTIMAL;
    for (int i = 0; i < k; i++) mask_set(&rec->mask_lo, &rec->mask_hi, S[i]);
    for (int i = 0; i < k; i++) {
        int st, pv; double z;
        lp1_child(&d, &a, S[i], &b, tol, &st, &pv, &z);
        rec->lp1_status = st; rec->lp1_pivots = pv; rec->z = z;
        rec->feasible = (st == ORC_OPTIMAL) && (z <= tol->tol_feas);
        lp1_state t = a; a = b; b = t;
        if (!rec->feasible) break;
    }
    if (rec->feasible) {
        opt_ws w; opt_ws_alloc(&d, &w);
        optimality(&d, S, k, tol, &w, rec, laws, cr_rows, n_cr_rows);
        opt_ws_free(&w);
    }
    free(a.T); free(a.bid); free(a.nid); free(b.T); free(b.bid); free(b.nid);
    free_data(&d);
    return 0;
}
