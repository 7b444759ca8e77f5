/*
 * gw_oracle.c -- CPU restatement of DPFEHM's groundwater solve, used ONLY as the
 * checker (tests, the smoke check, and the timed CPU baseline in bench.py).
 * Nothing in the shipped library links or calls this file.
 *
 * Parity status: the reference is Julia and cannot run in this environment, and
 * its tests hold no golden vectors. This restatement is pinned against the
 * reference's own analytic known-answer checks (Thiem, Theis; test/thiem.jl:10-12,
 * test/theis.jl:12-21) and against an independent direct solve (scipy spsolve)
 * on small grids; 1e-8 parity against the Julia package itself is unpinned.
 *
 * What it restates (reference paths are relative to the DPFEHM.jl project):
 *   - getfreenodes                      src/utilities.jl:10-24
 *   - groundwater residual / Jacobian   src/groundwater.jl:1-21 (macro body), :38
 *   - steady solve, S = V = 1           src/groundwater.jl:75-83
 *   - rrule pullback tangents           src/groundwater.jl:85-107
 *   - Ruge-Stueben AMG (classical strength theta=0.25, RS first-pass C/F
 *     splitting, direct interpolation, Galerkin RAP, Gauss-Seidel smoothing)
 *     as called at src/groundwater.jl:46-47,90-91,95-96; the package
 *     (AlgebraicMultigrid.jl 0.5.0, Manifest.toml:19-23) is not vendored, so the
 *     published Ruge-Stueben algorithm is restated here. The solve is AMG-
 *     preconditioned CG (the AMG+CG form of
 *     examples/fracture_network_solver_scaling/porous_media_comparison.jl:12-16).
 *   - face means: geometric exp(0.5(logKa+logKb))
 *     (examples/gw_steadystate_3d/inputdeck.jl:51) and harmonic 2/(1/Ka+1/Kb)
 *     (src/richards.jl:50-52), with their vector-Jacobian products.
 *   - transient: fixed-step backward Euler of dh/dt = -R(h) with the
 *     specificstorage*volumes scaling of src/groundwater.jl:7,15,17, and its
 *     discrete adjoint.
 *
 * Threads: OpenMP parallelises SpMV, vector ops and RAP; the Gauss-Seidel
 * smoother runs as per-thread blocks ("hybrid" GS) when more than one thread is
 * used, and as the exact sequential sweep with one thread.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_BAD_INPUT 1
#define ORC_NOT_CONVERGED 2
#define ORC_OOM 3
#define ORC_BREAKDOWN 4

static int g_threads = 1;

void orc_set_threads(int n) {
    g_threads = n < 1 ? 1 : n;
#ifdef _OPENMP
    omp_set_num_threads(g_threads);
#endif
}
int orc_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------ CSR */
typedef struct {
    int64_t n, m;   /* rows, cols */
    int64_t *rp;    /* n+1 */
    int32_t *ci;    /* nnz */
    double *v;      /* nnz */
} csr_t;

static void csr_free(csr_t *A) {
    if (!A) return;
    free(A->rp); free(A->ci); free(A->v);
    memset(A, 0, sizeof(*A));
}

static void spmv(const csr_t *A, const double *x, double *y) {
    int64_t n = A->n;
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (int64_t i = 0; i < n; i++) {
        double s = 0.0;
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) s += A->v[k] * x[A->ci[k]];
        y[i] = s;
    }
}

/* y = b - A x */
static void residual(const csr_t *A, const double *b, const double *x, double *y) {
    int64_t n = A->n;
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (int64_t i = 0; i < n; i++) {
        double s = b[i];
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) s -= A->v[k] * x[A->ci[k]];
        y[i] = s;
    }
}

static double dot(int64_t n, const double *a, const double *b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static) if (g_threads > 1)
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* sort each row by column and merge duplicate entries (summing values) */
static void csr_sort_merge(csr_t *A) {
    int64_t n = A->n;
    int64_t *newrp = (int64_t *)malloc((n + 1) * sizeof(int64_t));
    /* in-place per-row insertion sort, then compaction */
    for (int64_t i = 0; i < n; i++) {
        int64_t s = A->rp[i], e = A->rp[i + 1];
        for (int64_t k = s + 1; k < e; k++) {
            int32_t c = A->ci[k]; double v = A->v[k]; int64_t j = k - 1;
            while (j >= s && A->ci[j] > c) { A->ci[j + 1] = A->ci[j]; A->v[j + 1] = A->v[j]; j--; }
            A->ci[j + 1] = c; A->v[j + 1] = v;
        }
    }
    int64_t w = 0;
    newrp[0] = 0;
    for (int64_t i = 0; i < n; i++) {
        int64_t s = A->rp[i], e = A->rp[i + 1];
        int64_t rowstart = w;
        for (int64_t k = s; k < e; k++) {
            if (w > rowstart && A->ci[w - 1] == A->ci[k]) A->v[w - 1] += A->v[k];
            else { A->ci[w] = A->ci[k]; A->v[w] = A->v[k]; w++; }
        }
        newrp[i + 1] = w;
    }
    free(A->rp);
    A->rp = newrp;
}

static void csr_transpose(const csr_t *A, csr_t *T) {
    int64_t n = A->n, m = A->m, nnz = A->rp[n];
    T->n = m; T->m = n;
    T->rp = (int64_t *)calloc(m + 1, sizeof(int64_t));
    T->ci = (int32_t *)malloc((nnz > 0 ? nnz : 1) * sizeof(int32_t));
    T->v = (double *)malloc((nnz > 0 ? nnz : 1) * sizeof(double));
    for (int64_t k = 0; k < nnz; k++) T->rp[A->ci[k] + 1]++;
    for (int64_t j = 0; j < m; j++) T->rp[j + 1] += T->rp[j];
    int64_t *pos = (int64_t *)malloc((m > 0 ? m : 1) * sizeof(int64_t));
    memcpy(pos, T->rp, m * sizeof(int64_t));
    for (int64_t i = 0; i < n; i++)
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) {
            int64_t p = pos[A->ci[k]]++;
            T->ci[p] = (int32_t)i; T->v[p] = A->v[k];
        }
    free(pos);
}

/* C = A * B (Gustavson, two passes, rows in parallel) */
static void spgemm(const csr_t *A, const csr_t *B, csr_t *C) {
    int64_t n = A->n, m = B->m;
    C->n = n; C->m = m;
    C->rp = (int64_t *)calloc(n + 1, sizeof(int64_t));
#pragma omp parallel if (g_threads > 1)
    {
        int64_t *mark = (int64_t *)malloc((m > 0 ? m : 1) * sizeof(int64_t));
        for (int64_t j = 0; j < m; j++) mark[j] = -1;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; i++) {
            int64_t cnt = 0;
            for (int64_t ka = A->rp[i]; ka < A->rp[i + 1]; ka++) {
                int32_t k = A->ci[ka];
                for (int64_t kb = B->rp[k]; kb < B->rp[k + 1]; kb++) {
                    int32_t j = B->ci[kb];
                    if (mark[j] != i) { mark[j] = i; cnt++; }
                }
            }
            C->rp[i + 1] = cnt;
        }
        free(mark);
    }
    for (int64_t i = 0; i < n; i++) C->rp[i + 1] += C->rp[i];
    int64_t nnz = C->rp[n];
    C->ci = (int32_t *)malloc((nnz > 0 ? nnz : 1) * sizeof(int32_t));
    C->v = (double *)malloc((nnz > 0 ? nnz : 1) * sizeof(double));
#pragma omp parallel if (g_threads > 1)
    {
        int64_t *pos = (int64_t *)malloc((m > 0 ? m : 1) * sizeof(int64_t));
        for (int64_t j = 0; j < m; j++) pos[j] = -1;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; i++) {
            int64_t w = C->rp[i], s = w;
            for (int64_t ka = A->rp[i]; ka < A->rp[i + 1]; ka++) {
                int32_t k = A->ci[ka]; double av = A->v[ka];
                for (int64_t kb = B->rp[k]; kb < B->rp[k + 1]; kb++) {
                    int32_t j = B->ci[kb];
                    if (pos[j] < s) { pos[j] = w; C->ci[w] = j; C->v[w] = av * B->v[kb]; w++; }
                    else C->v[pos[j]] += av * B->v[kb];
                }
            }
        }
        free(pos);
    }
    csr_sort_merge(C);
}

/* ------------------------------------------------- Ruge-Stueben AMG setup */
typedef struct {
    csr_t A, P, R;    /* R = P^T */
    double *diag;
    double *x, *b, *r; /* work vectors */
    int64_t n;
} level_t;

typedef struct {
    int nlev;
    level_t lev[40];
    double *coarse_L; /* dense Cholesky factor of the coarsest operator (row-major lower) */
    int64_t nc;
} amg_t;

#define RS_F 0
#define RS_C 1
#define RS_U 2

/* classical strength: j strongly influences i if -a_ij >= theta * max_k (-a_ik), k != i */
static void classical_strength(const csr_t *A, double theta, csr_t *S) {
    int64_t n = A->n;
    S->n = n; S->m = n;
    S->rp = (int64_t *)calloc(n + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) {
        double mx = 0.0;
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++)
            if (A->ci[k] != i && -A->v[k] > mx) mx = -A->v[k];
        int64_t c = 0;
        if (mx > 0.0)
            for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++)
                if (A->ci[k] != i && -A->v[k] >= theta * mx) c++;
        S->rp[i + 1] = S->rp[i] + c;
    }
    int64_t nnz = S->rp[n];
    S->ci = (int32_t *)malloc((nnz > 0 ? nnz : 1) * sizeof(int32_t));
    S->v = (double *)malloc((nnz > 0 ? nnz : 1) * sizeof(double));
    for (int64_t i = 0; i < n; i++) {
        double mx = 0.0;
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++)
            if (A->ci[k] != i && -A->v[k] > mx) mx = -A->v[k];
        int64_t w = S->rp[i];
        if (mx > 0.0)
            for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++)
                if (A->ci[k] != i && -A->v[k] >= theta * mx) { S->ci[w] = A->ci[k]; S->v[w] = A->v[k]; w++; }
    }
}

/* binary max-heap keyed on (lambda, -index) with lazy deletion */
typedef struct { int64_t key; int32_t node; } hent_t;
typedef struct { hent_t *a; int64_t n, cap; } heap_t;
static int hgt(hent_t x, hent_t y) { return x.key > y.key || (x.key == y.key && x.node < y.node); }
static void hpush(heap_t *h, int64_t key, int32_t node) {
    if (h->n == h->cap) { h->cap = h->cap ? 2 * h->cap : 1024; h->a = (hent_t *)realloc(h->a, h->cap * sizeof(hent_t)); }
    int64_t i = h->n++;
    h->a[i].key = key; h->a[i].node = node;
    while (i > 0) {
        int64_t p = (i - 1) / 2;
        if (!hgt(h->a[i], h->a[p])) break;
        hent_t t = h->a[i]; h->a[i] = h->a[p]; h->a[p] = t; i = p;
    }
}
static hent_t hpop(heap_t *h) {
    hent_t top = h->a[0];
    h->a[0] = h->a[--h->n];
    int64_t i = 0;
    for (;;) {
        int64_t l = 2 * i + 1, r = l + 1, b = i;
        if (l < h->n && hgt(h->a[l], h->a[b])) b = l;
        if (r < h->n && hgt(h->a[r], h->a[b])) b = r;
        if (b == i) break;
        hent_t t = h->a[i]; h->a[i] = h->a[b]; h->a[b] = t; i = b;
    }
    return top;
}

/* RS first pass: repeatedly make the unassigned point with the largest measure
 * lambda (number of unassigned/F points it strongly influences) a C point, the
 * points strongly depending on it F points, and raise the measure of the new F
 * points' other strong connections. Points with no strong connections at all
 * become F points. */
static void rs_splitting(const csr_t *S, const csr_t *ST, int8_t *split) {
    int64_t n = S->n;
    int64_t *lam = (int64_t *)malloc((n > 0 ? n : 1) * sizeof(int64_t));
    heap_t h = {0};
    for (int64_t i = 0; i < n; i++) {
        lam[i] = ST->rp[i + 1] - ST->rp[i];
        if (lam[i] == 0 && S->rp[i + 1] == S->rp[i]) split[i] = RS_F;
        else { split[i] = RS_U; hpush(&h, lam[i], (int32_t)i); }
    }
    while (h.n > 0) {
        hent_t t = hpop(&h);
        int64_t i = t.node;
        if (split[i] != RS_U || t.key != lam[i]) continue;
        split[i] = RS_C;
        for (int64_t k = ST->rp[i]; k < ST->rp[i + 1]; k++) {
            int64_t j = ST->ci[k];
            if (split[j] != RS_U) continue;
            split[j] = RS_F;
            for (int64_t kk = S->rp[j]; kk < S->rp[j + 1]; kk++) {
                int64_t m = S->ci[kk];
                if (split[m] == RS_U) { lam[m]++; hpush(&h, lam[m], (int32_t)m); }
            }
        }
        for (int64_t k = S->rp[i]; k < S->rp[i + 1]; k++) {
            int64_t j = S->ci[k];
            if (split[j] == RS_U && lam[j] > 0) { lam[j]--; hpush(&h, lam[j], (int32_t)j); }
        }
    }
    free(lam); free(h.a);
}

/* direct interpolation: for an F point i,
 *   P_ij = -alpha * a_ij / a_ii (a_ij < 0), -beta * a_ij / a_ii (a_ij > 0), j in C cap S_i
 * with alpha = sum_{k != i, a_ik<0} a_ik / sum_{j in C cap S_i, a_ij<0} a_ij and beta likewise
 * for positive entries (if no strong positive C entry, positive entries are lumped to the diagonal). */
static int direct_interpolation(const csr_t *A, const csr_t *S, const int8_t *split, csr_t *P) {
    int64_t n = A->n;
    int32_t *cidx = (int32_t *)malloc((n > 0 ? n : 1) * sizeof(int32_t));
    int64_t nc = 0;
    for (int64_t i = 0; i < n; i++) cidx[i] = split[i] == RS_C ? (int32_t)nc++ : -1;
    P->n = n; P->m = nc;
    P->rp = (int64_t *)calloc(n + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) {
        if (split[i] == RS_C) { P->rp[i + 1] = 1; continue; }
        int64_t c = 0;
        for (int64_t k = S->rp[i]; k < S->rp[i + 1]; k++) if (split[S->ci[k]] == RS_C) c++;
        P->rp[i + 1] = c;
    }
    for (int64_t i = 0; i < n; i++) P->rp[i + 1] += P->rp[i];
    int64_t nnz = P->rp[n];
    P->ci = (int32_t *)malloc((nnz > 0 ? nnz : 1) * sizeof(int32_t));
    P->v = (double *)malloc((nnz > 0 ? nnz : 1) * sizeof(double));
    int bad = 0;
    for (int64_t i = 0; i < n; i++) {
        int64_t w = P->rp[i];
        if (split[i] == RS_C) { P->ci[w] = cidx[i]; P->v[w] = 1.0; continue; }
        double aii = 0.0, sum_neg = 0.0, sum_pos = 0.0, sn_strong = 0.0, sp_strong = 0.0;
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) {
            int32_t j = A->ci[k]; double a = A->v[k];
            if (j == i) { aii += a; continue; }
            if (a < 0) sum_neg += a; else sum_pos += a;
        }
        for (int64_t k = S->rp[i]; k < S->rp[i + 1]; k++) {
            int32_t j = S->ci[k]; double a = S->v[k];
            if (split[j] != RS_C) continue;
            if (a < 0) sn_strong += a; else sp_strong += a;
        }
        double alpha = sn_strong != 0.0 ? sum_neg / sn_strong : 0.0;
        double beta = 0.0;
        if (sp_strong != 0.0) beta = sum_pos / sp_strong;
        else aii += sum_pos;
        if (P->rp[i + 1] == P->rp[i]) continue;
        if (aii == 0.0) { bad = 1; aii = 1.0; }
        for (int64_t k = S->rp[i]; k < S->rp[i + 1]; k++) {
            int32_t j = S->ci[k]; double a = S->v[k];
            if (split[j] != RS_C) continue;
            P->ci[w] = cidx[j];
            P->v[w] = (a < 0 ? -alpha : -beta) * a / aii;
            w++;
        }
    }
    free(cidx);
    return bad ? ORC_BAD_INPUT : ORC_OK;
}

static void extract_diag(const csr_t *A, double *d) {
    for (int64_t i = 0; i < A->n; i++) {
        d[i] = 0.0;
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) if (A->ci[k] == i) d[i] += A->v[k];
    }
}

/* dense Cholesky of the coarsest operator; returns nonzero if not SPD */
static int dense_cholesky(const csr_t *A, double **Lout) {
    int64_t n = A->n;
    double *L = (double *)calloc((size_t)(n > 0 ? n : 1) * (n > 0 ? n : 1), sizeof(double));
    for (int64_t i = 0; i < n; i++)
        for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) L[i * n + A->ci[k]] += A->v[k];
    for (int64_t j = 0; j < n; j++) {
        double s = L[j * n + j];
        for (int64_t k = 0; k < j; k++) s -= L[j * n + k] * L[j * n + k];
        if (!(s > 0.0)) { free(L); return 1; }
        double d = sqrt(s);
        L[j * n + j] = d;
        for (int64_t i = j + 1; i < n; i++) {
            double t = L[i * n + j];
            for (int64_t k = 0; k < j; k++) t -= L[i * n + k] * L[j * n + k];
            L[i * n + j] = t / d;
        }
        for (int64_t i = 0; i < j; i++) L[i * n + j] = 0.0;
    }
    *Lout = L;
    return 0;
}

static void dense_chol_solve(const double *L, int64_t n, const double *b, double *x) {
    for (int64_t i = 0; i < n; i++) {
        double s = b[i];
        for (int64_t k = 0; k < i; k++) s -= L[i * n + k] * x[k];
        x[i] = s / L[i * n + i];
    }
    for (int64_t i = n - 1; i >= 0; i--) {
        double s = x[i];
        for (int64_t k = i + 1; k < n; k++) s -= L[k * n + i] * x[k];
        x[i] = s / L[i * n + i];
    }
}

static void amg_free(amg_t *M) {
    if (!M) return;
    for (int l = 0; l < M->nlev; l++) {
        level_t *L = &M->lev[l];
        if (l > 0) csr_free(&L->A); /* level-0 matrix is owned by the caller */
        csr_free(&L->P); csr_free(&L->R);
        free(L->diag); free(L->x); free(L->b); free(L->r);
    }
    free(M->coarse_L);
    memset(M, 0, sizeof(*M));
}

/* build a Ruge-Stueben hierarchy on A (A is borrowed, not copied) */
static int amg_setup(const csr_t *A, amg_t *M, double theta, int64_t max_coarse, int max_levels) {
    memset(M, 0, sizeof(*M));
    M->lev[0].A = *A;
    M->nlev = 1;
    for (;;) {
        level_t *L = &M->lev[M->nlev - 1];
        L->n = L->A.n;
        L->diag = (double *)malloc((L->n > 0 ? L->n : 1) * sizeof(double));
        L->x = (double *)malloc((L->n > 0 ? L->n : 1) * sizeof(double));
        L->b = (double *)malloc((L->n > 0 ? L->n : 1) * sizeof(double));
        L->r = (double *)malloc((L->n > 0 ? L->n : 1) * sizeof(double));
        extract_diag(&L->A, L->diag);
        if (L->n <= max_coarse || M->nlev >= max_levels) break;
        csr_t S, ST;
        classical_strength(&L->A, theta, &S);
        csr_transpose(&S, &ST);
        int8_t *split = (int8_t *)malloc(L->n);
        rs_splitting(&S, &ST, split);
        int rc = direct_interpolation(&L->A, &S, split, &L->P);
        free(split); csr_free(&S); csr_free(&ST);
        if (rc) return rc;
        if (L->P.m == 0 || L->P.m >= L->n) { csr_free(&L->P); break; }
        csr_transpose(&L->P, &L->R);
        csr_t AP;
        spgemm(&L->A, &L->P, &AP);
        level_t *Lc = &M->lev[M->nlev];
        spgemm(&L->R, &AP, &Lc->A);
        csr_free(&AP);
        M->nlev++;
    }
    level_t *Lc = &M->lev[M->nlev - 1];
    M->nc = Lc->n;
    if (M->nc > 20000) return ORC_BREAKDOWN; /* coarsening stalled: no dense solve that large */
    if (dense_cholesky(&Lc->A, &M->coarse_L)) return ORC_BREAKDOWN;
    return ORC_OK;
}

/* Gauss-Seidel sweep; forward when dir > 0, backward otherwise. With several
 * threads each thread sweeps its own contiguous block of rows. */
static void gauss_seidel(const csr_t *A, const double *diag, const double *b, double *x, int dir) {
    int64_t n = A->n;
    if (g_threads <= 1) {
        if (dir > 0) {
            for (int64_t i = 0; i < n; i++) {
                double s = b[i];
                for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) if (A->ci[k] != i) s -= A->v[k] * x[A->ci[k]];
                x[i] = s / diag[i];
            }
        } else {
            for (int64_t i = n - 1; i >= 0; i--) {
                double s = b[i];
                for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) if (A->ci[k] != i) s -= A->v[k] * x[A->ci[k]];
                x[i] = s / diag[i];
            }
        }
        return;
    }
#pragma omp parallel
    {
#ifdef _OPENMP
        int t = omp_get_thread_num(), nt = omp_get_num_threads();
#else
        int t = 0, nt = 1;
#endif
        int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        if (dir > 0) {
            for (int64_t i = lo; i < hi; i++) {
                double s = b[i];
                for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) if (A->ci[k] != i) s -= A->v[k] * x[A->ci[k]];
                x[i] = s / diag[i];
            }
        } else {
            for (int64_t i = hi - 1; i >= lo; i--) {
                double s = b[i];
                for (int64_t k = A->rp[i]; k < A->rp[i + 1]; k++) if (A->ci[k] != i) s -= A->v[k] * x[A->ci[k]];
                x[i] = s / diag[i];
            }
        }
    }
}

/* symmetric V(1,1) cycle: x = V(b) with zero initial guess */
static void vcycle(amg_t *M, int l, const double *b, double *x) {
    level_t *L = &M->lev[l];
    if (l == M->nlev - 1) { dense_chol_solve(M->coarse_L, M->nc, b, x); return; }
    memset(x, 0, L->n * sizeof(double));
    gauss_seidel(&L->A, L->diag, b, x, +1);
    residual(&L->A, b, x, L->r);
    level_t *Lc = &M->lev[l + 1];
    spmv(&L->R, L->r, Lc->b);
    vcycle(M, l + 1, Lc->b, Lc->x);
    /* x += P xc */
    int64_t n = L->n;
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (int64_t i = 0; i < n; i++) {
        double s = 0.0;
        for (int64_t k = L->P.rp[i]; k < L->P.rp[i + 1]; k++) s += L->P.v[k] * Lc->x[L->P.ci[k]];
        x[i] += s;
    }
    gauss_seidel(&L->A, L->diag, b, x, -1);
}

/* AMG-preconditioned CG; stops when ||b - A x|| <= reltol ||b|| (recursive residual,
 * confirmed by a true residual at exit). x holds the initial guess on entry. */
static int pcg(const csr_t *A, amg_t *M, const double *b, double *x, double reltol, int maxiter,
               int *iters_out, double *relres_out) {
    int64_t n = A->n;
    double *r = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
    double *z = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
    double *p = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
    double *q = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
    double nb = sqrt(dot(n, b, b));
    int status = ORC_OK, it = 0;
    if (nb == 0.0) {
        memset(x, 0, n * sizeof(double));
        if (iters_out) *iters_out = 0;
        if (relres_out) *relres_out = 0.0;
        free(r); free(z); free(p); free(q);
        return ORC_OK;
    }
    residual(A, b, x, r);
    double rn = sqrt(dot(n, r, r));
    if (rn > reltol * nb) {
        vcycle(M, 0, r, z);
        memcpy(p, z, n * sizeof(double));
        double rz = dot(n, r, z);
        for (it = 1; it <= maxiter; it++) {
            spmv(A, p, q);
            double pq = dot(n, p, q);
            if (!(pq > 0.0)) { status = ORC_BREAKDOWN; break; }
            double a = rz / pq;
#pragma omp parallel for schedule(static) if (g_threads > 1)
            for (int64_t i = 0; i < n; i++) { x[i] += a * p[i]; r[i] -= a * q[i]; }
            rn = sqrt(dot(n, r, r));
            if (rn <= reltol * nb) break;
            vcycle(M, 0, r, z);
            double rz2 = dot(n, r, z);
            double beta = rz2 / rz;
            rz = rz2;
#pragma omp parallel for schedule(static) if (g_threads > 1)
            for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        }
        if (it > maxiter) { it = maxiter; status = ORC_NOT_CONVERGED; }
    }
    residual(A, b, x, r);
    double tr = sqrt(dot(n, r, r)) / nb;
    if (iters_out) *iters_out = it;
    if (relres_out) *relres_out = tr;
    free(r); free(z); free(p); free(q);
    return status;
}

/* ---------------------------------------------------------- the problem */
typedef struct {
    int64_t N, F, nd, nfree;
    int64_t *na, *nb;       /* faces, 0-based */
    double *aol;            /* areas over lengths, F */
    int8_t *isfree;         /* N */
    int64_t *node2free;     /* N, -1 for Dirichlet nodes */
    int64_t *free2node;     /* nfree */
    int64_t *fslot_ab, *fslot_ba, *fslot_aa, *fslot_bb; /* CSR slots of each face's four entries, -1 when absent */
    csr_t A;                /* nfree x nfree, assembled with the current Ks (and storage term) */
    amg_t amg;
    int have_amg;
    double *hfree;          /* last steady solution */
    double *Ks;             /* last Ks, F */
    double *shift;          /* optional diagonal shift (storage / dt), nfree */
    double theta;
    int64_t max_coarse;
    int max_levels;
} orc_problem;

/* getfreenodes (src/utilities.jl:10-24), 0-based */
static void getfreenodes(orc_problem *P, const int64_t *dn) {
    P->isfree = (int8_t *)malloc(P->N > 0 ? P->N : 1);
    for (int64_t i = 0; i < P->N; i++) P->isfree[i] = 1;
    for (int64_t k = 0; k < P->nd; k++) P->isfree[dn[k]] = 0;
    P->node2free = (int64_t *)malloc((P->N > 0 ? P->N : 1) * sizeof(int64_t));
    int64_t j = 0;
    for (int64_t i = 0; i < P->N; i++) if (P->isfree[i]) j++;
    P->nfree = j;
    P->free2node = (int64_t *)malloc((j > 0 ? j : 1) * sizeof(int64_t));
    j = 0;
    for (int64_t i = 0; i < P->N; i++) {
        if (P->isfree[i]) { P->node2free[i] = j; P->free2node[j] = i; j++; }
        else P->node2free[i] = -1;
    }
}

orc_problem *orc_create(int64_t N, int64_t F, const int64_t *na, const int64_t *nb, const double *aol,
                        int64_t nd, const int64_t *dn) {
    if (N <= 0 || F < 0) return NULL;
    for (int64_t f = 0; f < F; f++)
        if (na[f] < 0 || na[f] >= N || nb[f] < 0 || nb[f] >= N || na[f] == nb[f]) return NULL;
    for (int64_t k = 0; k < nd; k++) if (dn[k] < 0 || dn[k] >= N) return NULL;
    orc_problem *P = (orc_problem *)calloc(1, sizeof(orc_problem));
    P->N = N; P->F = F; P->nd = nd;
    P->na = (int64_t *)malloc((F > 0 ? F : 1) * sizeof(int64_t));
    P->nb = (int64_t *)malloc((F > 0 ? F : 1) * sizeof(int64_t));
    P->aol = (double *)malloc((F > 0 ? F : 1) * sizeof(double));
    if (F) { memcpy(P->na, na, F * sizeof(int64_t)); memcpy(P->nb, nb, F * sizeof(int64_t)); memcpy(P->aol, aol, F * sizeof(double)); }
    getfreenodes(P, dn);
    P->theta = 0.25; P->max_coarse = 500; P->max_levels = 30;
    P->Ks = (double *)calloc(F > 0 ? F : 1, sizeof(double));
    P->hfree = (double *)calloc(P->nfree > 0 ? P->nfree : 1, sizeof(double));
    /* symbolic CSR of the free-node Jacobian (groundwater_h pattern): diagonal of
     * every free node plus, for each free-free face, both off-diagonal entries. */
    int64_t nf = P->nfree;
    csr_t *A = &P->A;
    A->n = nf; A->m = nf;
    A->rp = (int64_t *)calloc(nf + 1, sizeof(int64_t));
    for (int64_t i = 0; i < nf; i++) A->rp[i + 1] = 1;
    for (int64_t f = 0; f < F; f++) {
        int64_t a = P->node2free[na[f]], b = P->node2free[nb[f]];
        if (a >= 0 && b >= 0) { A->rp[a + 1]++; A->rp[b + 1]++; }
    }
    for (int64_t i = 0; i < nf; i++) A->rp[i + 1] += A->rp[i];
    int64_t nnz = A->rp[nf];
    A->ci = (int32_t *)malloc((nnz > 0 ? nnz : 1) * sizeof(int32_t));
    A->v = (double *)calloc(nnz > 0 ? nnz : 1, sizeof(double));
    int64_t *pos = (int64_t *)malloc((nf > 0 ? nf : 1) * sizeof(int64_t));
    for (int64_t i = 0; i < nf; i++) { A->ci[A->rp[i]] = (int32_t)i; pos[i] = A->rp[i] + 1; }
    for (int64_t f = 0; f < F; f++) {
        int64_t a = P->node2free[na[f]], b = P->node2free[nb[f]];
        if (a >= 0 && b >= 0) { A->ci[pos[a]++] = (int32_t)b; A->ci[pos[b]++] = (int32_t)a; }
    }
    free(pos);
    /* sort + merge duplicates (pattern only), then locate each face's slots */
    csr_sort_merge(A);
    P->fslot_ab = (int64_t *)malloc((F > 0 ? F : 1) * sizeof(int64_t));
    P->fslot_ba = (int64_t *)malloc((F > 0 ? F : 1) * sizeof(int64_t));
    P->fslot_aa = (int64_t *)malloc((F > 0 ? F : 1) * sizeof(int64_t));
    P->fslot_bb = (int64_t *)malloc((F > 0 ? F : 1) * sizeof(int64_t));
    for (int64_t f = 0; f < F; f++) {
        int64_t a = P->node2free[na[f]], b = P->node2free[nb[f]];
        P->fslot_ab[f] = P->fslot_ba[f] = P->fslot_aa[f] = P->fslot_bb[f] = -1;
        for (int pass = 0; pass < 2; pass++) {
            int64_t r = pass ? b : a, c1 = pass ? a : b;
            if (r < 0) continue;
            for (int64_t k = A->rp[r]; k < A->rp[r + 1]; k++) {
                if (A->ci[k] == r) { if (pass) P->fslot_bb[f] = k; else P->fslot_aa[f] = k; }
                if (c1 >= 0 && A->ci[k] == c1) { if (pass) P->fslot_ba[f] = k; else P->fslot_ab[f] = k; }
            }
        }
    }
    return P;
}

void orc_destroy(orc_problem *P) {
    if (!P) return;
    if (P->have_amg) amg_free(&P->amg);
    csr_free(&P->A);
    free(P->na); free(P->nb); free(P->aol); free(P->isfree); free(P->node2free); free(P->free2node);
    free(P->fslot_ab); free(P->fslot_ba); free(P->fslot_aa); free(P->fslot_bb);
    free(P->hfree); free(P->Ks); free(P->shift);
    free(P);
}

int64_t orc_nfree(const orc_problem *P) { return P->nfree; }
int64_t orc_nnz(const orc_problem *P) { return P->A.rp[P->A.n]; }
int orc_levels(const orc_problem *P) { return P->have_amg ? P->amg.nlev : 0; }
void orc_set_amg(orc_problem *P, double theta, int64_t max_coarse, int max_levels) {
    P->theta = theta; P->max_coarse = max_coarse; P->max_levels = max_levels;
}

/* Assemble A = groundwater_h and b = -groundwater_residuals(0) with S = V = 1
 * (src/groundwater.jl:4-20, :77-79). For every face and both orientations
 * (node1, node2): a free node1 gets +K*aol on its diagonal; a free node2 adds
 * -K*aol at (node1, node2); a Dirichlet node2 adds K*aol*dirichleths[node2] to
 * b[node1]. Free nodes add Qs to b. */
static void assemble(orc_problem *P, const double *Ks, const double *dh, const double *Qs, double *b) {
    csr_t *A = &P->A;
    memset(A->v, 0, A->rp[A->n] * sizeof(double));
    if (b) for (int64_t j = 0; j < P->nfree; j++) b[j] = Qs[P->free2node[j]];
    for (int64_t f = 0; f < P->F; f++) {
        double c = Ks[f] * P->aol[f];
        int64_t a = P->na[f], bb = P->nb[f];
        int64_t ja = P->node2free[a], jb = P->node2free[bb];
        if (ja >= 0) {
            A->v[P->fslot_aa[f]] += c;
            if (jb >= 0) A->v[P->fslot_ab[f]] -= c;
            else if (b) b[ja] += c * dh[bb];
        }
        if (jb >= 0) {
            A->v[P->fslot_bb[f]] += c;
            if (ja >= 0) A->v[P->fslot_ba[f]] -= c;
            else if (b) b[jb] += c * dh[a];
        }
    }
    if (P->shift)
        for (int64_t j = 0; j < P->nfree; j++)
            for (int64_t k = A->rp[j]; k < A->rp[j + 1]; k++) if (A->ci[k] == j) { A->v[k] += P->shift[j]; break; }
}

static int rebuild_amg(orc_problem *P) {
    if (P->have_amg) { amg_free(&P->amg); P->have_amg = 0; }
    int rc = amg_setup(&P->A, &P->amg, P->theta, P->max_coarse, P->max_levels);
    if (rc) { amg_free(&P->amg); return rc; }
    P->have_amg = 1;
    return ORC_OK;
}

/* Export the assembled operator (free-node CSR) and right-hand side. */
int orc_assemble(orc_problem *P, const double *Ks, const double *dh, const double *Qs,
                 int64_t *rp, int32_t *ci, double *v, double *b) {
    free(P->shift); P->shift = NULL;
    assemble(P, Ks, dh, Qs, b);
    int64_t nnz = P->A.rp[P->A.n];
    if (rp) memcpy(rp, P->A.rp, (P->A.n + 1) * sizeof(int64_t));
    if (ci) memcpy(ci, P->A.ci, nnz * sizeof(int32_t));
    if (v) memcpy(v, P->A.v, nnz * sizeof(double));
    return ORC_OK;
}

/* groundwater_steadystate (src/groundwater.jl:75-83): returns h over all N nodes,
 * dirichleths at Dirichlet nodes. */
int orc_steady_solve(orc_problem *P, const double *Ks, const double *dh, const double *Qs, double reltol,
                     int maxiter, double *h, int *iters, double *relres) {
    free(P->shift); P->shift = NULL;
    double *b = (double *)malloc((P->nfree > 0 ? P->nfree : 1) * sizeof(double));
    assemble(P, Ks, dh, Qs, b);
    memcpy(P->Ks, Ks, P->F * sizeof(double));
    int rc = rebuild_amg(P);
    if (rc) { free(b); return rc; }
    memset(P->hfree, 0, P->nfree * sizeof(double));
    rc = pcg(&P->A, &P->amg, b, P->hfree, reltol, maxiter, iters, relres);
    free(b);
    for (int64_t i = 0; i < P->N; i++) h[i] = P->isfree[i] ? P->hfree[P->node2free[i]] : dh[i];
    return rc;
}

/* rrule pullback (src/groundwater.jl:93-107) with cotangent delta[N]:
 *   lambda = A^{-T} delta[free]   (A is symmetric, so the forward hierarchy is reused)
 *   dKs_f  = -aol_f (h_a - h_b)(lambda_a - lambda_b), lambda = 0 and h = dirichleths at Dirichlet ends
 *   ddh_k  = sum_{faces (j,k), j free} K_f aol_f lambda_j + delta_k   for Dirichlet k, else 0
 *   dQs_i  = lambda_i for free i, else 0 */
int orc_steady_adjoint(orc_problem *P, const double *dh, const double *delta, double reltol, int maxiter,
                       double *dKs, double *ddh, double *dQs, int *iters, double *relres) {
    if (!P->have_amg) return ORC_BAD_INPUT;
    int64_t nf = P->nfree;
    double *rhs = (double *)malloc((nf > 0 ? nf : 1) * sizeof(double));
    double *lam = (double *)calloc(nf > 0 ? nf : 1, sizeof(double));
    for (int64_t j = 0; j < nf; j++) rhs[j] = delta[P->free2node[j]];
    int rc = pcg(&P->A, &P->amg, rhs, lam, reltol, maxiter, iters, relres);
    for (int64_t f = 0; f < P->F; f++) {
        int64_t a = P->na[f], b = P->nb[f];
        int64_t ja = P->node2free[a], jb = P->node2free[b];
        double ha = ja >= 0 ? P->hfree[ja] : dh[a], hb = jb >= 0 ? P->hfree[jb] : dh[b];
        double la = ja >= 0 ? lam[ja] : 0.0, lb = jb >= 0 ? lam[jb] : 0.0;
        dKs[f] = -P->aol[f] * (ha - hb) * (la - lb);
    }
    for (int64_t i = 0; i < P->N; i++) {
        ddh[i] = P->isfree[i] ? 0.0 : delta[i];
        dQs[i] = P->isfree[i] ? lam[P->node2free[i]] : 0.0;
    }
    for (int64_t f = 0; f < P->F; f++) {
        int64_t a = P->na[f], b = P->nb[f];
        int64_t ja = P->node2free[a], jb = P->node2free[b];
        double c = P->Ks[f] * P->aol[f];
        if (ja >= 0 && jb < 0) ddh[b] += c * lam[ja];
        if (jb >= 0 && ja < 0) ddh[a] += c * lam[jb];
    }
    free(rhs); free(lam);
    return rc;
}

/* ------------------------------------------------------------ face means */
/* kind 0: geometric exp(0.5(logKa+logKb)); kind 1: harmonic 2/(1/Ka+1/Kb), K = exp(logK) */
void orc_logk_to_faces(int64_t F, const int64_t *na, const int64_t *nb, const double *logK, int kind, double *Ks) {
    for (int64_t f = 0; f < F; f++) {
        double la = logK[na[f]], lb = logK[nb[f]];
        if (kind == 0) Ks[f] = exp(0.5 * (la + lb));
        else Ks[f] = 2.0 / (exp(-la) + exp(-lb));
    }
}

/* vector-Jacobian product: dlogK += (dKs/dlogK)^T dKs */
void orc_logk_to_faces_vjp(int64_t N, int64_t F, const int64_t *na, const int64_t *nb, const double *logK, int kind,
                           const double *dKs, double *dlogK) {
    for (int64_t i = 0; i < N; i++) dlogK[i] = 0.0;
    for (int64_t f = 0; f < F; f++) {
        double la = logK[na[f]], lb = logK[nb[f]];
        if (kind == 0) {
            double K = exp(0.5 * (la + lb));
            dlogK[na[f]] += 0.5 * K * dKs[f];
            dlogK[nb[f]] += 0.5 * K * dKs[f];
        } else {
            double Ka = exp(la), Kb = exp(lb);
            double K = 2.0 / (1.0 / Ka + 1.0 / Kb);
            dlogK[na[f]] += K * K / (2.0 * Ka) * dKs[f];
            dlogK[nb[f]] += K * K / (2.0 * Kb) * dKs[f];
        }
    }
}

/* --------------------------------------------------------------- transient */
/* Fixed-step backward Euler for S_i V_i dh_i/dt = Q_i - sum_f K_f aol_f (h_i - h_nb)
 * (src/groundwater.jl:7,15,17): (D/dt + A) h^{n+1} = (D/dt) h^n + b, D = diag(Ss V).
 * h0 and the states are over free nodes. states (nsteps x nfree) may be NULL.
 * Returns the final free-node state in hT. Every step solves to reltol with the
 * previous state as initial guess. */
int orc_transient_forward(orc_problem *P, const double *Ks, const double *dh, const double *Qs, const double *Ss,
                          const double *V, double dt, int nsteps, const double *h0, double reltol, int maxiter,
                          double *states, double *hT, int *total_iters) {
    int64_t nf = P->nfree;
    free(P->shift);
    P->shift = (double *)malloc((nf > 0 ? nf : 1) * sizeof(double));
    for (int64_t j = 0; j < nf; j++) { int64_t i = P->free2node[j]; P->shift[j] = Ss[i] * V[i] / dt; }
    double *b = (double *)malloc((nf > 0 ? nf : 1) * sizeof(double));
    double *rhs = (double *)malloc((nf > 0 ? nf : 1) * sizeof(double));
    double *h = (double *)malloc((nf > 0 ? nf : 1) * sizeof(double));
    assemble(P, Ks, dh, Qs, b);
    memcpy(P->Ks, Ks, P->F * sizeof(double));
    int rc = rebuild_amg(P);
    if (rc) { free(b); free(rhs); free(h); return rc; }
    memcpy(h, h0, nf * sizeof(double));
    int tot = 0;
    for (int n = 0; n < nsteps; n++) {
        for (int64_t j = 0; j < nf; j++) rhs[j] = P->shift[j] * h[j] + b[j];
        int it = 0; double rr = 0;
        int r2 = pcg(&P->A, &P->amg, rhs, h, reltol, maxiter, &it, &rr);
        tot += it;
        if (r2 && !rc) rc = r2;
        if (states) memcpy(states + (int64_t)n * nf, h, nf * sizeof(double));
    }
    memcpy(hT, h, nf * sizeof(double));
    if (total_iters) *total_iters = tot;
    free(b); free(rhs); free(h);
    return rc;
}

/* Discrete adjoint of orc_transient_forward for J = sum_n sum_k w_k (h^n[obs_k])^2 + gT . h^nsteps
 * (obs are node indices of free nodes; gT over free nodes, may be NULL).
 * states must hold all nsteps states from the forward pass (the oracle keeps them all).
 *   (D/dt + A) mu^n = dJ/dh^n + (D/dt) mu^{n+1},  mu^{nsteps+1} = 0
 *   dKs_f  = -sum_n aol_f (h^n_a - h^n_b)(mu^n_a - mu^n_b)
 *   ddh_k  = sum_n sum_{faces (j,k), j free} K_f aol_f mu^n_j     (Dirichlet k)
 *   dQs_i  = sum_n mu^n_i                                          (free i)
 *   dh0    = (D/dt) mu^1 over free nodes */
int orc_transient_adjoint(orc_problem *P, const double *dh, int nsteps, const double *states, int64_t nobs,
                          const int64_t *obs, const double *w, const double *gT, double reltol, int maxiter,
                          double *dKs, double *ddh, double *dQs, double *dh0, int *total_iters) {
    if (!P->have_amg || !P->shift) return ORC_BAD_INPUT;
    int64_t nf = P->nfree, N = P->N, F = P->F;
    double *mu = (double *)calloc(nf > 0 ? nf : 1, sizeof(double));
    double *rhs = (double *)malloc((nf > 0 ? nf : 1) * sizeof(double));
    for (int64_t f = 0; f < F; f++) dKs[f] = 0.0;
    for (int64_t i = 0; i < N; i++) { ddh[i] = 0.0; dQs[i] = 0.0; }
    int tot = 0, rc = ORC_OK;
    for (int n = nsteps - 1; n >= 0; n--) {
        const double *hn = states + (int64_t)n * nf;
        for (int64_t j = 0; j < nf; j++) rhs[j] = P->shift[j] * mu[j];
        for (int64_t k = 0; k < nobs; k++) {
            int64_t j = P->node2free[obs[k]];
            if (j >= 0) rhs[j] += 2.0 * w[k] * hn[j];
        }
        if (gT && n == nsteps - 1) for (int64_t j = 0; j < nf; j++) rhs[j] += gT[j];
        int it = 0; double rr = 0;
        int r2 = pcg(&P->A, &P->amg, rhs, mu, reltol, maxiter, &it, &rr);
        tot += it;
        if (r2 && !rc) rc = r2;
        for (int64_t f = 0; f < F; f++) {
            int64_t a = P->na[f], b = P->nb[f];
            int64_t ja = P->node2free[a], jb = P->node2free[b];
            double ha = ja >= 0 ? hn[ja] : dh[a], hb = jb >= 0 ? hn[jb] : dh[b];
            double la = ja >= 0 ? mu[ja] : 0.0, lb = jb >= 0 ? mu[jb] : 0.0;
            dKs[f] -= P->aol[f] * (ha - hb) * (la - lb);
            double c = P->Ks[f] * P->aol[f];
            if (ja >= 0 && jb < 0) ddh[b] += c * mu[ja];
            if (jb >= 0 && ja < 0) ddh[a] += c * mu[jb];
        }
        for (int64_t j = 0; j < nf; j++) dQs[P->free2node[j]] += mu[j];
    }
    if (dh0) for (int64_t j = 0; j < nf; j++) dh0[j] = P->shift[j] * mu[j];
    if (total_iters) *total_iters = tot;
    free(mu); free(rhs);
    return rc;
}
