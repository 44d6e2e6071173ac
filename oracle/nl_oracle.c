/*
 * nl_oracle.c -- CPU restatement of OpenNL's least-squares assembly and
 * Jacobi-preconditioned CG.  TEST INFRASTRUCTURE ONLY: used by tests/, by
 * __graft_entry__.smoke() as the checker and by bench.py's CPU-baseline leg;
 * the library (graphitethree_gb300/lib/libnl_gb300.so) never calls it.
 *
 * What it restates (OpenNL's source lives in the geogram submodule, which is
 * absent from the reference checkout, so the semantics follow the in-tree
 * call sites and the published algorithms):
 *   - row assembly in NL_LEAST_SQUARES mode with locked variables:
 *     plugins/OGF/WarpDrive/commands/voxel_grob_transport_commands.cpp:231-279
 *     (nlSolverParameteri(NL_LEAST_SQUARES), nlSetVariable/nlLockVariable,
 *     nlBegin(NL_ROW)/nlCoefficient/nlEnd(NL_ROW));
 *   - nlSolveSystemIterative(NL_CG) with nlNewJacobiPreconditioner,
 *     stopping on ||b - A x||/||b|| < eps or max_iter:
 *     src/lib/OGF/scene_graph/NL/matrix.cpp:364,390-393 and the
 *     solve_iterative contract in src/lib/OGF/scene_graph/NL/matrix.h:170-186;
 *   - nlMultMatrixVector (CRS SpMV): matrix.cpp:303.
 *
 * Exact conventions (shared with the GPU library, see include/nl.h):
 *   row r = sum_k val[k] x[var_k] = b_r with weight w_r; locked coefficients
 *   are moved to the right-hand side in coefficient order:
 *       s_r = b_r; for each locked k: s_r = s_r - val[k] * x[var_k]
 *   and for each free pair (i, j) of the row, in row order r:
 *       wa_i = w_r * a_i;  M[i][j] += wa_i * a_j;  rhs[i] += wa_i * s_r
 *   (no fused multiply-add: build with -ffp-contract=off).
 */
#include <math.h>
#include <time.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int n;
    long long nnz;
    int* rp;
    int* ci;
    double* va;
    double* rhs;   /* n_systems * n */
    int n_systems;
} nlo_system;

/* Dynamic sparse row: (col, val) pairs in insertion order. */
typedef struct {
    int* col;
    double* val;
    int len, cap;
} dyn_row;

static void dyn_add(dyn_row* r, int c, double v) {
    for (int t = 0; t < r->len; ++t) {
        if (r->col[t] == c) { r->val[t] = r->val[t] + v; return; }
    }
    if (r->len == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 16;
        r->col = (int*)realloc(r->col, sizeof(int) * r->cap);
        r->val = (double*)realloc(r->val, sizeof(double) * r->cap);
    }
    r->col[r->len] = c;
    r->val[r->len] = 0.0 + v;
    r->len++;
}

static int cmp_pair(const void* a, const void* b) {
    const int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* Assemble the normal equations (least_squares != 0) or the square system
 * from a row stream.  col[k] >= 0: free index; col[k] < 0: locked variable
 * -col[k]-1 with value xl[sys * n_vars + var].  rhs[sys * n_rows + r]. */
nlo_system* nlo_assemble(int least_squares, long long n_rows, const long long* row_ptr,
                         const int* col, const double* val, const double* rhs,
                         const double* weight, int n_free, int n_vars, const double* xl,
                         int n_systems) {
    nlo_system* S = (nlo_system*)calloc(1, sizeof(nlo_system));
    S->n = n_free;
    S->n_systems = n_systems;
    S->rhs = (double*)calloc((size_t)n_systems * (n_free > 0 ? n_free : 1), sizeof(double));
    double* s = (double*)malloc(sizeof(double) * (n_systems > 0 ? n_systems : 1));
    if (least_squares) {
        dyn_row* rows = (dyn_row*)calloc(n_free > 0 ? n_free : 1, sizeof(dyn_row));
        for (long long r = 0; r < n_rows; ++r) {
            const long long k0 = row_ptr[r], k1 = row_ptr[r + 1];
            const double w = weight ? weight[r] : 1.0;
            for (int sys = 0; sys < n_systems; ++sys) {
                double acc = rhs ? rhs[(size_t)sys * n_rows + r] : 0.0;
                for (long long k = k0; k < k1; ++k) {
                    if (col[k] < 0) {
                        const int var = -col[k] - 1;
                        const double t = val[k] * xl[(size_t)sys * n_vars + var];
                        acc = acc - t;
                    }
                }
                s[sys] = acc;
            }
            for (long long ki = k0; ki < k1; ++ki) {
                const int i = col[ki];
                if (i < 0) continue;
                const double wa = w * val[ki];
                for (long long kj = k0; kj < k1; ++kj) {
                    const int j = col[kj];
                    if (j < 0) continue;
                    const double prod = wa * val[kj];
                    dyn_add(&rows[i], j, prod);
                }
                for (int sys = 0; sys < n_systems; ++sys) {
                    const double t = wa * s[sys];
                    S->rhs[(size_t)sys * n_free + i] = S->rhs[(size_t)sys * n_free + i] + t;
                }
            }
        }
        /* compress, columns ascending */
        S->rp = (int*)malloc(sizeof(int) * (n_free + 1));
        long long nnz = 0;
        for (int i = 0; i < n_free; ++i) nnz += rows[i].len;
        S->nnz = nnz;
        S->ci = (int*)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
        S->va = (double*)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
        long long o = 0;
        S->rp[0] = 0;
        int* idx = NULL;
        int idx_cap = 0;
        for (int i = 0; i < n_free; ++i) {
            dyn_row* R = &rows[i];
            if (R->len > idx_cap) {
                idx_cap = R->len;
                idx = (int*)realloc(idx, sizeof(int) * 2 * idx_cap);
            }
            /* sort (col, position) pairs by col */
            for (int t = 0; t < R->len; ++t) { idx[2 * t] = R->col[t]; idx[2 * t + 1] = t; }
            qsort(idx, R->len, 2 * sizeof(int), cmp_pair);
            for (int t = 0; t < R->len; ++t) {
                S->ci[o] = idx[2 * t];
                S->va[o] = R->val[idx[2 * t + 1]];
                ++o;
            }
            S->rp[i + 1] = (int)o;
            free(R->col);
            free(R->val);
        }
        free(idx);
        free(rows);
    } else {
        /* square: row r is the equation of free variable r; order kept */
        S->rp = (int*)malloc(sizeof(int) * (n_rows + 1));
        long long nnz = 0;
        for (long long r = 0; r < n_rows; ++r)
            for (long long k = row_ptr[r]; k < row_ptr[r + 1]; ++k) nnz += col[k] >= 0;
        S->nnz = nnz;
        S->ci = (int*)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
        S->va = (double*)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
        long long o = 0;
        S->rp[0] = 0;
        for (long long r = 0; r < n_rows; ++r) {
            for (int sys = 0; sys < n_systems; ++sys) {
                double acc = rhs ? rhs[(size_t)sys * n_rows + r] : 0.0;
                for (long long k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
                    if (col[k] < 0) {
                        const int var = -col[k] - 1;
                        const double t = val[k] * xl[(size_t)sys * n_vars + var];
                        acc = acc - t;
                    }
                }
                S->rhs[(size_t)sys * n_free + r] = acc;
            }
            for (long long k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
                if (col[k] >= 0) { S->ci[o] = col[k]; S->va[o] = val[k]; ++o; }
            }
            S->rp[r + 1] = (int)o;
        }
    }
    free(s);
    return S;
}

void nlo_system_info(const nlo_system* S, int* n, long long* nnz) {
    *n = S->n;
    *nnz = S->nnz;
}

void nlo_system_copy(const nlo_system* S, int* rp, int* ci, double* va, double* rhs) {
    memcpy(rp, S->rp, sizeof(int) * (S->n + 1));
    memcpy(ci, S->ci, sizeof(int) * S->nnz);
    memcpy(va, S->va, sizeof(double) * S->nnz);
    memcpy(rhs, S->rhs, sizeof(double) * (size_t)S->n_systems * S->n);
}

void nlo_system_free(nlo_system* S) {
    if (!S) return;
    free(S->rp); free(S->ci); free(S->va); free(S->rhs);
    free(S);
}

/* y = A x (CRS), rows in parallel. */
void nlo_spmv(int n, const int* rp, const int* ci, const double* va, const double* x, double* y,
              int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = rp[i]; k < rp[i + 1]; ++k) s = s + va[k] * x[ci[k]];
        y[i] = s;
    }
    (void)nthreads;
}

static double dot(int n, const double* a, const double* b, int nthreads) {
    double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    (void)nthreads;
    return s;
}

static double wall_seconds(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return (double)clock() / CLOCKS_PER_SEC;
#endif
}

/* Jacobi-preconditioned CG (jacobi != 0) or plain CG.  x: initial guess in,
 * solution out.  Returns the status: 1 converged, 2 max_iter, 3 breakdown,
 * 4 time limit (max_seconds > 0: checked every 16 iterations; used by the
 * time-bounded CPU baseline). */
int nlo_pcg_timed(int n, const int* rp, const int* ci, const double* va, const double* b, double* x,
                  double eps, long long max_iter, int jacobi, int nthreads, double max_seconds,
                  long long* iters_out, double* rel_res_out) {
    const double t_start = max_seconds > 0.0 ? wall_seconds() : 0.0;
    double* r = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    double* z = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    double* p = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    double* q = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    double* d = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    int status = 0;
    long long it = 0;
    for (int i = 0; i < n; ++i) {
        double di = 0.0;
        if (jacobi)
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                if (ci[k] == i) di += va[k];
        d[i] = (jacobi && di != 0.0) ? 1.0 / di : 1.0;
    }
    const double bb = dot(n, b, b, nthreads);
    double rr = 0.0, rho = 0.0;
    if (!(bb > 0.0)) {
        for (int i = 0; i < n; ++i) x[i] = 0.0;
        status = bb == 0.0 ? 1 : 3;
        goto done;
    }
    nlo_spmv(n, rp, ci, va, x, q, nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int i = 0; i < n; ++i) {
        r[i] = b[i] - q[i];
        z[i] = d[i] * r[i];
        p[i] = z[i];
    }
    rho = dot(n, r, z, nthreads);
    rr = dot(n, r, r, nthreads);
    while (1) {
        if (rr <= eps * eps * bb) { status = 1; break; }
        if (it >= max_iter) { status = 2; break; }
        nlo_spmv(n, rp, ci, va, p, q, nthreads);
        const double pq = dot(n, p, q, nthreads);
        if (!(pq > 0.0)) { status = 3; break; }
        const double alpha = rho / pq;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
        for (int i = 0; i < n; ++i) {
            x[i] = x[i] + alpha * p[i];
            r[i] = r[i] - alpha * q[i];
            z[i] = d[i] * r[i];
        }
        const double rho_new = dot(n, r, z, nthreads);
        rr = dot(n, r, r, nthreads);
        ++it;
        if (rr <= eps * eps * bb) { status = 1; break; }
        if (it >= max_iter) { status = 2; break; }
        if (max_seconds > 0.0 && (it & 15) == 0 && wall_seconds() - t_start > max_seconds) {
            status = 4;
            break;
        }
        if (!(rho_new > 0.0)) { status = 3; break; }
        const double beta = rho_new / rho;
        rho = rho_new;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
done:
    if (iters_out) *iters_out = it;
    if (rel_res_out) *rel_res_out = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    free(r); free(z); free(p); free(q); free(d);
    return status;
}

int nlo_pcg(int n, const int* rp, const int* ci, const double* va, const double* b, double* x,
            double eps, long long max_iter, int jacobi, int nthreads, long long* iters_out,
            double* rel_res_out) {
    return nlo_pcg_timed(n, rp, ci, va, b, x, eps, max_iter, jacobi, nthreads, 0.0, iters_out,
                         rel_res_out);
}

/* SSOR preconditioner of a symmetric A = L + D + L^T, relaxation omega in
 * (0, 2): M = (D + omega L) D^-1 (D + omega L^T) / (omega (2 - omega)).
 * z = M^-1 r by the two sequential sweeps
 *   forward:  y_i = (omega (2 - omega) r_i - omega sum_{j<i} a_ij y_j) / d_i
 *   backward: z_i = y_i - (omega / d_i) sum_{j>i} a_ij z_j
 * (row entries in their CRS order; d_i = a_ii, 1 when missing or zero). */
static void ssor_apply(int n, const int* rp, const int* ci, const double* va, const double* d,
                       double omega, const double* r, double* y, double* z) {
    const double c = omega * (2.0 - omega);
    for (int i = 0; i < n; ++i) {
        double s = c * r[i];
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] < i) s = s - omega * va[k] * y[ci[k]];
        y[i] = s / d[i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = 0.0;
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] > i) s = s + va[k] * z[ci[k]];
        z[i] = y[i] - omega * s / d[i];
    }
}

static void ssor_diag(int n, const int* rp, const int* ci, const double* va, double* d) {
    for (int i = 0; i < n; ++i) {
        double di = 0.0;
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] == i) di += va[k];
        d[i] = di != 0.0 ? di : 1.0;
    }
}

/* PCG with the SSOR preconditioner (sequential sweeps, the rest as
 * nlo_pcg).  Returns 1 converged, 2 max_iter, 3 breakdown. */
int nlo_pcg_ssor(int n, const int* rp, const int* ci, const double* va, const double* b, double* x,
                 double eps, long long max_iter, double omega, long long* iters_out,
                 double* rel_res_out) {
    const size_t sz = sizeof(double) * (n > 0 ? n : 1);
    double *r = (double*)calloc(1, sz), *z = (double*)calloc(1, sz), *p = (double*)calloc(1, sz);
    double *q = (double*)calloc(1, sz), *d = (double*)calloc(1, sz), *y = (double*)calloc(1, sz);
    int status = 0;
    long long it = 0;
    ssor_diag(n, rp, ci, va, d);
    const double bb = dot(n, b, b, 1);
    double rr = 0.0, rho = 0.0;
    if (!(bb > 0.0)) {
        for (int i = 0; i < n; ++i) x[i] = 0.0;
        status = bb == 0.0 ? 1 : 3;
        goto done;
    }
    nlo_spmv(n, rp, ci, va, x, q, 1);
    for (int i = 0; i < n; ++i) r[i] = b[i] - q[i];
    ssor_apply(n, rp, ci, va, d, omega, r, y, z);
    for (int i = 0; i < n; ++i) p[i] = z[i];
    rho = dot(n, r, z, 1);
    rr = dot(n, r, r, 1);
    while (1) {
        if (rr <= eps * eps * bb) { status = 1; break; }
        if (it >= max_iter) { status = 2; break; }
        nlo_spmv(n, rp, ci, va, p, q, 1);
        const double pq = dot(n, p, q, 1);
        if (!(pq > 0.0)) { status = 3; break; }
        const double alpha = rho / pq;
        for (int i = 0; i < n; ++i) {
            x[i] = x[i] + alpha * p[i];
            r[i] = r[i] - alpha * q[i];
        }
        ssor_apply(n, rp, ci, va, d, omega, r, y, z);
        const double rho_new = dot(n, r, z, 1);
        rr = dot(n, r, r, 1);
        ++it;
        if (rr <= eps * eps * bb) { status = 1; break; }
        if (it >= max_iter) { status = 2; break; }
        if (!(rho_new > 0.0)) { status = 3; break; }
        const double beta = rho_new / rho;
        rho = rho_new;
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
done:
    if (iters_out) *iters_out = it;
    if (rel_res_out) *rel_res_out = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    free(r); free(z); free(p); free(q); free(d); free(y);
    return status;
}

/* z = M^-1 r of the SSOR preconditioner above (tests of the sweeps). */
void nlo_ssor_apply(int n, const int* rp, const int* ci, const double* va, double omega, const double* r,
                    double* z) {
    const size_t sz = sizeof(double) * (n > 0 ? n : 1);
    double *d = (double*)calloc(1, sz), *y = (double*)calloc(1, sz);
    ssor_diag(n, rp, ci, va, d);
    ssor_apply(n, rp, ci, va, d, omega, r, y, z);
    free(d); free(y);
}

int nlo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
