/*
 * nl_gb300.h -- explicit-handle C API of libnl_gb300 (no global state).
 *
 * The OpenNL API in nl.h keeps one "current" context per process, which is
 * what the reference's callers bind.  This header adds handle-based entry
 * points used by the batched solver, the solve server and the benchmarks.
 * Each function below names the reference interface it replaces or extends.
 *
 * Conventions: functions return 0 on success and a negative NLGB_E* code on
 * failure (message in nlgb_last_error()).  Vector arguments may be host or
 * device pointers unless stated otherwise; matrices live in GPU memory.
 */
#ifndef NL_GB300_HANDLE_API_H
#define NL_GB300_HANDLE_API_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NLGB_OK          0
#define NLGB_E_INVALID  -1   /* bad argument (sizes, indices, enums)      */
#define NLGB_E_DEVICE   -2   /* CUDA error or no device                   */
#define NLGB_E_NOMEM    -3   /* device allocation failed / over budget    */
#define NLGB_E_STATE    -4   /* call not valid in the object's state      */

typedef struct nlgb_matrix_s* nlgb_matrix;

/* Solve parameters (nlSolverParameteri/d of nl.h, per call). */
typedef struct {
    double    eps;            /* stop when ||b-Ax|| <= eps ||b||           */
    long long max_iter;       /* < 0: 5 n                                  */
    int       precision;      /* NL_GB300_PRECISION_DOUBLE / _MIXED        */
    double    inner_eps;      /* mixed: reliable-update factor (0.1)       */
    int       max_outer;      /* mixed: cap on reliable updates (100000)   */
} nlgb_params;

typedef struct {
    int       status;             /* NL_GB300_STATUS_*                     */
    long long iterations;         /* PCG iterations (inner ones if mixed)  */
    int       refinement_steps;   /* mixed: outer FP64 steps               */
    double    rel_residual;       /* residual the stopping test used       */
    double    true_rel_residual;  /* ||b-Ax||/||b|| recomputed in FP64     */
    double    seconds;            /* device time of the iteration (events) */
} nlgb_result;

/* ---- device / errors ---- */
int         nlgb_device_available(void);
const char* nlgb_last_error(void);
void        nlgb_default_params(nlgb_params* p);

/* ---- resident CRS matrices ----
 * Replaces the CRS matrix of nlMatrixCompress (matrix.cpp:309) with one that
 * stays in HBM.  rp/ci/va: host or device arrays (copied). */
nlgb_matrix nlgb_matrix_create(int n_rows, int n_cols, const int* rp, const int* ci,
                               const double* va);
void        nlgb_matrix_destroy(nlgb_matrix A);
int         nlgb_matrix_info(nlgb_matrix A, int* n_rows, long long* nnz, int* threads_per_row,
                             int* tile_rows);
/* Override the autotuner (threads_per_row in {1,2,4,8,16,32}, tile_rows a
 * power of two in [64, 2^20]; 0 keeps the current value). */
int         nlgb_matrix_set_layout(nlgb_matrix A, int threads_per_row, int tile_rows);
/* Copy the CRS arrays back to host buffers of size n+1 / nnz / nnz. */
int         nlgb_matrix_download(nlgb_matrix A, int* rp, int* ci, double* va);
/* Jacobi inverse diagonal (host buffer of n doubles). */
int         nlgb_matrix_jacobi(nlgb_matrix A, double* dinv);

/* ---- SpMV (nlMultMatrixVector, matrix.cpp:303) ---- */
int nlgb_spmv(nlgb_matrix A, const double* x, double* y);
/* FP32 values/vectors; x, y device pointers. */
int nlgb_spmv32(nlgb_matrix A, const float* x, float* y);
/* Time `reps` back-to-back FP64 SpMVs on the library stream with CUDA
 * events (x, y device pointers); *ms = average per launch. */
int nlgb_spmv_timed(nlgb_matrix A, const double* x, double* y, int reps, double* ms);
int nlgb_spmv32_timed(nlgb_matrix A, const float* x, float* y, int reps, double* ms);

/* ---- one solve (nlSolveSystemIterative(NL_CG, Jacobi), matrix.cpp:390) ----
 * x holds the initial guess on entry and the solution on exit. */
int nlgb_solve(nlgb_matrix A, const double* b, double* x, const nlgb_params* prm,
               nlgb_result* res);

/* ---- many independent solves in one persistent-kernel launch ----
 * The batched form of nlSolveSystemIterative for many uneven systems, e.g.
 * the per-chart LSCM solves of mesh_make_atlas (called at
 * src/lib/OGF/mesh/commands/mesh_grob_surface_commands.cpp:724).  A[i] may
 * repeat (several right-hand sides of one matrix).  b[i], x[i]: host or
 * device vectors of A[i]'s size; x[i] is the initial guess on entry.  Each
 * system converges (or stops) on its own; results are bit-identical to
 * nlgb_solve on the same system.  *kernel_seconds: device time of the
 * launch (CUDA events). */
int nlgb_batch_solve(int n_sys, const nlgb_matrix* A, const double* const* b, double* const* x,
                     const nlgb_params* prm, nlgb_result* res, double* kernel_seconds);

/* ---- least-squares / square assembly on the GPU (nlEnd(NL_MATRIX) of an
 * NL_LEAST_SQUARES context, voxel_grob_transport_commands.cpp:232-279) ----
 * Row stream: row r has coefficients [row_ptr[r], row_ptr[r+1]) of
 * (col, val), col >= 0 a free-variable index, col < 0 the locked variable
 * -col-1 whose value is xl[sys * n_vars + var]; rhs[sys * n_rows + r];
 * weight: NULL or n_rows row weights.  All host pointers.  Outputs the
 * normal matrix (least_squares != 0) or the square matrix, and rhs_out
 * (host, n_systems * n_free). */
int nlgb_assemble(int least_squares, long long n_rows, const long long* row_ptr, const int* col,
                  const double* val, const double* rhs, const double* weight, int n_free,
                  int n_vars, const double* xl, int n_systems, nlgb_matrix* A_out,
                  double* rhs_out, double* seconds);

/* ---- bulk rows for the current OpenNL context ----
 * Exactly equivalent to, for each row r: nlBegin(NL_ROW); nlCoefficient(
 * var[k], val[k]) for k in [row_ptr[r], row_ptr[r+1]); nlMultiRightHandSide(
 * s, rhs[r * n_systems + s]); nlRowScaling(weight ? weight[r] : 1);
 * nlEnd(NL_ROW).  (var are VARIABLE indices, host arrays.) */
int nlgb_add_rows(long long n_rows, const long long* row_ptr, const int* var, const double* val,
                  const double* rhs, const double* weight);
/* Bulk nlSetVariable / nlLockVariable / nlGetVariable on the current
 * context (values[sys * n + i]). */
int nlgb_set_variables(const double* values, const unsigned char* locked);
int nlgb_get_variables(double* values);

#ifdef __cplusplus
}
#endif

#endif /* NL_GB300_HANDLE_API_H */
