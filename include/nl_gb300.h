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
    int       precision;      /* NL_GB300_PRECISION_DOUBLE / _MIXED /
                                 _DOUBLE_FLOAT (_AUTO = _MIXED for a matrix
                                 given directly)                          */
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
    double    algo_bytes;         /* algorithmic HBM bytes moved by the solve:
                                     per FP64 iteration 12 nnz + 108 n, per FP32
                                     iteration 8 nnz + 56 n, per reliable update
                                     12 nnz + 52 n, + initial/final residuals;
                                     a double-float iteration counts as FP64 */
    int       precision;          /* precision that ran: NL_GB300_PRECISION_DOUBLE,
                                     _MIXED (also after an FP64 fallback) or
                                     _DOUBLE_FLOAT                         */
} nlgb_result;

/* ---- device / errors ---- */
int         nlgb_device_available(void);
/* Kernels this library has launched in the process so far (host launches
 * plus the kernel nodes executed inside the solver's CUDA graphs). */
long long   nlgb_kernel_launches(void);
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
 * multiple of 64 in [64, 2^20]; 0 keeps the current value). */
int         nlgb_matrix_set_layout(nlgb_matrix A, int threads_per_row, int tile_rows);
/* General (non-symmetric) square systems: BiCGSTAB or GMRES(restart), FP64,
 * right-preconditioned by the Jacobi diagonal (jacobi != 0) or not.  Same
 * solvers as nlSolveSystemIterative(NL_BICGSTAB / NL_GMRES) (reference:
 * src/lib/OGF/scene_graph/NL/matrix.cpp:390-393), on a matrix handle.
 * b, x: host or device vectors; x is the initial guess.  res->iterations:
 * BiCGSTAB iterations or GMRES inner steps. */
#define NLGB_KRYLOV_BICGSTAB 1
#define NLGB_KRYLOV_GMRES    2
int         nlgb_solve_krylov(nlgb_matrix A, const double* b, double* x, int method, double eps,
                              long long max_iter, int restart, int jacobi, nlgb_result* res);

/* Mesh system builders on the GPU.  Replace the host-side row emission of
 * Graphite's mesh_compute_LSCM and mesh_smooth commands (reference:
 * src/lib/OGF/mesh/commands/mesh_grob_surface_commands.cpp:759 and :703,
 * whose builders emit rows through nlBegin(NL_ROW)/nlCoefficient): one GPU
 * thread per triangle writes the rows, then the normal-equation assembly of
 * nlgb_assemble builds the system.  xyz: n_verts x 3 doubles, tris:
 * n_tris x 3 vertex indices (host or device arrays).
 *
 * LSCM: variables u_k = 2k, v_k = 2k + 1; the two pinned vertices (pins, or
 * NULL for 0 and n_verts - 1) are locked at pin_uv = (u0, v0, u1, v1) (NULL:
 * (0, 0) and (1, 1)); the matrix is over the 2 n_verts - 4 free variables and
 * rhs_out (host or device, may be NULL) receives the right-hand side.
 * Fairing: the cotangent Laplacian + lambda I (L_ij = -(cot a + cot b) / 2).
 * An out-of-range triangle index returns NLGB_E_INVALID.  *seconds: build
 * time on the host clock (may be NULL). */
int         nlgb_build_lscm(int n_verts, const double* xyz, int n_tris, const int* tris,
                            const int* pins, const double* pin_uv, nlgb_matrix* A_out,
                            double* rhs_out, double* seconds);
int         nlgb_build_fairing(int n_verts, const double* xyz, int n_tris, const int* tris,
                               double lambda, nlgb_matrix* A_out, double* seconds);
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

/* ---- one FP64 solve without any device allocation ----
 * No counterpart in the reference: an addition for callers that cannot
 * allocate GPU memory -- host applications that reserve all device memory
 * for their own pools and must keep their footprint fixed, or interactive
 * loops that cannot afford the device synchronisation cudaMalloc/cudaFree
 * imply.  Same FP64 Jacobi-PCG as nlgb_solve (NL_GB300_PRECISION_DOUBLE
 * only).  rp, ci, va (CRS, n x n), b and x are caller-owned DEVICE buffers
 * (x 16-byte aligned; initial guess in, solution out); all scratch lives in
 * one static device array of the library (8.1 MiB per GPU, kept until the
 * process exits), so n is limited to 262144 rows (larger n: NLGB_E_INVALID).
 * The first call on a device looks up the array's address with that device
 * current (cudaGetSymbolAddress); make that first call before any stream
 * capture begins.  Every call reuses the same array and clears what must
 * start at zero: calls that overlap on the GPU race and must be serialised
 * by the caller.  stream: a cudaStream_t (NULL:
 * the default stream); the call returns when the solve is finished
 * (res->seconds: host time of the call).  n == 0 returns at once
 * (converged). */
int nlgb_solve_noalloc(int n, const int* rp, const int* ci, const double* va, const double* b,
                       double* x, const nlgb_params* prm, nlgb_result* res, void* stream);

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

/* ---- solve server: continuous batching under an HBM budget ----
 * No reference counterpart as a component: in Graphite every nlSolve is a
 * synchronous call made under the global command lock
 * (src/lib/OGF/scene_graph/commands/commands.cpp:99-117).  The server
 * accepts solves of any size at any time, admits them while their device
 * footprint fits the HBM budget, keeps their matrices and Krylov state
 * resident until convergence and advances every admitted system together:
 * each "epoch" is one persistent-kernel launch over the active systems (see
 * NLGB_SCHEDULE_*); requests arriving meanwhile are uploaded and built (or
 * their least-squares rows assembled) by an admission thread on a second
 * stream while the epoch runs, and join the next epoch.  A result does not depend on what else
 * is in flight (bit-identical alone and in any mix). */
typedef struct nlgb_server_s* nlgb_server;

#define NLGB_SERVER_BATCHED 0   /* continuous batching, persistent kernel     */
#define NLGB_SERVER_SERIAL  1   /* one request at a time, graph-captured PCG  */

/* Scheduling of the batched server.  SRPT (shortest remaining processing
 * time, the default): `streams` CUDA streams each run one system at a time
 * as a chunk of CUDA-graph PCG iterations lasting about epoch_ms; whenever a
 * stream is free it takes the system with the least estimated remaining work
 * (iterations left, extrapolated from the system's residual history, times
 * its bytes per iteration); a new system first gets a short probe (16
 * iterations).  A request that just arrived starts within about epoch_ms,
 * light requests finish first, and work-heavy ones progress whenever a
 * stream has nothing lighter to do.  ALL: epochs of the persistent batched
 * kernel in which every active system runs epoch_iters iterations. */
#define NLGB_SCHEDULE_SRPT 0
#define NLGB_SCHEDULE_ALL  1

typedef struct {
    size_t    hbm_budget_bytes;  /* admission limit (default 150e9)            */
    int       mode;              /* NLGB_SERVER_BATCHED / NLGB_SERVER_SERIAL    */
    int       precision;         /* NL_GB300_PRECISION_MIXED (default) / _DOUBLE /
                                    _DOUBLE_FLOAT / _AUTO: FP64 for
                                    least-squares row and LSCM mesh
                                    submissions, mixed for the others     */
    double    eps;               /* relative residual (default 1e-10)          */
    long long max_iter;          /* < 0: 5 n per system                         */
    double    inner_eps;         /* mixed reliable-update factor (0.1)         */
    long long epoch_iters;       /* iterations per system per epoch (256)      */
    int       max_systems;       /* active systems at once (8192; <= 65536)    */
    int       schedule;          /* NLGB_SCHEDULE_SRPT (default) / _ALL         */
    double    epoch_ms;          /* SRPT: target length of a chunk (10 ms)     */
    int       streams;           /* SRPT: concurrent chunks (default 16)        */
    double    eps_least_squares; /* relative residual of least-squares
                                    submissions (rows with least_squares,
                                    LSCM meshes); <= 0 (default): eps.  The
                                    normal equations square kappa, so a
                                    solution error bound (e.g. 1e-8 against a
                                    direct solve) can need a residual below
                                    the one square systems stop at.        */
    int       min_tile_rows;     /* batched server: each system is cut into
                                    tiles of at least this many rows (rounded
                                    up to a multiple of 128).  0 (default): the
                                    single-system autotuner's tiling, which
                                    spreads one system over every SM.  When
                                    many systems share the GPU, fewer and
                                    fuller CTAs per system pay: 1024 completed
                                    5 % more requests of the serving stream
                                    than 0.  Results stay bit-identical alone
                                    and in any mix; against nlgb_solve they
                                    are bit-identical when the matrix has the
                                    same layout (nlgb_matrix_set_layout).   */
    int       chunk_cta_budget;  /* batched SRPT server: a chunk starts only
                                    while the phase-kernel CTAs of the chunks
                                    in flight, its own included, stay within
                                    this many (the first chunk always starts).
                                    0 (default): no limit; < 0: one resident
                                    wave of the phase kernels (SMs x 8).  With
                                    one wave, large systems no longer share
                                    the GPU many ways and finish sooner: on the
                                    serving stream 20 % more requests
                                    completed over 60 s and 6 % more in the
                                    4-s window (32 streams, tiles of at least
                                    2,048 rows).  Scheduling only: results do
                                    not change.                              */
} nlgb_server_config;

typedef struct {
    long long submitted, completed, failed, rejected;
    double    p50_latency_s, p99_latency_s, mean_latency_s, max_latency_s;
    double    solves_per_s;      /* completed / (last completion - first arrival) */
    double    wall_s;            /* first arrival -> last completion           */
    double    kernel_s;          /* device time of all epochs / serial solves  */
    long long epochs;
    long long iterations;        /* PCG iterations over all systems            */
    double    algo_bytes;        /* algorithmic HBM bytes over all systems     */
    size_t    peak_bytes;        /* peak admitted device footprint             */
    size_t    budget_bytes;
    double    graph_s;           /* part of kernel_s spent in graph chunks
                                    (large FP64 systems continued on the
                                    single-system graph executor once only
                                    such systems are left)                   */
    double    graph_algo_bytes;  /* part of algo_bytes: iterations run there   */
    long long graph_epochs;      /* part of epochs run as graph chunks         */
    size_t    used_bytes;        /* device footprint admitted now              */
    double    byte_seconds;      /* admitted footprint integrated over time
                                    since the clock (re)started: the mean HBM
                                    occupancy is byte_seconds / elapsed time  */
    double    epoch_algo_bytes;  /* algorithmic bytes of every iteration run in
                                    the epochs (finished or not)               */
} nlgb_server_stats;

void        nlgb_server_default_config(nlgb_server_config* cfg);
nlgb_server nlgb_server_create(const nlgb_server_config* cfg);
/* Restart the server clock at 0 (arrival times are relative to it). */
void        nlgb_server_reset_clock(nlgb_server srv);
double      nlgb_server_now(nlgb_server srv);
/* Square SPD system in CRS form with n_rhs right-hand sides b[k*n + i]
 * (x0: NULL or n_rhs*n initial guesses).  x_out (host, n_rhs*n) receives the
 * solutions and must stay valid until nlgb_server_wait returns.  The input
 * arrays are copied before the call returns.  arrival_s: time on the server
 * clock before which the request is not admitted (< 0: now).  Returns a
 * ticket >= 0 or a negative NLGB_E* code (e.g. a request larger than the
 * whole budget is rejected with NLGB_E_NOMEM). */
long long   nlgb_server_submit_crs(nlgb_server srv, int n, const int* rp, const int* ci,
                                   const double* va, int n_rhs, const double* b, const double* x0,
                                   double* x_out, double arrival_s);
/* Least-squares (or square) row stream, assembled on the GPU at admission;
 * same conventions as nlgb_assemble; x_out holds n_rhs * n_free values. */
long long   nlgb_server_submit_rows(nlgb_server srv, int least_squares, long long n_rows,
                                    const long long* row_ptr, const int* col, const double* val,
                                    const double* rhs, const double* weight, int n_free,
                                    int n_vars, const double* xl, int n_rhs, const double* x0,
                                    double* x_out, double arrival_s);
/* A triangle mesh whose system the server builds on the GPU at admission
 * (nlgb_build_lscm / nlgb_build_fairing).  NLGB_MESH_LSCM: one system over
 * the 2 n_verts - 4 free variables (pins / pin_uv as in nlgb_build_lscm,
 * NULL for the defaults), n_rhs must be 1 and b NULL.  NLGB_MESH_FAIRING:
 * L + lambda I over n_verts variables, b holds n_rhs * n_verts right-hand
 * sides.  x0 (may be NULL) and x_out hold n_rhs * n values.  Reference: the
 * solve of mesh_compute_LSCM / mesh_smooth
 * (src/lib/OGF/mesh/commands/mesh_grob_surface_commands.cpp:759, :703). */
#define NLGB_MESH_LSCM    0
#define NLGB_MESH_FAIRING 1
long long   nlgb_server_submit_mesh(nlgb_server srv, int mesh_kind, int n_verts, const double* xyz,
                                    int n_tris, const int* tris, const int* pins,
                                    const double* pin_uv, double lambda, int n_rhs,
                                    const double* b, const double* x0, double* x_out,
                                    double arrival_s);
/* Block until the ticket completes; res: n_rhs entries (may be NULL). */
int         nlgb_server_wait(nlgb_server srv, long long ticket, nlgb_result* res,
                             double* latency_s);
int         nlgb_server_drain(nlgb_server srv);
int         nlgb_server_get_stats(nlgb_server srv, nlgb_server_stats* st);
/* Stop admitting and abort: queued requests fail at once, active systems
 * stop at the next epoch boundary (a solve running on a graph executor, e.g.
 * the SERIAL mode's, within one while-loop pass of 4 iterations) with
 * NL_GB300_STATUS_ABORTED; nlgb_server_wait reports those requests as
 * failed. */
void        nlgb_server_abort(nlgb_server srv);
void        nlgb_server_destroy(nlgb_server srv);

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
