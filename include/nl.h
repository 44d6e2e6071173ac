/*
 * nl.h -- OpenNL-compatible C API of libnl_gb300 (sparse least-squares /
 * SPD solves on one GB300 GPU).
 *
 * This header restates the OpenNL API surface that Graphite's callers bind.
 * The reference calls these symbols from:
 *   plugins/OGF/WarpDrive/commands/voxel_grob_transport_commands.cpp:231-287
 *       (context API: nlNewContext ... nlSolve ... nlGetVariable)
 *   src/lib/OGF/scene_graph/NL/matrix.cpp:51-66,121-440
 *       (matrix API: nlSparseMatrixNew/Add, nlMatrixCompress,
 *        nlMultMatrixVector, nlNewJacobiPreconditioner,
 *        nlSolveSystemIterative, nlMatrixFactorize, nlInitExtension)
 *   src/lib/OGF/scene_graph/NL/blas.cpp:66-144  (NLBlas table)
 * OpenNL's own header lives in the geogram submodule, which is not part of
 * the reference checkout, so the numeric values of the NLenum constants
 * below are this library's own: it is a SOURCE-level drop-in (callers
 * recompile against this header), not a binary one.
 *
 * Semantics (documented here because they are the contract the GPU path and
 * the CPU oracle both implement):
 *   - A row is the equation  sum_j a_j x_j = b  (b set by nlRightHandSide,
 *     default 0).  nlRowScaling(w) weights the row by w in least-squares mode.
 *     Repeated nlCoefficient(j, .) calls within one row are summed.
 *   - NL_LEAST_SQUARES = NL_TRUE: the system solved is the normal equations
 *     over the FREE variables,
 *        (sum_r w_r a_r,f a_r,f^T) x_f = sum_r w_r a_r,f (b_r - a_r,l . x_l)
 *     where l ranges over locked variables (values from nlSetVariable).
 *     Assembly happens on the GPU (row-merge into CRS).
 *   - NL_LEAST_SQUARES = NL_FALSE: the k-th row given is the equation of the
 *     k-th free variable (free variables numbered by increasing index); the
 *     number of rows must equal the number of free variables.
 *   - nlSolve runs Jacobi-preconditioned CG on the GPU from the current
 *     variable values, until ||b - A x||_2 <= NL_THRESHOLD * ||b||_2
 *     (recursively updated residual for NL_GB300_PRECISION_DOUBLE, then the
 *     true FP64 residual is recomputed and, if it misses the threshold, the
 *     iteration continues with a lower recursive threshold; the true FP64
 *     residual for NL_GB300_PRECISION_MIXED) or NL_MAX_ITERATIONS.
 *     Defaults: NL_THRESHOLD = 1e-10, NL_MAX_ITERATIONS = 5 * n_free.
 *   - Errors never abort the process: void calls report through
 *     nlGetError()/nlGetErrorString() and stderr; nlSolve returns NL_FALSE.
 *   - One current context per process (OpenNL semantics, not thread-safe);
 *     the explicit-handle API in nl_gb300.h has no global state.
 */
#ifndef NL_GB300_OPENNL_H
#define NL_GB300_OPENNL_H

#ifdef __cplusplus
extern "C" {
#endif

#define NL_GB300_VERSION_MAJOR 1
#define NL_GB300_VERSION_MINOR 0

typedef unsigned int   NLenum;
typedef unsigned char  NLboolean;
typedef unsigned int   NLbitfield;
typedef void           NLvoid;
typedef signed char    NLbyte;
typedef short          NLshort;
typedef int            NLint;
typedef unsigned char  NLubyte;
typedef unsigned short NLushort;
typedef unsigned int   NLuint;
typedef unsigned long  NLulong;
typedef int            NLsizei;
typedef float          NLfloat;
typedef double         NLdouble;
typedef void*          NLContext;

#define NL_FALSE 0x0
#define NL_TRUE  0x1

/* ---- nlSolverParameteri / nlGetIntegerv / nlGetDoublev names ---- */
#define NL_SOLVER              0x100
#define NL_NB_VARIABLES        0x101
#define NL_LEAST_SQUARES       0x102
#define NL_MAX_ITERATIONS      0x103
#define NL_THRESHOLD           0x104
#define NL_OMEGA               0x105
#define NL_SYMMETRIC           0x106
#define NL_USED_ITERATIONS     0x107
#define NL_ERROR               0x108
#define NL_INNER_ITERATIONS    0x109
#define NL_ELAPSED_TIME        0x10a
#define NL_PRECONDITIONER      0x10b
#define NL_GFLOPS              0x10c
#define NL_NNZ                 0x10d
#define NL_NB_SYSTEMS          0x10e
/* library-specific parameters */
#define NL_GB300_PRECISION         0x1a0 /* NL_GB300_PRECISION_DOUBLE/_MIXED/_AUTO/_DOUBLE_FLOAT */
#define NL_GB300_INNER_THRESHOLD   0x1a1 /* mixed: FP64 reliable update once the FP32 residual fell by this factor (default 0.1) */
#define NL_GB300_REFINEMENT_STEPS  0x1a2 /* query: outer FP64 refinement steps used */
#define NL_GB300_STATUS            0x1a3 /* query: NL_GB300_STATUS_* of the last solve */
#define NL_GB300_TRUE_RESIDUAL     0x1a4 /* query: ||b-Ax||/||b|| recomputed in FP64 */
#define NL_GB300_THREADS_PER_ROW   0x1a5 /* 0 = autotune (default), else 1..32 */
#define NL_GB300_ASSEMBLY_TIME     0x1a6 /* query: seconds spent in GPU assembly */
#define NL_GB300_MAX_REFINEMENT    0x1a7 /* mixed: cap on FP64 reliable updates (default 100000) */

#define NL_GB300_PRECISION_DOUBLE 0x0
#define NL_GB300_PRECISION_MIXED  0x1
/* AUTO: FP64 for least-squares systems (normal equations: kappa(A^T A) =
 * kappa(A)^2, beyond what FP32 values can represent on mesh problems), mixed
 * for systems given as square rows or CRS. */
#define NL_GB300_PRECISION_AUTO   0x2
/* DOUBLE_FLOAT: the FP64 Jacobi-PCG (same stopping rule on the recursive
 * residual, true FP64 residual reported) with r, p, q, x, the matrix and
 * 1/diag held as unevaluated float pairs hi + lo (~48 significand bits)
 * computed on the FP32 pipe; the initial and final residuals are FP64.
 * Matrices with a value or 1/diagonal outside [2^-100, 2^100] run in FP64.
 * Opt-in: on very ill-conditioned systems (kappa ~ 1e10) it needs more
 * iterations than FP64 and its recursive residual drifts further from the
 * true one. */
#define NL_GB300_PRECISION_DOUBLE_FLOAT 0x3

#define NL_GB300_STATUS_NONE       0
#define NL_GB300_STATUS_CONVERGED  1
#define NL_GB300_STATUS_MAX_ITER   2
#define NL_GB300_STATUS_BREAKDOWN  3  /* p^T A p <= 0 or a NaN/Inf scalar   */
#define NL_GB300_STATUS_STAGNATION 4  /* mixed: refinement stopped improving */
#define NL_GB300_STATUS_DEVICE_ERR 5  /* CUDA error (message in nlGetErrorString) */
#define NL_GB300_STATUS_BAD_INPUT  6  /* rejected before touching the GPU     */
#define NL_GB300_STATUS_ABORTED    7  /* host abort flag raised              */
/* FP64 / double-float: the recursive residual met NL_THRESHOLD, and the true
 * FP64 residual recomputed then did not, even after the iteration was
 * continued with a lower recursive threshold (up to 4 times) -- the
 * attainable accuracy of the recurrence lies above NL_THRESHOLD.  The
 * solution is returned (nlSolve returns NL_TRUE: OpenNL's own stopping
 * rule was met); NL_GB300_TRUE_RESIDUAL gives the true residual. */
#define NL_GB300_STATUS_TRUE_RESIDUAL_STALLED 8

/* ---- solvers / preconditioners ---- */
#define NL_SOLVER_DEFAULT 0x000
#define NL_CG             0x200
#define NL_BICGSTAB       0x201  /* general square systems, FP64 */
#define NL_GMRES          0x202  /* restarted every NL_INNER_ITERATIONS steps, FP64 */

#define NL_PRECOND_NONE    0x000
#define NL_PRECOND_JACOBI  0x300
#define NL_PRECOND_SSOR    0x301  /* SSOR with relaxation NL_OMEGA (default 1.5):
                                     level-scheduled sweeps on the GPU, CG /
                                     BiCGSTAB / GMRES (symmetric matrices) */

/* ---- nlEnable / nlDisable / nlIsEnabled ---- */
#define NL_NORMALIZE_ROWS  0x400
#define NL_VERBOSE         0x401
#define NL_NO_VARIABLES_INDIRECTION 0x402

/* ---- nlBegin / nlEnd primitives ---- */
#define NL_SYSTEM  0x0
#define NL_MATRIX  0x1
#define NL_ROW     0x2
#define NL_MATRIX_PATTERN 0x3

/* ---- error codes (nlGetError) ---- */
#define NL_NO_ERROR          0x0
#define NL_INVALID_ENUM      0x1
#define NL_INVALID_VALUE     0x2
#define NL_INVALID_OPERATION 0x3
#define NL_OUT_OF_MEMORY     0x4
#define NL_DEVICE_ERROR      0x5

/* ---- context API (voxel_grob_transport_commands.cpp:231-287) ---- */
NLContext nlNewContext(void);
void      nlDeleteContext(NLContext context);
void      nlMakeCurrent(NLContext context);
NLContext nlGetCurrent(void);
NLboolean nlInitExtension(const char* extension);   /* matrix.cpp:51-66 */
NLboolean nlExtensionIsInitialized(const char* extension);

void      nlSolverParameterd(NLenum pname, NLdouble param);
void      nlSolverParameteri(NLenum pname, NLint param);
void      nlGetBooleanv(NLenum pname, NLboolean* params);
void      nlGetDoublev(NLenum pname, NLdouble* params);
void      nlGetIntegerv(NLenum pname, NLint* params);
void      nlEnable(NLenum pname);
void      nlDisable(NLenum pname);
NLboolean nlIsEnabled(NLenum pname);
NLenum    nlGetError(void);
const char* nlGetErrorString(void);

void      nlSetVariable(NLuint i, NLdouble value);
void      nlMultiSetVariable(NLuint i, NLuint k, NLdouble value);
NLdouble  nlGetVariable(NLuint i);
NLdouble  nlMultiGetVariable(NLuint i, NLuint k);
void      nlLockVariable(NLuint i);
void      nlUnlockVariable(NLuint i);
NLboolean nlVariableIsLocked(NLuint i);

void      nlBegin(NLenum primitive);
void      nlEnd(NLenum primitive);
void      nlCoefficient(NLuint i, NLdouble value);
void      nlAddIJCoefficient(NLuint i, NLuint j, NLdouble value);
void      nlAddIRightHandSide(NLuint i, NLdouble value);
void      nlMultiAddIRightHandSide(NLuint i, NLuint k, NLdouble value);
void      nlRightHandSide(NLdouble value);
void      nlMultiRightHandSide(NLuint k, NLdouble value);
void      nlRowScaling(NLdouble value);
NLboolean nlSolve(void);

/* ---- matrix API (scene_graph/NL/matrix.cpp) ---- */
#define NL_MATRIX_NONE           0x0
#define NL_MATRIX_SPARSE_DYNAMIC 0x1001
#define NL_MATRIX_CRS            0x1002
#define NL_MATRIX_SUPERLU_EXT    0x1003
#define NL_MATRIX_CHOLMOD_EXT    0x1004
#define NL_MATRIX_FUNCTION       0x1005
#define NL_MATRIX_OTHER          0x1006
#define NL_MATRIX_GB300_DEVICE   0x1010  /* resident CRS in GPU memory */

#define NL_MATRIX_STORE_ROWS      1
#define NL_MATRIX_STORE_COLUMNS   2
#define NL_MATRIX_STORE_SYMMETRIC 4

#define NL_SUPERLU_EXT           0x210
#define NL_PERM_SUPERLU_EXT      0x211
#define NL_SYMMETRIC_SUPERLU_EXT 0x212
#define NL_CHOLMOD_EXT           0x213

struct NLMatrixStruct;
typedef struct NLMatrixStruct* NLMatrix;
/* OGF::NL::Matrix casts its matrix to NLSparseMatrix* before
 * nlSparseMatrixAdd (matrix.cpp:163,237,257,291): here every matrix object
 * starts with NLMatrixStruct, so the two names are one type. */
typedef struct NLMatrixStruct NLSparseMatrix;
typedef void (*NLDestroyMatrixFunc)(NLMatrix M);
typedef void (*NLMultMatrixVectorFunc)(NLMatrix M, const double* x, double* y);

/* Leading fields are read directly by OGF::NL::Matrix (matrix.cpp:130-141);
 * the rest of each matrix object is private to the library. */
struct NLMatrixStruct {
    NLuint m;
    NLuint n;
    NLenum type;
    NLDestroyMatrixFunc destroy_func;
    NLMultMatrixVectorFunc mult_func;
};

NLMatrix nlSparseMatrixNew(NLuint m, NLuint n, NLenum storage);   /* matrix.cpp:121 */
void     nlSparseMatrixAdd(NLMatrix M, NLuint i, NLuint j, NLdouble value); /* :163 */
void     nlDeleteMatrix(NLMatrix M);                               /* :125,396 */
void     nlMatrixCompress(NLMatrix* M);                            /* :309 */
void     nlMultMatrixVector(NLMatrix M, const double* x, double* y); /* :303 */
NLuint   nlMatrixNNZ(NLMatrix M);
NLMatrix nlNewJacobiPreconditioner(NLMatrix M);                   /* :364 */
/* SSOR of a square symmetric sparse matrix, M = (D + w L) D^-1 (D + w L^T) /
 * (w (2 - w)); must not outlive M nor follow changes to it (the reference
 * wrapper creates it just before nlSolveSystemIterative and deletes it after). */
NLMatrix nlNewSSORPreconditioner(NLMatrix M, double omega);       /* :367 */
NLMatrix nlMatrixFactorize(NLMatrix M, NLenum solver);            /* :317-327, returns NULL */

/* ---- BLAS abstraction (scene_graph/NL/blas.cpp:66-144) ---- */
struct NLBlas;
typedef struct NLBlas* NLBlas_t;
typedef enum { NL_HOST_MEMORY = 0, NL_DEVICE_MEMORY = 1 } NLmemoryType;

typedef void   (*FUNPTR_copy)(NLBlas_t, int n, const double* x, int incx, double* y, int incy);
typedef void   (*FUNPTR_scal)(NLBlas_t, int n, double a, double* x, int incx);
typedef double (*FUNPTR_dot)(NLBlas_t, int n, const double* x, int incx, const double* y, int incy);
typedef double (*FUNPTR_nrm2)(NLBlas_t, int n, const double* x, int incx);
typedef void   (*FUNPTR_axpy)(NLBlas_t, int n, double a, const double* x, int incx, double* y, int incy);
typedef void   (*FUNPTR_mul)(NLBlas_t, int n, const double* x, double* y); /* y <- x .* y */

/* The table's vector arguments may be host or device pointers: the
 * computation always runs on the GPU (host vectors are staged through device
 * buffers, two PCIe / C2C transfers per call).  Increments follow BLAS:
 * element i of a vector with increment inc sits at i * inc, or at
 * (n - 1 - i) * |inc| when inc < 0; inc == 0 is rejected. */
struct NLBlas {
    FUNPTR_copy Dcopy;
    FUNPTR_scal Dscal;
    FUNPTR_dot  Ddot;
    FUNPTR_nrm2 Dnrm2;
    FUNPTR_axpy Daxpy;
    FUNPTR_mul  Dmul;
    NLboolean   has_unified_memory;
    double      flops;
    long long   used_ram[2];
    long long   max_used_ram[2];
};

NLBlas_t nlHostBlas(void);     /* blas.cpp:66, matrix.cpp:391 */
NLBlas_t nlCUDABlas(void);     /* same table; name kept for OpenNL's CUDA-extension callers */
void     nlBlasResetStats(NLBlas_t blas);

/* Iterative solve of M x = b (matrix.cpp:390-393).  M: CRS, dynamic or
 * device matrix; P: NULL, a Jacobi or an SSOR preconditioner; b, x: host or device
 * vectors of size M->n (x is the initial guess).  solver: NL_CG /
 * NL_SOLVER_DEFAULT (Jacobi-PCG), NL_BICGSTAB or NL_GMRES (restart length
 * inner_iter; both FP64, right-preconditioned by P); returns the number of
 * iterations used. */
NLuint nlSolveSystemIterative(NLBlas_t blas, NLMatrix M, NLMatrix P,
                              const double* b, double* x, NLenum solver,
                              double eps, NLuint max_iter, NLuint inner_iter);

#ifdef __cplusplus
}
#endif

#endif /* NL_GB300_OPENNL_H */
