"""Host-side logic of the OpenNL context API: the state machine, parameter
validation, error reporting and row bookkeeping.  No compute call reaches
the GPU here (nlSolve is only called where the test expects the no-device
error)."""
import numpy as np
import pytest

from graphitethree_gb300 import opennl as nl


@pytest.fixture
def ctx(nllib):
    c = nl.nlNewContext()
    nl.nlGetError()
    yield c
    nl.nlDeleteContext(c)


def test_context_lifecycle(ctx):
    assert nl.nlGetCurrent() == ctx
    other = nl.nlNewContext()
    assert nl.nlGetCurrent() == other
    nl.nlMakeCurrent(ctx)
    assert nl.nlGetCurrent() == ctx
    nl.nlDeleteContext(other)
    assert nl.nlGetCurrent() == ctx


def test_parameters_roundtrip(ctx):
    nl.nlSolverParameteri(nl.NL_NB_VARIABLES, 10)
    nl.nlSolverParameteri(nl.NL_LEAST_SQUARES, nl.NL_TRUE)
    nl.nlSolverParameterd(nl.NL_THRESHOLD, 1e-7)
    nl.nlSolverParameteri(nl.NL_MAX_ITERATIONS, 123)
    nl.nlSolverParameteri(nl.NL_GB300_PRECISION, nl.NL_GB300_PRECISION_MIXED)
    assert nl.nlGetIntegerv(nl.NL_NB_VARIABLES) == 10
    assert nl.nlGetIntegerv(nl.NL_LEAST_SQUARES) == 1
    assert nl.nlGetDoublev(nl.NL_THRESHOLD) == 1e-7
    assert nl.nlGetIntegerv(nl.NL_MAX_ITERATIONS) == 123
    assert nl.nlGetIntegerv(nl.NL_GB300_PRECISION) == nl.NL_GB300_PRECISION_MIXED
    assert nl.nlGetError() == nl.NL_NO_ERROR
    nl.nlSolverParameteri(nl.NL_GB300_PRECISION, nl.NL_GB300_PRECISION_DOUBLE_FLOAT)
    assert nl.nlGetIntegerv(nl.NL_GB300_PRECISION) == nl.NL_GB300_PRECISION_DOUBLE_FLOAT
    assert nl.nlGetError() == nl.NL_NO_ERROR
    nl.nlSolverParameteri(nl.NL_GB300_PRECISION, nl.NL_GB300_PRECISION_AUTO)
    assert nl.nlGetIntegerv(nl.NL_GB300_PRECISION) == nl.NL_GB300_PRECISION_AUTO
    nl.nlSolverParameteri(nl.NL_GB300_PRECISION, 7)
    assert nl.nlGetError() == nl.NL_INVALID_ENUM
    assert nl.nlGetIntegerv(nl.NL_GB300_PRECISION) == nl.NL_GB300_PRECISION_AUTO


def test_bad_parameters_are_rejected(ctx):
    nl.nlSolverParameteri(0x7777, 1)
    assert nl.nlGetError() == nl.NL_INVALID_ENUM
    nl.nlSolverParameterd(nl.NL_THRESHOLD, -1.0)
    assert nl.nlGetError() == nl.NL_INVALID_VALUE
    nl.nlSolverParameteri(nl.NL_GB300_THREADS_PER_ROW, 3)
    assert nl.nlGetError() == nl.NL_INVALID_VALUE
    nl.nlSolverParameteri(nl.NL_NB_SYSTEMS, 0)
    assert nl.nlGetError() == nl.NL_INVALID_VALUE


def test_state_machine_order_is_enforced(ctx):
    nl.nlBegin(nl.NL_ROW)                 # no system yet
    assert nl.nlGetError() == nl.NL_INVALID_OPERATION
    nl.nlBegin(nl.NL_SYSTEM)              # NL_NB_VARIABLES unset
    assert nl.nlGetError() == nl.NL_INVALID_VALUE
    nl.nlSolverParameteri(nl.NL_NB_VARIABLES, 3)
    nl.nlBegin(nl.NL_SYSTEM)
    assert nl.nlGetError() == nl.NL_NO_ERROR
    nl.nlCoefficient(0, 1.0)              # outside a row
    assert nl.nlGetError() == nl.NL_INVALID_OPERATION
    nl.nlBegin(nl.NL_MATRIX)
    nl.nlLockVariable(0)                  # locking after NL_MATRIX
    assert nl.nlGetError() == nl.NL_INVALID_OPERATION
    nl.nlBegin(nl.NL_ROW)
    nl.nlCoefficient(7, 1.0)              # index out of range
    assert nl.nlGetError() == nl.NL_INVALID_VALUE
    nl.nlEnd(nl.NL_ROW)
    assert nl.nlSolve() == 0              # system not constructed
    assert nl.nlGetError() == nl.NL_INVALID_OPERATION


def test_square_system_needs_one_row_per_free_variable(ctx):
    nl.nlSolverParameteri(nl.NL_NB_VARIABLES, 3)
    nl.nlBegin(nl.NL_SYSTEM)
    nl.nlLockVariable(2)
    nl.nlBegin(nl.NL_MATRIX)
    nl.nlBegin(nl.NL_ROW); nl.nlCoefficient(0, 2.0); nl.nlEnd(nl.NL_ROW)
    nl.nlEnd(nl.NL_MATRIX)
    assert nl.nlGetError() == nl.NL_INVALID_OPERATION
    assert "one row per free variable" in nl.nlGetErrorString()


def test_variables_and_locks(ctx):
    nl.nlSolverParameteri(nl.NL_NB_VARIABLES, 4)
    nl.nlSolverParameteri(nl.NL_NB_SYSTEMS, 2)
    nl.nlBegin(nl.NL_SYSTEM)
    nl.nlSetVariable(1, 2.5)
    nl.nlMultiSetVariable(3, 1, -1.0)
    nl.nlLockVariable(1)
    assert nl.nlVariableIsLocked(1) and not nl.nlVariableIsLocked(0)
    nl.nlUnlockVariable(1)
    assert not nl.nlVariableIsLocked(1)
    assert nl.nlGetVariable(1) == 2.5 and nl.nlMultiGetVariable(3, 1) == -1.0
    nl.nlMultiSetVariable(0, 2, 1.0)      # system index out of range
    assert nl.nlGetError() == nl.NL_INVALID_VALUE


def test_ssor_preconditioner_parameter(ctx):
    """NL_PRECOND_SSOR is accepted (the GPU runs it, tests/test_gpu_ssor.py);
    without a device nlSolve fails loudly instead of returning a result."""
    nl.nlSolverParameteri(nl.NL_NB_VARIABLES, 1)
    nl.nlSolverParameteri(nl.NL_PRECONDITIONER, nl.NL_PRECOND_SSOR)
    nl.nlSolverParameterd(nl.NL_OMEGA, 1.2)
    assert nl.nlGetIntegerv(nl.NL_PRECONDITIONER) == nl.NL_PRECOND_SSOR
    assert nl.nlGetDoublev(nl.NL_OMEGA) == 1.2
    if nl.nlInitExtension("GB300"):
        pytest.skip("a GPU is present: the solve itself is covered by the GPU tests")
    nl.nlBegin(nl.NL_SYSTEM); nl.nlBegin(nl.NL_MATRIX)
    nl.nlBegin(nl.NL_ROW); nl.nlCoefficient(0, 1.0); nl.nlRightHandSide(1.0); nl.nlEnd(nl.NL_ROW)
    nl.nlEnd(nl.NL_MATRIX); nl.nlEnd(nl.NL_SYSTEM)
    assert nl.nlSolve() == 0


def test_krylov_solver_parameters(ctx):
    for solver in (nl.NL_CG, nl.NL_BICGSTAB, nl.NL_GMRES):
        nl.nlSolverParameteri(nl.NL_SOLVER, solver)
        assert nl.nlGetIntegerv(nl.NL_SOLVER) == solver
    nl.nlSolverParameteri(nl.NL_INNER_ITERATIONS, 12)
    assert nl.nlGetIntegerv(nl.NL_INNER_ITERATIONS) == 12
    nl.nlSolverParameteri(nl.NL_INNER_ITERATIONS, 0)      # a restart length must be >= 1
    assert nl.nlGetError() == nl.NL_INVALID_VALUE
    assert nl.nlGetIntegerv(nl.NL_INNER_ITERATIONS) == 12


def test_solve_without_gpu_reports_device_error(nllib, ctx):
    if nllib.nlgb_device_available():
        pytest.skip("a GPU is present")
    nl.nlSolverParameteri(nl.NL_NB_VARIABLES, 1)
    nl.nlBegin(nl.NL_SYSTEM); nl.nlBegin(nl.NL_MATRIX)
    nl.nlBegin(nl.NL_ROW); nl.nlCoefficient(0, 2.0); nl.nlRightHandSide(1.0); nl.nlEnd(nl.NL_ROW)
    nl.nlEnd(nl.NL_MATRIX); nl.nlEnd(nl.NL_SYSTEM)
    assert nl.nlSolve() == 0                       # no CPU fallback
    assert "CUDA" in nl.nlGetErrorString()
    assert nl.nlGetIntegerv(nl.NL_GB300_STATUS) == nl.NL_GB300_STATUS_DEVICE_ERR


def test_bulk_rows_equal_per_call_rows(ctx):
    # nlgb_add_rows validates indices and appends rows like nlBegin/nlEnd(NL_ROW)
    nl.nlSolverParameteri(nl.NL_NB_VARIABLES, 3)
    nl.nlBegin(nl.NL_SYSTEM); nl.nlBegin(nl.NL_MATRIX)
    rc = nl.nlgbAddRows(np.array([0, 2]), np.array([0, 5]), np.array([1.0, 1.0]))
    assert rc != 0 and nl.nlGetError() == nl.NL_INVALID_VALUE
    rc = nl.nlgbAddRows(np.array([0, 2, 3]), np.array([0, 1, 2]), np.array([1.0, 1.0, 2.0]),
                        np.array([[1.0], [2.0]]))
    assert rc == 0


def test_matrix_api_host_side(nllib):
    M = nl.nlSparseMatrixNew(3, 3, nl.NL_MATRIX_STORE_ROWS)
    for i in range(3):
        nl.nlSparseMatrixAdd(M, i, i, 2.0)
    nl.nlSparseMatrixAdd(M, 0, 1, 1.0)
    nl.nlSparseMatrixAdd(M, 0, 1, 1.0)    # duplicates are summed
    assert nl.nlMatrixNNZ(M) == 4
    nl.nlSparseMatrixAdd(M, 5, 0, 1.0)    # out of bounds: rejected
    assert nl.nlMatrixNNZ(M) == 4
    M = nl.nlMatrixCompress(M)
    assert nl.nlMatrixNNZ(M) == 4
    assert nl.nlNewSSORPreconditioner(M, 2.5) is None     # relaxation outside (0, 2)
    assert nl.nlMatrixFactorize(M, nl.NL_SUPERLU_EXT) is None
    nl.nlDeleteMatrix(M)
