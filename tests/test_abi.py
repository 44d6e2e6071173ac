"""The C-ABI library loads and exports every symbol its headers declare.
No compute call is made here (no GPU needed)."""
import ctypes
import re

from graphitethree_gb300 import _lib
from graphitethree_gb300.build import INCLUDE, lib_path


def test_library_is_in_tree(nllib):
    assert lib_path().exists()
    assert str(lib_path()).startswith(str(INCLUDE.parent))


def test_every_declared_function_is_exported(nllib):
    names = _lib.header_functions()
    assert len(names) > 60, names
    missing = [n for n in names if not hasattr(nllib, n)]
    assert not missing, missing


def test_reference_call_sites_are_covered():
    # Symbols the reference binds (voxel_grob_transport_commands.cpp:231-287,
    # scene_graph/NL/matrix.cpp, blas.cpp).
    needed = """nlNewContext nlSolverParameteri nlEnable nlBegin nlSetVariable nlLockVariable
    nlCoefficient nlEnd nlSolve nlGetVariable nlDeleteContext nlGetCurrent nlInitExtension
    nlSparseMatrixNew nlSparseMatrixAdd nlDeleteMatrix nlMatrixCompress nlMultMatrixVector
    nlNewJacobiPreconditioner nlNewSSORPreconditioner nlSolveSystemIterative nlHostBlas
    nlMatrixFactorize""".split()
    declared = set(_lib.header_functions())
    assert not [n for n in needed if n not in declared]


def test_header_constants_are_distinct():
    k = _lib.header_constants()
    for group in ("NL_GB300_STATUS_", "NLGB_E_"):
        vals = [v for n, v in k.items() if n.startswith(group)]
        assert len(vals) == len(set(vals))
    assert k["NL_TRUE"] == 1 and k["NL_FALSE"] == 0


def test_nlmatrix_header_layout():
    # OGF::NL::Matrix reads m, n and type directly (matrix.cpp:130-141).
    text = (INCLUDE / "nl.h").read_text()
    body = re.search(r"struct NLMatrixStruct \{(.*?)\};", text, re.S).group(1)
    fields = re.findall(r"\b(\w+);", body)
    assert fields[:5] == ["m", "n", "type", "destroy_func", "mult_func"]


def test_extension_hook_rejects_direct_solvers(nllib):
    assert nllib.nlInitExtension(b"SUPERLU") == 0
    assert nllib.nlInitExtension(b"CHOLMOD") == 0
    assert nllib.nlInitExtension(None) == 0


def test_no_alloc_free_library_load(nllib):
    # loading must not require a GPU: the library initialises CUDA lazily
    assert isinstance(nllib, ctypes.CDLL)


def test_server_config_mirror_matches_header():
    """The ctypes mirror of nlgb_server_config lists the header's fields in
    the header's order (the struct is passed by pointer)."""
    text = (INCLUDE / "nl_gb300.h").read_text()
    body = text.split("} nlgb_server_config;")[0].rsplit("typedef struct {", 1)[1]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"\b(\w+);", body)
    assert fields == [f[0] for f in _lib.NlgbServerConfig._fields_]
