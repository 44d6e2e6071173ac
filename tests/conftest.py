import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
os.environ.setdefault("NLGB_QUIET", "1")

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")


@pytest.fixture(scope="session")
def nllib():
    """The in-tree libnl_gb300.so (built on demand)."""
    from graphitethree_gb300 import _lib
    from graphitethree_gb300.build import build as build_lib
    build_lib()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def golden_names():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name):
    """Golden fixture -> (RowStream, dict of expected arrays)."""
    from graphitethree_gb300.systems import RowStream
    d = np.load(GOLDEN / f"{name}.npz")
    rs = RowStream(n_vars=int(d["n_vars"]), row_ptr=d["row_ptr"], var=d["var"], val=d["val"],
                   rhs=d["rhs"], locked=d["locked"], values=d["values"],
                   least_squares=bool(d["least_squares"]),
                   weight=d["weight"] if int(d["has_weight"]) else None)
    return rs, {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def gpu_ok(nllib):
    if not nllib.nlgb_device_available():
        pytest.skip("no CUDA device")
    return True
