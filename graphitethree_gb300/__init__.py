"""graphitethree_gb300 -- GB300-native replacement of the OpenNL sparse-solver
hot path behind Graphite's LSCM parameterisation and Laplacian fairing.

The product is the C-ABI library ``lib/libnl_gb300.so`` (OpenNL API in
``include/nl.h``, handle API in ``include/nl_gb300.h``), built from the CUDA
and C++ sources in ``csrc/`` for sm_103a by ``build.build()``.  The Python
modules are thin bindings (``opennl``, ``solver``) and the seeded workload
generators (``meshes``, ``systems``).
"""
import os

# The solve server runs up to 16 CUDA streams at once; with the driver's
# default of 8 hardware work queues, streams share queues and their chunks
# serialise behind one another.  The setting is read when the process
# creates its CUDA context, so it only takes effect when this package is
# imported before the first CUDA call; an explicit value is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from .build import build, lib_path  # noqa: E402,F401

__version__ = "1.0.0"


def load():
    """Load libnl_gb300 (fails loudly when it has not been built)."""
    from . import _lib
    return _lib.load()
