"""Device-resident FP64 vectors for the scripting path.

The reference exposes OGF::NL::Vector to Python as a numpy array over host
memory (plugins/OGF/gompy/interpreter/nl_vector_interop.cpp) and passes it
to OGF::NL::Matrix (src/lib/OGF/scene_graph/NL/matrix.cpp: mult,
solve_iterative).  Here a Vector lives in HBM: it exposes
__cuda_array_interface__ (torch / cupy can view it without a copy), and the
opennl wrappers (nlMultMatrixVector, nlSolveSystemIterative) hand its
device pointer straight to the library, so repeated products and solves on
a compressed matrix (itself kept on the device) move no vector data over
PCIe.  Device memory comes from PyTorch's allocator.  Ordering: the library
synchronises its own stream before each call returns, and a Vector
synchronises PyTorch's stream after each of its own writes, so the two
streams never touch a vector at the same time."""
from __future__ import annotations

import numpy as np


class Vector:
    """A contiguous float64 vector on the current CUDA device."""

    def __init__(self, n_or_values, device: str = "cuda"):
        import torch
        if np.isscalar(n_or_values):
            self._t = torch.zeros(int(n_or_values), dtype=torch.float64, device=device)
        else:
            host = np.ascontiguousarray(n_or_values, np.float64).reshape(-1)
            self._t = torch.from_numpy(host).to(device)
        torch.cuda.current_stream(self._t.device).synchronize()

    @property
    def __cuda_array_interface__(self):
        return self._t.__cuda_array_interface__

    @property
    def tensor(self):
        """The underlying torch tensor (shares the memory)."""
        return self._t

    def numpy(self) -> np.ndarray:
        """Host copy."""
        return self._t.cpu().numpy()

    def __len__(self) -> int:
        return int(self._t.shape[0])

    def copy_from(self, values) -> "Vector":
        import torch
        host = np.ascontiguousarray(values, np.float64).reshape(-1)
        self._t.copy_(torch.from_numpy(host))
        torch.cuda.current_stream(self._t.device).synchronize()
        return self
