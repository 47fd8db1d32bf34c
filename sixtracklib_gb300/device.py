"""Device-resident tracking for PyTorch callers.

:class:`DeviceTracker` holds a lattice compiled onto the GPU
(``st_DeviceLattice``) and tracks particle column blocks that already live in
device memory as torch tensors (21 x n, 8-byte elements; see
:mod:`sixtracklib_gb300.particles`).  Kernels run on the caller's current
torch CUDA stream.  PyTorch provides the memory and the stream; the tracking
itself is the engine's CUDA kernel.
"""

from __future__ import annotations

import numpy as np

from . import _native
from .cbuffer import CBuffer
from .particles import Particles


def _stream_handle(tensor):
    import torch

    return torch.cuda.current_stream(tensor.device).cuda_stream


def _check_cols(cols):
    import torch

    if not (isinstance(cols, torch.Tensor) and cols.is_cuda):
        raise TypeError("particle columns must be a CUDA tensor")
    if cols.dim() != 2 or cols.shape[0] != 21 or cols.element_size() != 8 or not cols.is_contiguous():
        raise ValueError("particle columns must be a contiguous 21 x n tensor of 8-byte words")
    return int(cols.shape[1])


class DeviceTracker:
    def __init__(self, lattice, config: str | None = None):
        cb = lattice if isinstance(lattice, CBuffer) else getattr(lattice, "cbuffer", lattice)
        img = np.ascontiguousarray(cb.to_image() if isinstance(cb, CBuffer) else cb, dtype=np.uint64)
        self._lib = _native.load()
        self._ptr = self._lib.st_DeviceLattice_new(img.ctypes.data, img.nbytes,
                                                    (config or "").encode())
        if not self._ptr:
            raise RuntimeError("st_DeviceLattice_new failed: " + _native.last_error())
        self.config = config or ""

    def __del__(self):
        try:
            if self._ptr:
                self._lib.st_DeviceLattice_delete(self._ptr)
                self._ptr = None
        except Exception:
            pass

    @property
    def num_elements(self) -> int:
        return int(self._lib.st_DeviceLattice_num_elements(self._ptr))

    @property
    def num_chunks(self) -> int:
        return int(self._lib.st_DeviceLattice_num_chunks(self._ptr))

    def track_until(self, cols, until_turn: int) -> int:
        n = _check_cols(cols)
        return int(self._lib.st_DeviceLattice_track_until(self._ptr, cols.data_ptr(), n,
                                                           int(until_turn), _stream_handle(cols)))

    def launch_until(self, cols, until_turn: int) -> None:
        """Asynchronous launch on the current stream (no status read)."""
        n = _check_cols(cols)
        rc = self._lib.st_DeviceLattice_launch_until(self._ptr, cols.data_ptr(), n,
                                                      int(until_turn), _stream_handle(cols))
        if rc != 0:
            raise RuntimeError("launch failed: " + _native.last_error())

    def last_status(self) -> int:
        return int(self._lib.st_DeviceLattice_last_status(self._ptr))

    def track_line(self, cols, begin: int, end: int, finish_turn: bool = False) -> int:
        n = _check_cols(cols)
        return int(self._lib.st_DeviceLattice_track_line(self._ptr, cols.data_ptr(), n, int(begin),
                                                          int(end), bool(finish_turn),
                                                          _stream_handle(cols)))


def to_device(particles: Particles, device="cuda"):
    """Copy a particle set's column block to the GPU (int64 view)."""
    import torch

    return torch.from_numpy(particles.block.copy().view(np.int64)).to(device)


def from_device(cols) -> np.ndarray:
    """Column block back on the host as u64 words."""
    return cols.detach().cpu().numpy().view(np.uint64)
