"""Batched tracking of many lattice variants (one persistent kernel).

:class:`BatchTracker` groups compiled lattices (:class:`DeviceTracker`) and
their particle column blocks (torch CUDA tensors, 21 x n each) into one
``st_BatchTracker``: every launch of the engine's persistent batch kernel
advances all variants, so that variants with few particles share the GPU
instead of each leaving most of it idle.  Runs of launches can be captured
into a CUDA graph and replayed; the launch shape is chosen by the engine's
autotuner.  Results are bit-identical to tracking each variant on its own.
"""

from __future__ import annotations

import ctypes as C

from . import _native
from .device import DeviceTracker, _check_cols


class BatchTracker:
    def __init__(self, trackers: list[DeviceTracker], config: str | None = None):
        if not trackers:
            raise ValueError("at least one lattice is needed")
        self._lib = _native.load()
        self.trackers = list(trackers)  # keep the lattices alive
        arr = (C.c_void_p * len(trackers))(*[t._ptr for t in trackers])
        self._ptr = self._lib.st_BatchTracker_new(arr, len(trackers), (config or "").encode())
        if not self._ptr:
            raise RuntimeError("st_BatchTracker_new: " + _native.last_error())
        self._cols = None

    def __del__(self):
        try:
            if self._ptr:
                self._lib.st_BatchTracker_delete(self._ptr)
                self._ptr = None
        except Exception:
            pass

    def set_particles(self, cols: list) -> None:
        """One 21 x n tensor per variant (kept referenced by the batch)."""
        if len(cols) != len(self.trackers):
            raise ValueError("one particle block per lattice variant")
        ns = [_check_cols(c) if c is not None else 0 for c in cols]
        ptrs = (C.c_void_p * len(cols))(*[c.data_ptr() if c is not None else None for c in cols])
        nn = (C.c_int64 * len(cols))(*ns)
        if self._lib.st_BatchTracker_set_particles(self._ptr, ptrs, nn) != 0:
            raise RuntimeError("set_particles: " + _native.last_error())
        self._cols = list(cols)

    def _stream(self):
        import torch

        return torch.cuda.current_stream().cuda_stream

    def track_until(self, from_turn: int, until_turn: int) -> int:
        return int(self._lib.st_BatchTracker_track_until(self._ptr, int(from_turn),
                                                         int(until_turn), self._stream()))

    def capture(self, turns_per_replay: int) -> None:
        if self._lib.st_BatchTracker_capture(self._ptr, int(turns_per_replay)) != 0:
            raise RuntimeError("capture: " + _native.last_error())

    def set_turn(self, turn: int) -> None:
        if self._lib.st_BatchTracker_set_turn(self._ptr, int(turn), self._stream()) != 0:
            raise RuntimeError("set_turn: " + _native.last_error())

    def replay(self) -> None:
        if self._lib.st_BatchTracker_replay(self._ptr, self._stream()) != 0:
            raise RuntimeError("replay: " + _native.last_error())

    def status(self) -> int:
        return int(self._lib.st_BatchTracker_status(self._ptr, self._stream()))

    @property
    def shape(self) -> dict:
        v = [C.c_int32() for _ in range(4)]
        self._lib.st_BatchTracker_get_shape(self._ptr, *[C.byref(x) for x in v])
        return {"threads_per_block": v[0].value, "blocks_per_sm": v[1].value,
                "stages": v[2].value, "turns_per_launch": v[3].value}

    def autotune(self, sample_fraction: float = 1 / 16, trial_turns: int = 4) -> float:
        """Pick the fastest launch shape on a sample; returns its trial time (ms)."""
        best = C.c_double()
        if self._lib.st_BatchTracker_autotune(self._ptr, float(sample_fraction),
                                              int(trial_turns), C.byref(best)) != 0:
            raise RuntimeError("autotune: " + _native.last_error())
        return best.value
