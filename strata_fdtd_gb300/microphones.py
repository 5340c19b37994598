"""Virtual microphones at physical positions (core/solver.py:797-1438 of
rjwalters/strata-fdtd), omnidirectional, recorded on the GPU.

The reference records omni microphones through its native batch kernel:
grid positions as float32, corner weights formed in float
(``_kernels/src/microphones.cpp:16-80``) and the float sum from zero of
weight x pressure over the 8 corners after each step (``:82-118``).  The
weights here are formed with the same float32 arithmetic on the host and the
sum runs in ``k_mic_gather``, so the waveforms are bit-identical.
Directional patterns (which the reference evaluates in its Python path from
interpolated velocities) are not part of the GB300 path.
"""
from __future__ import annotations

import numpy as np

_CORNERS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0), (0, 0, 1), (1, 0, 1), (0, 1, 1),
            (1, 1, 1)]


class Microphone:
    """Omnidirectional microphone at ``position`` (metres)."""

    def __init__(self, position, name=None, pattern="omni", direction=None, up=None):
        if pattern != "omni":
            raise NotImplementedError(
                "directional microphone patterns are not implemented by the GB300 backend")
        self.position = tuple(float(v) for v in position)
        self.name = name
        self.pattern = "omni"
        self._data: list[float] = []
        self._times: list[float] = []
        self._solver = None
        self._grid_position = None
        self.corner_cells = None
        self.weights = None

    def is_directional(self) -> bool:
        return False

    def _initialize(self, solver) -> None:
        """core/solver.py:930-960: grid position = position / dx, inside the
        domain; corner cells and float32 weights as microphones.cpp:16-80."""
        gx, gy, gz = (p / solver.dx for p in self.position)
        if not (0 <= gx < solver.shape[0] - 1 and 0 <= gy < solver.shape[1] - 1
                and 0 <= gz < solver.shape[2] - 1):
            raise ValueError(f"Microphone position {self.position} is outside simulation domain.")
        self._grid_position = (gx, gy, gz)
        g = [np.float32(v) for v in self._grid_position]
        i0 = [int(v) for v in g]
        fx, fy, fz = (np.float32(v - np.float32(i)) for v, i in zip(g, i0))
        one = np.float32(1.0)
        w = [(one - fx) * (one - fy) * (one - fz), fx * (one - fy) * (one - fz),
             (one - fx) * fy * (one - fz), fx * fy * (one - fz), (one - fx) * (one - fy) * fz,
             fx * (one - fy) * fz, (one - fx) * fy * fz, fx * fy * fz]
        self.weights = np.array(w, dtype=np.float32)
        self.corner_cells = np.array(
            [np.ravel_multi_index((i0[0] + a, i0[1] + b, i0[2] + c), solver.shape)
             for a, b, c in _CORNERS], dtype=np.int64)
        self._solver = solver

    @property
    def data(self) -> list:
        if self._solver is not None:
            self._solver._flush_traces()
        return self._data

    def get_waveform(self, weighting=None) -> np.ndarray:
        if weighting not in (None, "Z"):
            raise NotImplementedError("frequency weighting is outside the GB300 path")
        return np.array(self.data, dtype=np.float32)

    def get_time_axis(self) -> np.ndarray:
        self.data  # noqa: B018 - flushes pending samples
        return np.array(self._times, dtype=np.float64)

    def get_sample_rate(self) -> float:
        return 1.0 / self._solver.dt

    def clear(self) -> None:
        self.data  # noqa: B018
        self._data.clear()
        self._times.clear()

    def __len__(self) -> int:
        return len(self.data)
