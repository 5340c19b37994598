"""Virtual microphones at physical positions (core/solver.py:786-1438 of
rjwalters/strata-fdtd), recorded on the GPU.

Every microphone is one or four *rows* of the plan's microphone table
(``sf_plan_set_microphones_ex``): 8 corner cells, 8 float32 weights and the
field they read.  ``k_mic_gather`` forms the float sum from 0 of weight x
field over the corners after each step.

The reference has two recording paths, and the weights follow whichever one
it would take (``FDTDSolver._record_microphones``, core/solver.py:2441-2461):

* all microphones omnidirectional -> its native batch kernel: grid positions
  as float32 and corner weights in float arithmetic
  (``_kernels/src/microphones.cpp:16-80``), sum as ``:82-118``;
* any microphone directional -> ``Microphone.record`` for every microphone:
  FP64 weights (``_compute_trilinear_weights``, core/solver.py:965-1002)
  which NumPy rounds to float32 when it multiplies them with the float32
  field, and float32 sums.  A directional microphone adds three rows: vx, vy
  and vz at its position shifted half a cell back along the component's axis
  and clamped (``_interpolate_velocity``, :1060-1118).

The polar-pattern combination (``_compute_directional_output``,
:1120-1179) runs on the host over the recorded rows with the reference's own
NumPy scalar types, so standard and custom patterns give the reference's
samples bit for bit.
"""
from __future__ import annotations

from typing import Callable

import numpy as np

_CORNERS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0), (0, 0, 1), (1, 0, 1), (0, 1, 1),
            (1, 1, 1)]

# pattern coefficient k of output = (1 - k) p + k rho c (v . d)  (core/solver.py:787-794)
POLAR_PATTERNS: dict[str, float] = {
    "omni": 0.0,
    "subcardioid": 0.3,
    "cardioid": 0.5,
    "supercardioid": 0.63,
    "hypercardioid": 0.75,
    "figure8": 1.0,
}


def _weights_fp64(gx: float, gy: float, gz: float):
    """Corner cells and FP64 weights of Microphone._compute_trilinear_weights."""
    i0, j0, k0 = int(gx), int(gy), int(gz)
    fx, fy, fz = gx - i0, gy - j0, gz - k0
    w = [(1 - fx) * (1 - fy) * (1 - fz), fx * (1 - fy) * (1 - fz), (1 - fx) * fy * (1 - fz),
         fx * fy * (1 - fz), (1 - fx) * (1 - fy) * fz, fx * (1 - fy) * fz, (1 - fx) * fy * fz,
         fx * fy * fz]
    cells = [(i0 + a, j0 + b, k0 + c) for a, b, c in _CORNERS]
    return cells, w


class Microphone:
    """Microphone at ``position`` (metres) with a polar ``pattern`` (a name of
    POLAR_PATTERNS or a callable gain(theta)), pointing along ``direction``."""

    def __init__(self, position, name=None, pattern: str | Callable[[float], float] = "omni",
                 direction=None, up=None):
        self.position = position
        self.name = name
        if isinstance(pattern, str):
            if pattern not in POLAR_PATTERNS:
                raise ValueError(f"Unknown pattern '{pattern}'. "
                                 f"Valid patterns: {list(POLAR_PATTERNS.keys())}")
            self._pattern_name = pattern
            self._pattern_k = POLAR_PATTERNS[pattern]
            self._custom_pattern = None
        elif callable(pattern):
            self._pattern_name = "custom"
            self._pattern_k = None
            self._custom_pattern = pattern
        else:
            raise TypeError(f"pattern must be str or callable, got {type(pattern).__name__}")
        self.pattern = pattern
        d = np.array((1.0, 0.0, 0.0) if direction is None else direction, dtype=np.float64)
        dn = np.linalg.norm(d)
        if dn < 1e-10:
            raise ValueError("direction vector cannot be zero")
        self._direction = d / dn
        u = np.array((0.0, 0.0, 1.0) if up is None else up, dtype=np.float64)
        un = np.linalg.norm(u)
        if un < 1e-10:
            raise ValueError("up vector cannot be zero")
        self._up = u / un
        if abs(np.dot(self._direction, self._up)) > 0.999:
            raise ValueError("direction and up vectors cannot be parallel")
        self._data: list = []
        self._times: list[float] = []
        self._solver = None
        self._solver_dt = None
        self._solver_rho = None
        self._solver_c = None
        self._grid_position = None

    @property
    def direction(self):
        return tuple(self._direction)

    def is_directional(self) -> bool:
        return self._pattern_name != "omni"

    def _initialize(self, solver) -> None:
        """core/solver.py:930-963: grid position = position / dx, strictly
        inside the domain."""
        self._solver_dt = solver.dt
        self._solver_rho = solver.rho
        self._solver_c = solver.c
        gx = self.position[0] / solver.dx
        gy = self.position[1] / solver.dx
        gz = self.position[2] / solver.dx
        self._grid_position = (gx, gy, gz)
        if not (0 <= gx < solver.shape[0] - 1 and 0 <= gy < solver.shape[1] - 1
                and 0 <= gz < solver.shape[2] - 1):
            raise ValueError(f"Microphone position {self.position} is outside simulation domain.")
        self._solver = solver

    # -- rows of the device table --------------------------------------------
    def _rows(self, shape, python_path: bool):
        """[(field, 8 flat cells, 8 float32 weights)] this microphone records."""
        gx, gy, gz = self._grid_position
        if not python_path:  # native batch kernel (microphones.cpp:16-80)
            g = [np.float32(v) for v in self._grid_position]
            i0 = [int(v) for v in g]
            fx, fy, fz = (np.float32(v - np.float32(i)) for v, i in zip(g, i0))
            one = np.float32(1.0)
            w = [(one - fx) * (one - fy) * (one - fz), fx * (one - fy) * (one - fz),
                 (one - fx) * fy * (one - fz), fx * fy * (one - fz), (one - fx) * (one - fy) * fz,
                 fx * (one - fy) * fz, (one - fx) * fy * fz, fx * fy * fz]
            cells = [np.ravel_multi_index((i0[0] + a, i0[1] + b, i0[2] + c), shape)
                     for a, b, c in _CORNERS]
            return [(0, np.array(cells, np.int64), np.array(w, np.float32))]
        cells, w = _weights_fp64(gx, gy, gz)
        rows = [(0, np.array([np.ravel_multi_index(c, shape) for c in cells], np.int64),
                 np.array(w, dtype=np.float64).astype(np.float32))]
        if self.is_directional():
            nx, ny, nz = shape
            for axis in range(3):  # _interpolate_velocity (core/solver.py:1060-1118)
                g = [gx, gy, gz]
                g[axis] -= 0.5
                g[0] = max(0.0, min(g[0], nx - 1.001))
                g[1] = max(0.0, min(g[1], ny - 1.001))
                g[2] = max(0.0, min(g[2], nz - 1.001))
                vc, vw = _weights_fp64(*g)
                flat = [np.ravel_multi_index((min(i, nx - 1), min(j, ny - 1), min(k, nz - 1)),
                                             shape) for i, j, k in vc]
                rows.append((1 + axis, np.array(flat, np.int64),
                             np.array(vw, dtype=np.float64).astype(np.float32)))
        return rows

    def _append(self, samples: np.ndarray, times) -> None:
        """Add recorded rows (float32 [steps, rows]) as output samples."""
        if not self.is_directional():
            self._data.extend(samples[:, 0].tolist())
            self._times.extend(times)
            return
        p, vx, vy, vz = (samples[:, q] for q in range(4))
        d0, d1, d2 = self._direction[0], self._direction[1], self._direction[2]
        Z = self._solver_rho * self._solver_c
        if self._custom_pattern is None:
            k = self._pattern_k
            vd = vx * d0 + vy * d1 + vz * d2            # float64 (float32 x np.float64)
            out = (1 - k) * p + k * Z * vd               # float32 term + float64 term
            self._data.extend(out.tolist())
        else:  # per sample, with the reference's scalar types (core/solver.py:1160-1174)
            for t in range(samples.shape[0]):
                px, ux, uy, uz = (np.float32(samples[t, q]) for q in range(4))
                vd = ux * d0 + uy * d1 + uz * d2
                v_mag = np.sqrt(ux ** 2 + uy ** 2 + uz ** 2)
                if v_mag > 1e-20:
                    theta = np.arccos(np.clip(vd / v_mag, -1.0, 1.0))
                else:
                    theta = 0.0
                self._data.append(px * self._custom_pattern(theta))
        self._times.extend(times)

    # -- reference accessors ---------------------------------------------------
    @property
    def data(self) -> list:
        if self._solver is not None:
            self._solver._flush_traces()
        return self._data

    def get_waveform(self, weighting=None) -> np.ndarray:
        """The recorded pressure (float32), A- or C-weighted when asked
        (core/solver.py:1175-1206)."""
        waveform = np.array(self.data, dtype=np.float32)
        if weighting in ("Z", None) or len(waveform) == 0:
            return waveform
        from .weighting import apply_weighting

        return apply_weighting(waveform, self.get_sample_rate(), weighting).astype(np.float32)

    def _recorded(self):
        if len(self.data) == 0:
            raise RuntimeError("No data recorded. Run simulation first.")

    def get_spl(self, weighting=None, p_ref: float = 2e-5) -> float:
        """Sound pressure level of the recording in dB (core/solver.py:1226-1258)."""
        from .weighting import calculate_spl

        self._recorded()
        return calculate_spl(self.get_waveform(weighting=weighting), p_ref)

    def get_leq(self, weighting=None, duration: float | None = None,
                p_ref: float = 2e-5) -> float:
        """Equivalent continuous level, over the latest ``duration`` seconds
        when given (core/solver.py:1260-1296)."""
        from .weighting import calculate_leq

        self._recorded()
        return calculate_leq(self.get_waveform(weighting=weighting), self.get_sample_rate(),
                             duration, p_ref)

    def get_time_weighted_level(self, weighting=None, time_constant: str = "fast",
                                p_ref: float = 2e-5) -> np.ndarray:
        """Fast / slow / impulse time-weighted level per sample
        (core/solver.py:1298-1335)."""
        from .weighting import calculate_time_weighted_level

        self._recorded()
        return calculate_time_weighted_level(self.get_waveform(weighting=weighting),
                                             self.get_sample_rate(), time_constant, p_ref)

    def to_wav(self, filepath: str, sample_rate: int = 44100, normalize: bool = True,
               bit_depth: int = 16) -> None:
        """Mono WAV of the recording, linearly resampled to ``sample_rate``
        when the step rate differs by more than 1 Hz, peak-normalised to 0.95
        (core/solver.py:1337-1418)."""
        import wave

        self._recorded()
        if bit_depth not in (16, 32):
            raise ValueError("bit_depth must be 16 or 32")
        waveform = self.get_waveform()
        if self._solver_dt is not None:
            rate = 1.0 / self._solver_dt
            if abs(rate - sample_rate) > 1.0:
                n = int(len(waveform) * sample_rate / rate)
                if n != len(waveform):
                    waveform = np.interp(np.linspace(0, len(waveform) - 1, n),
                                         np.arange(len(waveform)), waveform).astype(np.float32)
        if normalize:
            peak = np.max(np.abs(waveform))
            if peak > 0:
                waveform = waveform / peak * 0.95
        dtype, full = (np.int16, 32767) if bit_depth == 16 else (np.int32, 2147483647)
        with wave.open(filepath, "wb") as out:
            out.setnchannels(1)
            out.setsampwidth(bit_depth // 8)
            out.setframerate(sample_rate)
            out.writeframes((waveform * full).astype(dtype).tobytes())

    def record(self, pressure_field, time: float, vx=None, vy=None, vz=None) -> None:
        """Record one sample from host fields, as the reference's Python path
        does (core/solver.py:1004-1058): the pressure (and, for a directional
        pattern, the three velocities) interpolated with the microphone's
        weights, combined with its polar pattern."""
        if getattr(self, "_grid_position", None) is None:
            raise RuntimeError("Microphone not initialized. Add to solver first.")
        p = np.asarray(pressure_field)
        fields = [p]
        if self.is_directional():
            if vx is None or vy is None or vz is None:
                raise ValueError("Velocity fields (vx, vy, vz) are required for directional "
                                 "microphones")
            fields += [np.asarray(vx), np.asarray(vy), np.asarray(vz)]
        row = []
        for f, cells, w in self._rows(p.shape, python_path=True):
            acc = np.float32(0.0)
            flat = fields[f].reshape(-1)
            for c, wc in zip(cells, w):
                acc = np.float32(acc + np.float32(wc * flat[c]))
            row.append(acc)
        self._append(np.array([row], dtype=np.float32), [float(time)])

    def get_time_axis(self) -> np.ndarray:
        self.data  # noqa: B018 - flushes pending samples
        return np.array(self._times, dtype=np.float64)

    def get_sample_rate(self) -> float:
        if self._solver_dt is None:
            raise RuntimeError("Microphone not initialized. Add to solver first.")
        return 1.0 / self._solver_dt

    def clear(self) -> None:
        self.data  # noqa: B018
        self._data.clear()
        self._times.clear()

    def __len__(self) -> int:
        return len(self.data)
