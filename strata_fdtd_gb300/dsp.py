"""Source-signal processing for multi-driver cabinets (dsp/ of
rjwalters/strata-fdtd): crossovers, a parametric equaliser and a delay, each
a waveform object (``waveform(t, dt)``) that wraps another, so its output
drives a point, plane or membrane source like a pulse does.

Filters run once per step rate on the host over the source's samples at
that rate (forward-backward, so without phase shift) and are cached;
``waveform`` then reads the filtered sample at index int(t / dt).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Protocol, runtime_checkable

import numpy as np


@runtime_checkable
class WaveformProtocol(Protocol):
    """Anything with ``waveform(t, dt)`` giving values at times t."""

    def waveform(self, t, dt: float): ...


def _source_samples(source, dt: float) -> np.ndarray:
    """The source at the step rate: an audio file's resampled samples, else
    its waveform over its duration (1 s when it has none)."""
    if hasattr(source, "_resample_for_dt"):
        return source._resample_for_dt(dt)
    rate = int(round(1.0 / dt))
    n = int(getattr(source, "duration_seconds", 1.0) * rate)
    return source.waveform(np.arange(n) * dt, dt)


def _sample_at(samples: np.ndarray, t, dt: float, source) -> np.ndarray:
    idx = (np.asarray(t) / dt).astype(np.int64)
    ok = (idx >= 0) & (idx < len(samples))
    out = np.zeros_like(np.asarray(t), dtype=np.float32)
    out[ok] = samples[idx[ok]]
    return getattr(source, "amplitude", 1.0) * out


@dataclass
class FilteredWaveform:
    """``source`` low-, high- or band-passed at ``frequency`` (a pair for
    band-pass) by a Butterworth, Bessel or Linkwitz-Riley filter of
    ``order`` (dsp/crossover.py:43-212).  Linkwitz-Riley is the
    half-order Butterworth applied twice."""

    source: Any
    filter_type: str
    frequency: Any
    order: int = 4
    design: str = "linkwitz-riley"
    _filtered_cache: dict = field(default_factory=dict, init=False, repr=False)

    def _design_filter(self, sample_rate: int):
        from scipy import signal

        nyq = sample_rate / 2
        if isinstance(self.frequency, tuple):
            wn = (self.frequency[0] / nyq, self.frequency[1] / nyq)
            if wn[0] >= 1.0 or wn[1] >= 1.0:
                raise ValueError(f"Filter frequencies {self.frequency} exceed Nyquist "
                                 f"frequency {nyq} Hz for sample rate {sample_rate} Hz")
        else:
            wn = self.frequency / nyq
            if wn >= 1.0:
                raise ValueError(f"Filter frequency {self.frequency} Hz exceeds Nyquist "
                                 f"frequency {nyq} Hz for sample rate {sample_rate} Hz")
        if self.design == "linkwitz-riley":
            return signal.butter(max(1, self.order // 2), wn, btype=self.filter_type)
        if self.design == "butterworth":
            return signal.butter(self.order, wn, btype=self.filter_type)
        if self.design == "bessel":
            return signal.bessel(self.order, wn, btype=self.filter_type, norm="phase")
        raise ValueError(f"Unknown filter design: {self.design}")

    def _apply_filter(self, samples, sample_rate: int) -> np.ndarray:
        """Forward-backward filtering (twice for Linkwitz-Riley); signals
        too short for it are edge-padded and filtered forward."""
        from scipy import signal

        b, a = self._design_filter(sample_rate)
        passes = 2 if self.design == "linkwitz-riley" else 1
        pad = 3 * max(len(b), len(a))
        if len(samples) <= pad:
            out = np.pad(samples, (pad, pad), mode="edge")
            for _ in range(passes):
                out = signal.lfilter(b, a, out)
            return out[pad:-pad].astype(np.float32)
        out = samples
        for _ in range(passes):
            out = signal.filtfilt(b, a, out)
        return out.astype(np.float32)

    def waveform(self, t, dt: float) -> np.ndarray:
        rate = int(round(1.0 / dt))
        if rate not in self._filtered_cache:
            self._filtered_cache[rate] = self._apply_filter(_source_samples(self.source, dt),
                                                            rate)
        return _sample_at(self._filtered_cache[rate], t, dt, self.source)

    @property
    def duration_seconds(self) -> float:
        return getattr(self.source, "duration_seconds", 0.0)


@dataclass
class Crossover:
    """Two-way crossover at ``frequency`` (dsp/crossover.py:215-291)."""

    frequency: float
    order: int = 4
    type: str = "linkwitz-riley"

    def lowpass(self, waveform) -> FilteredWaveform:
        return FilteredWaveform(waveform, "lowpass", self.frequency, self.order, self.type)

    def highpass(self, waveform) -> FilteredWaveform:
        return FilteredWaveform(waveform, "highpass", self.frequency, self.order, self.type)


@dataclass
class ThreeWayCrossover:
    """Woofer below ``low_freq``, midrange band-passed between the two,
    tweeter above ``high_freq`` (dsp/crossover.py:294-403)."""

    low_freq: float
    high_freq: float
    order: int = 4
    type: str = "linkwitz-riley"

    def __post_init__(self) -> None:
        if self.low_freq >= self.high_freq:
            raise ValueError(f"low_freq ({self.low_freq}) must be less than "
                             f"high_freq ({self.high_freq})")

    def woofer(self, waveform) -> FilteredWaveform:
        return FilteredWaveform(waveform, "lowpass", self.low_freq, self.order, self.type)

    def midrange(self, waveform) -> FilteredWaveform:
        return FilteredWaveform(waveform, "bandpass", (self.low_freq, self.high_freq),
                                self.order, self.type)

    def tweeter(self, waveform) -> FilteredWaveform:
        return FilteredWaveform(waveform, "highpass", self.high_freq, self.order, self.type)


@dataclass
class DelayedWaveform:
    """``source`` shifted later by ``delay_seconds`` (its value at time 0
    before then; dsp/delay.py:20-116)."""

    source: Any
    delay_seconds: float

    def waveform(self, t, dt: float) -> np.ndarray:
        return self.source.waveform(np.maximum(np.asarray(t) - self.delay_seconds, 0.0), dt)

    @property
    def duration_seconds(self) -> float:
        return getattr(self.source, "duration_seconds", 0.0) + self.delay_seconds

    @property
    def delay_samples(self) -> int:
        raise NotImplementedError("delay_samples requires sample rate. Use delay_seconds / dt.")


@dataclass
class EQBand:
    """One band: peaking, low or high shelf, low- or high-pass."""

    frequency: float
    gain_db: float
    q: float
    type: str


def _biquad(band: EQBand, sample_rate: int):
    """Normalised (b, a) of the band by the Audio EQ Cookbook formulas
    (R. Bristow-Johnson), Q floored at 0.1 (dsp/eq.py:65-143)."""
    w0 = 2 * np.pi * band.frequency / sample_rate
    cw, sw = np.cos(w0), np.sin(w0)
    A = 10 ** (band.gain_db / 40)
    q = max(band.q, 0.1)
    kind = band.type
    if kind in ("lowpass", "highpass", "peaking"):
        alpha = sw / (2 * q)
        if kind == "lowpass":
            b = ((1 - cw) / 2, 1 - cw, (1 - cw) / 2)
            a = (1 + alpha, -2 * cw, 1 - alpha)
        elif kind == "highpass":
            b = ((1 + cw) / 2, -(1 + cw), (1 + cw) / 2)
            a = (1 + alpha, -2 * cw, 1 - alpha)
        else:
            b = (1 + alpha * A, -2 * cw, 1 - alpha * A)
            a = (1 + alpha / A, -2 * cw, 1 - alpha / A)
    elif kind in ("lowshelf", "highshelf"):
        alpha = sw / 2 * np.sqrt((A + 1 / A) * (1 / q - 1) + 2)
        r = 2 * np.sqrt(A) * alpha
        if kind == "lowshelf":
            b = (A * ((A + 1) - (A - 1) * cw + r), 2 * A * ((A - 1) - (A + 1) * cw),
                 A * ((A + 1) - (A - 1) * cw - r))
            a = ((A + 1) + (A - 1) * cw + r, -2 * ((A - 1) + (A + 1) * cw),
                 (A + 1) + (A - 1) * cw - r)
        else:
            b = (A * ((A + 1) + (A - 1) * cw + r), -2 * A * ((A - 1) + (A + 1) * cw),
                 A * ((A + 1) + (A - 1) * cw - r))
            a = ((A + 1) - (A - 1) * cw + r, 2 * ((A - 1) - (A + 1) * cw),
                 (A + 1) - (A - 1) * cw - r)
    else:
        raise ValueError(f"Unknown EQ band type: {kind}")
    return (np.array([b[0] / a[0], b[1] / a[0], b[2] / a[0]], dtype=np.float64),
            np.array([1.0, a[1] / a[0], a[2] / a[0]], dtype=np.float64))


@dataclass
class EQWaveform:
    """``source`` through the bands in order (dsp/eq.py:40-207)."""

    source: Any
    bands: list
    _processed_cache: dict = field(default_factory=dict, init=False, repr=False)

    def _apply_eq(self, samples, sample_rate: int) -> np.ndarray:
        from scipy import signal

        out = samples.astype(np.float64)
        for band in self.bands:
            b, a = _biquad(band, sample_rate)
            pad = 3 * max(len(b), len(a))
            if len(out) > pad:
                out = signal.filtfilt(b, a, out)
            else:
                out = signal.lfilter(b, a, np.pad(out, (pad, pad), mode="edge"))[pad:-pad]
        return out.astype(np.float32)

    def waveform(self, t, dt: float) -> np.ndarray:
        rate = int(round(1.0 / dt))
        if rate not in self._processed_cache:
            self._processed_cache[rate] = self._apply_eq(_source_samples(self.source, dt), rate)
        return _sample_at(self._processed_cache[rate], t, dt, self.source)

    @property
    def duration_seconds(self) -> float:
        return getattr(self.source, "duration_seconds", 0.0)


@dataclass
class ParametricEQ:
    """A list of EQ bands applied to any waveform (dsp/eq.py:210-331)."""

    bands: list = field(default_factory=list)

    def add_band(self, frequency, gain_db, q, type) -> "ParametricEQ":
        self.bands.append(EQBand(frequency=frequency, gain_db=gain_db, q=q, type=type))
        return self

    def clear(self) -> "ParametricEQ":
        self.bands.clear()
        return self

    def apply(self, waveform) -> EQWaveform:
        return EQWaveform(source=waveform, bands=list(self.bands))


def create_baffle_step_compensation(baffle_width, speed_of_sound=343.0, boost_db=3.0):
    """A low shelf of ``boost_db`` at c / (2 w), Q 0.707."""
    return ParametricEQ().add_band(speed_of_sound / (2 * baffle_width), boost_db, 0.707,
                                   "lowshelf")
