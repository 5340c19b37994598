"""Frequency weighting and sound levels of recorded waveforms
(analysis/weighting.py of rjwalters/strata-fdtd), on the host.

A and C weighting are the analog IEC 61672-1 responses -- zeros at s = 0
(four for A, two for C), double poles at 2 pi f1 and 2 pi f4, single poles at
2 pi f2 and 2 pi f3 for A -- scaled to unit gain at 1 kHz and mapped to the
sample rate by the bilinear transform, applied as second-order sections.
Levels: SPL from the RMS, Leq over the whole or the latest part of a
recording, and the exponentially time-weighted level (fast 125 ms, slow 1 s,
impulse 35 ms).
"""
from __future__ import annotations

import numpy as np

P_REF = 2e-5  # reference pressure in air, Pa

# IEC 61672-1 pole frequencies, Hz
_F1, _F2, _F3, _F4 = 20.598997, 107.65265, 737.86223, 12194.217
_W1, _W2, _W3, _W4 = (2 * np.pi * f for f in (_F1, _F2, _F3, _F4))

_SOS_CACHE: dict = {}


def _design(zeros: int, poles, fs: float):
    """Second-order sections of the analog response s^zeros / prod(s + w),
    scaled to gain 1 at 1 kHz, by the bilinear transform at rate fs."""
    from scipy import signal

    w_ref = 2 * np.pi * 1000.0
    gain = np.prod([np.sqrt(w_ref**2 + w**2) for w in poles]) / w_ref**zeros
    z, p, k = signal.bilinear_zpk([0] * zeros, [-w for w in poles], gain, fs)
    return signal.zpk2sos(z, p, k)


def get_weighting_sos(weighting, fs: float):
    """SOS coefficients of weighting "A" or "C" at rate fs (None for "Z" or
    None: no filter)."""
    if weighting in ("Z", None):
        return None
    key = (weighting, fs)
    if key not in _SOS_CACHE:
        if weighting == "A":
            _SOS_CACHE[key] = _design(4, (_W1, _W1, _W2, _W3, _W4, _W4), fs)
        elif weighting == "C":
            _SOS_CACHE[key] = _design(2, (_W1, _W1, _W4, _W4), fs)
        else:
            raise ValueError(f"Unknown weighting type: {weighting!r}. "
                             "Valid options: 'A', 'C', 'Z', or None")
    return _SOS_CACHE[key]


def apply_weighting(waveform, fs: float, weighting) -> np.ndarray:
    """The waveform filtered by the weighting (float64)."""
    sos = get_weighting_sos(weighting, fs)
    if sos is None:
        return np.asarray(waveform).astype(np.float64)
    from scipy import signal

    return signal.sosfilt(sos, waveform).astype(np.float64)


def calculate_spl(waveform, p_ref: float = P_REF) -> float:
    """20 log10(p_rms / p_ref); -inf for silence."""
    rms = np.sqrt(np.mean(np.asarray(waveform) ** 2))
    return -np.inf if rms == 0 else 20 * np.log10(rms / p_ref)


def calculate_leq(waveform, fs: float, duration: float | None = None,
                  p_ref: float = P_REF) -> float:
    """Equivalent continuous level over the latest ``duration`` seconds (all
    of the recording when None or longer than it)."""
    waveform = np.asarray(waveform)
    if duration is not None:
        n = int(duration * fs)
        if n < len(waveform):
            waveform = waveform[-n:]
    return calculate_spl(waveform, p_ref)


_TAU = {"fast": 0.125, "slow": 1.0, "impulse": 0.035}


def calculate_time_weighted_level(waveform, fs: float, time_constant: str = "fast",
                                  p_ref: float = P_REF) -> np.ndarray:
    """Per-sample level of the squared pressure averaged by a one-pole filter
    with the time constant's decay, floored at 1e-20 Pa^2."""
    from scipy import signal

    alpha = 1 - np.exp(-1 / (fs * _TAU[time_constant]))
    avg = signal.lfilter([alpha], [1, -(1 - alpha)], np.asarray(waveform) ** 2)
    return 10 * np.log10(np.maximum(avg, 1e-20) / p_ref**2)


def weighting_response(weighting, fs: float, n_points: int = 1024):
    """(frequencies, magnitude in dB) of the weighting filter at n_points
    frequencies from 0 to fs / 2 (analysis/weighting.py:304-333); flat 0 dB
    for "Z" or None."""
    sos = get_weighting_sos(weighting, fs)
    if sos is None:
        return np.linspace(0, fs / 2, n_points), np.zeros(n_points)
    from scipy import signal

    f, h = signal.sosfreqz(sos, worN=n_points, fs=fs)
    return f, 20 * np.log10(np.maximum(np.abs(h), 1e-20))
