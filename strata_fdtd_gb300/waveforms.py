"""Audio files as source waveforms (core/waveforms.py of rjwalters/strata-fdtd).

``AudioFileWaveform`` has GaussianPulse's ``waveform(t, dt)`` interface, so a
point, plane or membrane source takes it in place of a pulse; the solver
evaluates such a waveform once per step on the host and hands the values to
the step kernels in its source table.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np


@dataclass
class AudioFileWaveform:
    """Samples of an audio file, resampled to the solve's step rate.

    ``channel`` picks one channel of a multichannel file or "mix" averages
    them; ``start_time`` and ``duration`` (seconds) trim it; past its end the
    waveform is zero, or wraps around when ``loop``.  WAV files are read with
    scipy; other formats need the soundfile package."""

    filepath: object
    amplitude: float = 1.0
    channel: object = "mix"
    start_time: float = 0.0
    duration: float | None = None
    loop: bool = False
    _samples: np.ndarray | None = field(default=None, init=False, repr=False)
    _native_sr: int | None = field(default=None, init=False, repr=False)
    _resampled: dict = field(default_factory=dict, init=False, repr=False)

    def __post_init__(self) -> None:
        path = Path(self.filepath)
        if not path.exists():
            raise FileNotFoundError(f"Audio file not found: {path}")
        if path.suffix.lower() == ".wav":
            from scipy.io import wavfile

            sr, data = wavfile.read(path)
        else:
            try:
                import soundfile
            except ImportError as e:
                raise ImportError(f"soundfile package required for {path.suffix} files. "
                                  "Install with: pip install soundfile") from e
            data, sr = soundfile.read(path)
        self._native_sr = sr
        # integer PCM to [-1, 1) floats
        if data.dtype == np.int16:
            data = data.astype(np.float32) / 32768.0
        elif data.dtype == np.int32:
            data = data.astype(np.float32) / 2147483648.0
        elif data.dtype == np.uint8:
            data = (data.astype(np.float32) - 128) / 128.0
        else:
            data = data.astype(np.float32)
        if data.ndim > 1:
            if self.channel == "mix":
                data = np.mean(data, axis=1)
            elif self.channel >= data.shape[1]:
                raise ValueError(f"Channel {self.channel} requested but file only has "
                                 f"{data.shape[1]} channels")
            else:
                data = data[:, self.channel]
        first = int(self.start_time * sr)
        if first >= len(data):
            raise ValueError(f"start_time {self.start_time}s is beyond end of file "
                             f"({len(data) / sr:.2f}s)")
        last = None if self.duration is None else first + int(self.duration * sr)
        self._samples = data[first:last].astype(np.float32)

    def _at_rate(self, dt: float) -> np.ndarray:
        """The samples at the step rate round(1/dt) (Fourier resampling,
        cached per rate)."""
        rate = int(round(1.0 / dt))
        if rate not in self._resampled:
            if rate == self._native_sr:
                out = self._samples
            else:
                from scipy import signal

                n = int(len(self._samples) * rate / self._native_sr)
                out = signal.resample(self._samples, n).astype(np.float32)
            self._resampled[rate] = out
        return self._resampled[rate]

    _resample_for_dt = _at_rate  # the name the filters look for (dsp.py)

    def waveform(self, t, dt: float) -> np.ndarray:
        """Values at times t: the sample at index int(t / dt), scaled by the
        amplitude (zero outside the recording unless it loops)."""
        samples = self._at_rate(dt)
        t = np.asarray(t)
        idx = (t / dt).astype(np.int64)
        if self.loop:
            return self.amplitude * samples[idx % len(samples)]
        ok = (idx >= 0) & (idx < len(samples))
        out = np.zeros_like(t, dtype=np.float32)
        out[ok] = samples[idx[ok]]
        return self.amplitude * out

    @property
    def duration_seconds(self) -> float:
        if self._samples is None or self._native_sr is None:
            return 0.0
        return len(self._samples) / self._native_sr

    @property
    def native_sample_rate(self) -> int:
        return self._native_sr or 0

    @property
    def num_samples(self) -> int:
        return 0 if self._samples is None else len(self._samples)
