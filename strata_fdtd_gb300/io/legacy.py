"""File export of a solve's results without HDF5 (io/legacy.py of
rjwalters/strata-fdtd): field snapshots as raw binary (float16, float32 or
min-max scaled uint8, optionally strided), velocity snapshots interleaved
or one file per component, the geometry mask as packed bits or run-length
JSON, probe traces and solver metadata as JSON, and a whole solve as a
directory with a manifest.  The files are byte for byte those the
reference writes for the same solve (the snapshots and traces of the GPU
solver equal the reference's), so its viewers and loaders read them.

Snapshots reach the host through the solver's asynchronous snapshot path;
the conversions here are NumPy's, in the reference's order of operations
(the uint8 scaling's rounding depends on it)."""
from __future__ import annotations

import json
from pathlib import Path
from typing import Any

import numpy as np

_FLOAT = {"float16": np.float16, "float32": np.float32}


def _strided(a, step: int):
    return a[::step, ::step, ::step] if step > 1 else a


def export_snapshot(pressure, path, format: str = "float16", downsample: int = 1) -> dict:
    """Write one pressure field (every ``downsample``-th cell per axis) as
    raw binary; uint8 maps [min, max] linearly onto 0..255 and records the
    range."""
    p = _strided(np.asarray(pressure), downsample)
    extra = {}
    if format in _FLOAT:
        data = p.astype(_FLOAT[format])
    elif format == "uint8":
        lo, hi = p.min(), p.max()
        span = hi - lo
        unit = (p - lo) / span if span > 0 else np.zeros_like(p)
        data = (unit * 255).astype(np.uint8)
        extra["value_range"] = [float(lo), float(hi)]
    else:
        raise ValueError(f"Unknown format: {format}")
    data.tofile(Path(path))
    return {"shape": list(data.shape), "dtype": str(data.dtype), "format": format,
            "downsample": downsample, "file": str(Path(path)), "bytes": data.nbytes, **extra}


def export_velocity_snapshot(vx, vy, vz, path_prefix, format: str = "float16",
                             downsample: int = 1, interleaved: bool = True) -> dict:
    """Write cell-centred velocities: ``<prefix>.bin`` holding (vx, vy, vz)
    per cell, or ``<prefix>_vx.bin`` etc.  Any format but float16 is written
    as float32."""
    dt = np.float16 if format == "float16" else np.float32
    comps = {n: _strided(np.asarray(v), downsample).astype(dt)
             for n, v in (("vx", vx), ("vy", vy), ("vz", vz))}
    # "dtype" is the text of the NumPy scalar type, "<class 'numpy.float16'>",
    # as the reference records it
    head = {"shape": list(comps["vx"].shape), "dtype": str(dt)}
    if interleaved:
        packed = np.stack([c.ravel() for c in comps.values()], axis=1).ravel()
        f = Path(f"{path_prefix}.bin")
        packed.tofile(f)
        return {**head, "format": "interleaved", "downsample": downsample, "components": 3,
                "file": str(f), "bytes": packed.nbytes}
    files = {}
    for n, c in comps.items():
        f = Path(f"{path_prefix}_{n}.bin")
        c.tofile(f)
        files[n] = str(f)
    return {**head, "format": "separate", "downsample": downsample, "components": 3,
            "files": files, "bytes": sum(c.nbytes for c in comps.values())}


def _runs(flat: np.ndarray) -> list:
    """Run-length encoding of a flat bool array as {"v": value, "n": length}."""
    edges = np.flatnonzero(flat[1:] != flat[:-1]) + 1
    starts = np.concatenate([[0], edges])
    ends = np.concatenate([edges, [flat.size]])
    return [{"v": bool(flat[s]), "n": int(e - s)} for s, e in zip(starts, ends)]


def export_geometry(geometry, path, format: str = "binary") -> dict:
    """Write the air mask as packed bits (C order, most significant bit
    first) or as run-length JSON."""
    g = np.asarray(geometry)
    path = Path(path)
    if format == "binary":
        bits = np.packbits(g.flatten())
        bits.tofile(path)
        return {"shape": list(g.shape), "format": "packed_bits", "file": str(path),
                "bytes": bits.nbytes}
    if format == "json":
        runs = _runs(g.flatten())
        with open(path, "w") as fh:
            json.dump({"shape": list(g.shape), "format": "rle", "runs": runs}, fh)
        return {"shape": list(g.shape), "format": "rle_json", "file": str(path),
                "runs": len(runs)}
    raise ValueError(f"Unknown format: {format}")


def export_probe_data(solver, path, probe_names=None) -> dict:
    """Write the probe traces (all, or those named) with the sample rate,
    step, duration and sample count as JSON."""
    traces = solver.get_probe_data()
    if probe_names is not None:
        traces = {n: d for n, d in traces.items() if n in probe_names}
    doc = {"sample_rate": solver.get_sample_rate(), "dt": solver.dt, "duration": solver.time,
           "n_samples": solver.step_count,
           "probes": {n: {"position": list(solver._probes[n].position), "data": d.tolist()}
                      for n, d in traces.items()}}
    with open(Path(path), "w") as fh:
        json.dump(doc, fh, indent=2)
    return {"file": str(Path(path)), "n_probes": len(doc["probes"]),
            "n_samples": doc["n_samples"], "sample_rate": doc["sample_rate"]}


def _source_entry(src) -> dict:
    pos = src.position
    return {"type": src.source_type, "position": list(pos) if isinstance(pos, tuple) else pos,
            "frequency": src.frequency, "bandwidth": src.bandwidth}


def export_metadata(solver, path, extra=None) -> None:
    """Write the grid, physics, time-stepping state, probes and sources as
    JSON (``extra`` under its own key)."""
    doc = {
        "grid": {"shape": list(solver.shape), "resolution": solver.dx,
                 "physical_size": [n * solver.dx for n in solver.shape]},
        "physics": {"c": solver.c, "rho": solver.rho},
        "simulation": {"dt": solver.dt, "cfl_limit": solver.dx / (solver.c * np.sqrt(3)),
                       "current_time": solver.time, "step_count": solver.step_count},
        "probes": {n: {"position": list(p.position)} for n, p in solver._probes.items()},
        "sources": [_source_entry(s) for s in solver._sources],
    }
    if extra:
        doc["extra"] = extra
    with open(Path(path), "w") as fh:
        json.dump(doc, fh, indent=2)


def export_simulation(solver, output_dir, prefix: str = "sim", include_snapshots: bool = True,
                      include_velocity=None, snapshot_format: str = "float16",
                      snapshot_downsample: int = 1) -> dict:
    """Write a finished solve into ``output_dir``: ``<prefix>_metadata.json``,
    ``_probes.json``, ``_geometry.bin``, ``_snapshot_NNNN.bin`` per pressure
    snapshot, ``_velocity_NNNN.bin`` per velocity snapshot (by default when
    the solve captured any) and ``_manifest.json`` listing them.  Returns
    the manifest with its own path added."""
    out = Path(output_dir)
    out.mkdir(parents=True, exist_ok=True)
    name = lambda tail: out / f"{prefix}_{tail}"  # noqa: E731
    files: dict[str, Any] = {}
    export_metadata(solver, name("metadata.json"))
    files["metadata"] = str(name("metadata.json"))
    export_probe_data(solver, name("probes.json"))
    files["probes"] = str(name("probes.json"))
    export_geometry(solver.geometry, name("geometry.bin"))
    files["geometry"] = str(name("geometry.bin"))
    if include_snapshots:
        files["snapshots"] = [
            {**export_snapshot(p, name(f"snapshot_{n:04d}.bin"), format=snapshot_format,
                               downsample=snapshot_downsample), "time": t}
            for n, (t, p) in enumerate(solver.get_snapshots())]
    vel = solver.get_velocity_snapshots()
    if (include_velocity if include_velocity is not None else len(vel) > 0) and vel:
        files["velocitySnapshots"] = [
            {**export_velocity_snapshot(vx, vy, vz, name(f"velocity_{n:04d}"),
                                        format=snapshot_format, downsample=snapshot_downsample,
                                        interleaved=True), "time": t}
            for n, (t, vx, vy, vz) in enumerate(vel)]
    with open(name("manifest.json"), "w") as fh:
        json.dump(files, fh, indent=2)
    files["manifest"] = str(name("manifest.json"))
    return files


def load_probe_data(path) -> dict:
    """The probe JSON with each trace as a float32 array."""
    with open(Path(path)) as fh:
        doc = json.load(fh)
    for p in doc["probes"].values():
        p["data"] = np.array(p["data"], dtype=np.float32)
    return doc


def load_snapshot(path, shape, dtype: str = "float16") -> np.ndarray:
    return np.fromfile(Path(path), dtype=np.dtype(dtype)).reshape(shape)


def load_geometry(path, shape, format: str = "binary") -> np.ndarray:
    """The air mask from packed bits or run-length JSON."""
    if format == "binary":
        n = int(np.prod(shape))
        return np.unpackbits(np.fromfile(Path(path), dtype=np.uint8))[:n].reshape(shape).astype(bool)
    if format == "json":
        with open(Path(path)) as fh:
            runs = json.load(fh)["runs"]
        flat = np.repeat([r["v"] for r in runs], [r["n"] for r in runs]).astype(bool)
        return flat.reshape(shape)
    raise ValueError(f"Unknown format: {format}")
