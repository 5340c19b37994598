"""Result files without HDF5 (strata_fdtd_gb300.io.legacy, io/legacy.py of
the reference) against the files the reference's own exporters wrote
(tests/golden/legacy_io.npz, tests/golden/make_golden.py ``legacy``):
every array exporter option byte for byte on CPU, the loaders round trip,
and on the GPU a small solve with pressure and velocity snapshots exported
whole -- metadata, probe traces, geometry, snapshots and manifest byte for
byte the reference's (the GPU solve equals the reference's)."""
import types

import numpy as np
import pytest

import cases as C
import strata_fdtd_gb300 as S
from conftest import golden
from strata_fdtd_gb300.io import HDF5ResultWriter
from strata_fdtd_gb300.io import legacy as L

G = golden("legacy_io")


def _expect(group):
    meta = {k.split("__", 2)[2]: str(G[k]) for k in G.files if k.startswith(f"meta__{group}__")}
    files = {k.split("__", 2)[2]: G[k].tobytes() for k in G.files
             if k.startswith(f"file__{group}__")}
    return meta, files


def _compare(got, want):
    (gm, gf), (wm, wf) = got, want
    assert sorted(gf) == sorted(wf)
    for name in wf:
        assert gf[name] == wf[name], name
    assert gm == wm


@pytest.mark.filterwarnings("ignore:overflow encountered in cast")
def test_array_exports_match_reference_bytes(tmp_path):
    _compare(C.legacy_array_exports(L, str(tmp_path)), _expect("arrays"))


@pytest.mark.filterwarnings("ignore:overflow encountered in cast")
def test_loaders_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    p = rng.standard_normal((5, 6, 7)).astype(np.float32)
    L.export_snapshot(p, tmp_path / "p.bin", format="float32")
    np.testing.assert_array_equal(L.load_snapshot(tmp_path / "p.bin", (5, 6, 7), "float32"), p)
    L.export_snapshot(p, tmp_path / "h.bin")
    np.testing.assert_array_equal(L.load_snapshot(tmp_path / "h.bin", (5, 6, 7)),
                                  p.astype(np.float16))
    g = rng.random((5, 6, 7)) > 0.5
    for fmt, name in (("binary", "g.bin"), ("json", "g.json")):
        L.export_geometry(g, tmp_path / name, format=fmt)
        np.testing.assert_array_equal(L.load_geometry(tmp_path / name, g.shape, format=fmt), g)
    with pytest.raises(ValueError):
        L.export_snapshot(p, tmp_path / "x.bin", format="int8")
    with pytest.raises(ValueError):
        L.export_geometry(g, tmp_path / "x", format="png")
    with pytest.raises(NotImplementedError):
        HDF5ResultWriter("x.h5")


@pytest.mark.gpu
def test_solve_export_matches_reference_files(tmp_path):
    api = types.SimpleNamespace(FDTDSolver=S.FDTDSolver, UniformGrid=S.UniformGrid, PML=S.PML,
                                GaussianPulse=S.GaussianPulse)
    case = C.LEGACY_CASE
    solver = C.build_case(api, case)
    solver.enable_snapshots(case["snapshot_interval"], capture_velocity=True)
    solver.run_steps(case["steps"])
    got = C.legacy_solve_exports(L, solver, str(tmp_path))
    _compare(got, _expect("solve"))
    doc = L.load_probe_data(tmp_path / "run_probes.json")
    for name, trace in solver.get_probe_data().items():
        np.testing.assert_array_equal(doc["probes"][name]["data"], trace)
