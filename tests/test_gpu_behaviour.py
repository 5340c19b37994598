"""Behaviour of the GPU solver as a drop-in for the reference API: physical
properties of the scheme (CFL step, propagation speed, energy in a closed
box, PML and Mur absorption, solids, cavity modes) and the solver controls
(run durations, reset, snapshots, energy tracking and reports, frequency
response).  The reference's own tests check the same behaviours
(tests/test_fdtd.py); the set-ups and tolerances here are this project's."""
import warnings

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import strata_fdtd_gb300 as S  # noqa: E402

C_AIR, RHO = 343.0, 1.204


def _solver(shape=(40, 40, 40), res=1e-3, courant=0.5, **kw):
    return S.FDTDSolver(grid=S.UniformGrid(shape, res), c=C_AIR, rho=RHO, courant=courant, **kw)


def test_time_step_is_the_cfl_limit_times_courant():
    for res, courant in ((1e-3, 0.5), (2e-3, 0.9), (5e-4, 0.3)):
        s = _solver((10, 10, 10), res, courant)
        assert s.dt == pytest.approx(courant * res / (C_AIR * np.sqrt(3)), rel=1e-15)
        assert s.dt * C_AIR * np.sqrt(3) / res <= 1.0


def test_pulse_travels_at_the_speed_of_sound():
    """A one-way plane pulse (pressure and matching x-velocity, so nothing
    travels back to the wall behind it) along a narrow rigid duct: the
    delay between probes 120 cells apart (cross-correlation peak) matches
    c within 1.5 %, at two Courant numbers."""
    for courant in (0.5, 0.9):
        s = _solver((240, 8, 8), courant=courant)
        x = np.arange(240, dtype=np.float64)

        def g(u):
            return np.exp(-((u - 40.0) ** 2) / (2 * 4.0**2))

        p = g(x).astype(np.float32)
        vx = (g(x + 0.5 + 0.5 * C_AIR * s.dt / 1e-3) / (RHO * C_AIR)).astype(np.float32)
        vx[-1] = 0.0
        s.p[...] = p[:, None, None]
        s.vx[...] = vx[:, None, None]
        s.add_probe("a", (70, 4, 4))
        s.add_probe("b", (190, 4, 4))
        s.run_steps(int(np.ceil(4.8e-4 / s.dt)))
        a, b = (s.get_probe_data()[k].astype(np.float64) for k in ("a", "b"))
        lag = np.argmax(np.correlate(b, a, mode="full")) - (len(a) - 1)
        assert 120e-3 / (lag * s.dt) == pytest.approx(C_AIR, rel=0.015)
        assert a.min() > -1e-3 * a.max()  # no backward-travelling half


def test_energy_stays_bounded_in_a_closed_box():
    """Rigid walls all round, no absorber, a smooth Gaussian blob of
    pressure: the discrete energy (pressure and velocity half a step apart)
    stays within a few percent of its start for 600 steps."""
    s = _solver((30, 30, 30))
    i, j, k = np.meshgrid(*(np.arange(30),) * 3, indexing="ij")
    s.p[...] = np.exp(-((i - 15) ** 2 + (j - 15) ** 2 + (k - 15) ** 2) / (2 * 3.0**2))
    s.run_steps(600, track_energy=True, energy_sample_interval=20)
    e = np.array([v for _, _, v in s.get_energy_history()])
    assert len(e) == 31 and np.all(np.isfinite(e)) and e.min() > 0
    assert e.max() / e.min() < 1.1
    assert e[-1] / e[0] == pytest.approx(1.0, abs=0.03)


def test_pml_drains_the_energy():
    s = _solver((40, 40, 40))
    s.add_boundary(S.PML(depth=8))
    s.p[20, 20, 20] = 1.0
    s.run_steps(600, track_energy=True, energy_sample_interval=50)
    rep = s.energy_report()
    assert rep["conservation_status"] == "decaying"
    assert rep["final_energy"] < 0.05 * rep["max_energy"]


def test_pml_and_mur_reduce_the_echo_from_the_far_wall():
    def echo(boundary):
        s = _solver((100, 24, 24))
        if boundary is not None:
            s.add_boundary(boundary)
        s.add_source(S.GaussianPulse(position=(30, 12, 12), frequency=15000.0))
        s.add_probe("p", (30, 12, 12))
        s.run_steps(700)
        tr = s.get_probe_data()["p"]
        return np.abs(tr[350:]).max()  # after the direct pulse, while echoes return
    rigid = echo(None)
    assert echo(S.PML(depth=10)) < 0.5 * rigid
    assert echo(S.ABCFirstOrder()) < rigid


def test_solids_block_propagation_and_hold_zero_pressure():
    s = _solver((60, 30, 30))
    geom = np.ones(s.shape, dtype=bool)
    geom[30:34, :, :] = False  # a full wall across x
    s.set_geometry(geom)
    s.add_source(S.GaussianPulse(position=(15, 15, 15), frequency=10000.0))
    s.add_probe("behind", (45, 15, 15))
    s.run_steps(300)
    assert np.abs(s.get_probe_data()["behind"]).max() == 0.0
    assert np.all(s.p[30:34] == 0.0)
    assert np.all(s.vx[29:34] == 0.0)  # faces into and inside the wall


def test_cavity_fundamental_mode():
    """A rigid 60 x 20 x 20 mm box rings at c / (2 L) along its long axis."""
    s = _solver((60, 20, 20), courant=0.5)
    s.add_source(S.GaussianPulse(position=(3, 10, 10), frequency=6000.0))
    s.add_probe("end", (57, 10, 10))
    s.run_steps(16000)
    f, mag = s.get_frequency_response("end")
    band = (f > 1500) & (f < 4500)
    peak = f[band][np.argmax(mag[band])]
    assert peak == pytest.approx(C_AIR / (2 * 0.060), rel=0.05)


def test_run_duration_sets_the_step_count_and_time():
    s = _solver((16, 16, 16))
    s.run(duration=50.5 * s.dt)
    assert s.step_count == 51
    assert s.time == pytest.approx(51 * s.dt, rel=1e-12)
    assert s.get_sample_rate() == pytest.approx(1.0 / s.dt)


def test_reset_clears_fields_traces_and_history():
    s = _solver((16, 16, 16))
    s.add_source(S.GaussianPulse(position=(8, 8, 8), frequency=20000.0))
    s.add_probe("c", (8, 8, 8))
    s.run_steps(40, track_energy=True)
    assert np.abs(s.p).max() > 0
    s.reset()
    assert s.step_count == 0 and s.time == 0.0
    assert np.all(s.p == 0) and np.all(s.vx == 0)
    assert len(s.get_probe_data()["c"]) == 0
    assert s.get_energy_history() == []
    s.run_steps(40)
    a = s.get_probe_data()["c"].copy()
    s.reset()
    s.run_steps(40)
    np.testing.assert_array_equal(s.get_probe_data()["c"], a)  # deterministic


def test_snapshots_at_the_interval_with_centred_velocity():
    s = _solver((16, 16, 16))
    s.add_source(S.GaussianPulse(position=(8, 8, 8), frequency=20000.0))
    s.enable_snapshots(interval=10, capture_velocity=True)
    s.run_steps(35)
    snaps = s.get_snapshots()
    assert len(snaps) == 4  # steps 0, 10, 20, 30
    t, p = snaps[-1]
    assert p.shape == s.shape and t == pytest.approx(30 * s.dt, rel=1e-12)
    vs = s.get_velocity_snapshots()
    assert len(vs) == 4 and vs[-1][1].shape == s.shape


def test_energy_report_and_drift_warning():
    s = _solver((20, 20, 20), warn_energy_drift=True, energy_drift_threshold=0.01)
    s.add_source(S.GaussianPulse(position=(10, 10, 10), frequency=20000.0))
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        s.run_steps(60, track_energy=True)
    assert any("Energy drift" in str(x.message) for x in w)  # the source adds energy
    rep = s.energy_report()
    assert rep["n_samples"] == 61 and rep["conservation_status"] == "growing"
    with pytest.raises(ValueError):
        _solver((8, 8, 8)).energy_report()


def test_frequency_response_bins():
    s = _solver((16, 16, 16))
    s.add_source(S.GaussianPulse(position=(8, 8, 8), frequency=20000.0))
    s.add_probe("c", (8, 8, 8))
    s.run_steps(100)
    f, mag = s.get_frequency_response("c")
    assert len(f) == len(mag) == 128 // 2 + 1
    assert f[-1] == pytest.approx(0.5 / s.dt)


def test_duplicate_names_and_bad_positions_are_rejected():
    s = _solver((16, 16, 16))
    s.add_probe("a", (1, 1, 1))
    with pytest.raises(ValueError):
        s.add_probe("a", (2, 2, 2))
    with pytest.raises(ValueError):
        s.add_source(S.GaussianPulse(position=(16, 0, 0), frequency=1000.0))
    with pytest.raises(ValueError):
        s.set_geometry(np.ones((15, 16, 16), dtype=bool))


def test_snapshots_equal_the_oracle_state_and_numpy_centring():
    """Snapshot contents (staged on the device, copied to host beside the
    following steps) are the oracle's p after the due steps, and the
    centred velocities equal the reference's NumPy float32 averaging of the
    oracle's staggered fields."""
    import cases as C
    from oracle import oracle as O
    from test_gpu_parity import API

    case = dict(shape=(18, 21, 24), res=1e-3, courant=0.6, pml=dict(depth=3),
                geometry=dict(kind="blocks", seed=5, n_boxes=2, n_spheres=1),
                sources=[("point", (9, 10, 11), 25000.0, 1.0)], probes=[("a", (4, 5, 6))],
                steps=30)
    ref = C.build_case(O.make_api(), case)
    s = C.build_case(API, case)
    s.enable_snapshots(interval=7, capture_velocity=True)
    s.run_steps(12)
    s.step()
    s.run_steps(17)
    want = []
    for q in range(30):
        ref.step()
        if q % 7 == 0:
            vx, vy, vz = ref.vx, ref.vy, ref.vz
            cx = np.zeros(vx.shape, np.float32)
            cx[1:] = 0.5 * (vx[:-1] + vx[1:])
            cx[0] = 0.5 * vx[0]
            cy = np.zeros(vy.shape, np.float32)
            cy[:, 1:] = 0.5 * (vy[:, :-1] + vy[:, 1:])
            cy[:, 0] = 0.5 * vy[:, 0]
            cz = np.zeros(vz.shape, np.float32)
            cz[:, :, 1:] = 0.5 * (vz[:, :, :-1] + vz[:, :, 1:])
            cz[:, :, 0] = 0.5 * vz[:, :, 0]
            want.append((q, ref.p.copy(), cx, cy, cz))
    snaps, vsnaps = s.get_snapshots(), s.get_velocity_snapshots()
    assert [round(t / s.dt) for t, _ in snaps] == [w[0] for w in want]
    for (t, p), (tv, *cv), (q, wp, *wc) in zip(snaps, vsnaps, want):
        assert t == tv
        np.testing.assert_array_equal(p, wp, err_msg=f"p after step {q}")
        for got, exp, name in zip(cv, wc, "xyz"):
            np.testing.assert_array_equal(got, exp, err_msg=f"centred v{name} after step {q}")


def test_waveform_table_matches_per_step_calls_on_this_host():
    """The same check with the NumPy of the machine that runs the GPU."""
    from test_abi_host import waveform_table_matches_per_step_calls
    waveform_table_matches_per_step_calls(20000)


def test_async_field_load_and_readback_on_a_copy_stream():
    """load_fields_async / fields_async / probe_data_async on a copy stream
    around steps on the compute stream (the pattern of the end-to-end bench:
    two replicas alternating) give the same bits as assigning the fields,
    stepping and reading p, vz and the traces synchronously."""
    shape = (40, 36, 44)
    rng = np.random.default_rng(11)
    host = {f: torch.from_numpy(rng.standard_normal(shape).astype(np.float32) * 1e-3)
            .pin_memory().numpy() for f in ("p", "vx", "vy", "vz")}
    geom = np.ones(shape, dtype=bool)
    geom[18:22, 10:30, 6:40] = False
    for f in host:
        host[f][~geom] = 0.0

    def make():
        s = _solver(shape)
        s.add_boundary(S.PML(depth=6))
        s.set_geometry(geom)
        s.add_source(S.GaussianPulse(position=(10, 18, 22), frequency=8000.0))
        s.add_probe("a", (30, 18, 22))
        s.add_probe("b", (12, 30, 8))
        return s

    ref = make()
    for f in host:
        setattr(ref, f, host[f].copy())  # an assigned array becomes the solver's field
    ref.run_steps(64)
    want = {"p": ref.p.copy(), "vz": ref.vz.copy()}
    want_tr = ref.get_probe_data()

    reps = (make(), make())
    comp, cp = torch.cuda.current_stream(), torch.cuda.Stream()
    outs = [{f: torch.empty(shape, dtype=torch.float32).pin_memory().numpy() for f in ("p", "vz")}
            for _ in reps]
    got = []
    for k, a in enumerate(reps):
        with torch.cuda.stream(cp):
            a.load_fields_async(**host)
            up = torch.cuda.Event()
            up.record(cp)
        comp.wait_event(up)
        a.run_steps(64)
        ran = torch.cuda.Event()
        ran.record(comp)
        with torch.cuda.stream(cp):
            cp.wait_event(ran)
            got.append((a.fields_async(("p", "vz"), out=outs[k]), a.probe_data_async()))
    for fp, ft in got:
        fields, traces = fp(), ft()
        for f in ("p", "vz"):
            np.testing.assert_array_equal(fields[f], want[f])
        for n in want_tr:
            np.testing.assert_array_equal(traces[n], want_tr[n])
    assert np.abs(want_tr["a"]).max() > 0
    with pytest.raises(ValueError):
        reps[0].load_fields_async(p=np.zeros((3, 3, 3), dtype=np.float32))
    with pytest.raises(ValueError):
        reps[0].load_fields_async(q=host["p"])


def test_closed_pipe_keeps_its_energy_one_step_at_a_time():
    """A closed rigid pipe (110 x 25 x 25 cells of 2 mm, air in the
    100 x 15 x 15 interior, five cells of solid around it) started from a
    single-cell pressure value, stepped one step() at a time with the energy
    read after each: after 2000 steps at least a tenth of the energy at step
    10 is left.  Rigid faces are applied between the velocity and the
    pressure updates; applying them after the pressure update drains the
    pipe by orders of magnitude (the reference's own regression check for
    that ordering, tests/test_fdtd.py:167-219)."""
    s = S.FDTDSolver(shape=(110, 25, 25), resolution=2e-3, c=C_AIR)
    g = np.zeros(s.shape, dtype=bool)
    g[5:105, 5:20, 5:20] = True
    s.set_geometry(g)
    s.p[55, 12, 12] = 1e-5
    e10 = None
    for n in range(2000):
        s.step()
        e = s.compute_energy()
        if n == 10:
            e10 = e
    assert e10 > 0
    assert e / e10 > 0.1, e / e10


def test_point_and_plane_sources_inject_where_they_are_placed():
    """A point source changes its own cell in the first step; a plane source
    (axis 0, index 5) changes every cell of its plane and leaves a plane
    five cells away at zero (tests/test_fdtd.py:484-515 check the same)."""
    s = _solver((20, 20, 20))
    s.add_source(S.GaussianPulse(position=(10, 10, 10), frequency=1000))
    assert s.p[10, 10, 10] == 0.0
    s.step()
    assert s.p[10, 10, 10] != 0.0

    s = S.FDTDSolver(shape=(30, 20, 20), resolution=3e-3)
    s.add_source(S.GaussianPulse(position={"axis": 0, "index": 5}, frequency=1000,
                                 source_type="plane"))
    s.step()
    assert np.all(s.p[5] != 0.0)
    assert np.allclose(s.p[10], 0.0, atol=1e-10)


def test_geometry_optimizer_voxelises_on_the_gpu():
    """GeometryOptimizer (geometry/parametric.py): Nelder-Mead over a
    parametric horn, each evaluation voxelised on the GPU, lowers the
    objective (the distance of the horn's cell count from a target) and
    respects its constraints."""
    from strata_fdtd_gb300 import geometry as G

    grid = S.UniformGrid((40, 40, 60), 5e-3)
    horn = G.ParametricHorn(throat_radius=0.02, mouth_radius=0.05, length=0.15,
                            axis_start=(0.1, 0.1, 0.03))
    cs = G.ConstraintSet()
    cs.add_ratio_constraint("throat_radius", "mouth_radius", 1.5)
    opt = G.GeometryOptimizer(horn, grid, constraints=cs)
    target = 3000

    def objective(mask):
        return abs(int(mask.sum()) - target)

    start = objective(horn.voxelize(grid))
    res = opt.optimize(objective, options=dict(maxfev=60))
    assert res["nfev"] > 0 and res["objective"] <= start
    assert cs.is_feasible(res["parameters"])
    assert res["geometry"].voxelize(grid).sum() > 0
