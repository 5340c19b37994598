"""The reverse-time adjoint (sf_diff_*): gradients of the probe-trace loss
w.r.t. the density field, checked against torch.autograd through a plain
PyTorch stepping of the same scheme and against central finite differences.

Tolerances: FP64 and double-word ("dw", the default) adjoints vs FP64
autograd, rel 1e-9 and 1e-8 (same arithmetic up to summation order; dw
carries about 48 bits); FP64 adjoint vs central differences (h = 1e-3), rel
1e-5 (O(h^2) truncation); at the 128^3 x 2000-step workload, per sampled
cell against FP64 central differences: the default dw adjoint rel 1e-4
(the stated target), the FP64 adjoint rel 1e-5, the FP32 adjoint rel 2e-3
(its documented accuracy); probe traces from the in-kernel and the separate
gather bit-equal in every precision, and at small size with 6 probes the
FP32 adjoint vs the FP64 adjoint within 1e-4 of the largest gradient
entry."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from strata_fdtd_gb300.adjoint import DifferentiableSolver, reference_loss_torch  # noqa: E402
from strata_fdtd_gb300.workloads import design_field  # noqa: E402


def _small(dtype, K=25):
    return DifferentiableSolver((16, 14, 18), pml_depth=3, frequency=20000.0, source=(5, 7, 9),
                                probes=[(12, 7, 9), (8, 3, 14)], dtype=dtype,
                                checkpoint_every=K)


@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-9), ("dw", 1e-8)])
def test_adjoint_matches_autograd_fp64(dtype, rtol):
    s = _small(dtype)
    theta = torch.tensor(design_field(s.shape, region=8, seed=1, sigma=1.5), device="cuda")
    target = s.forward(torch.tensor(design_field(s.shape, region=8, seed=2, sigma=1.5),
                                    device="cuda"), 60)[0]
    th = theta.clone().requires_grad_(True)
    loss = s.loss(th, target, 60)
    loss.backward()
    ref_th = theta.clone().requires_grad_(True)
    ref = reference_loss_torch(_small(torch.float64), ref_th, target, 60)
    ref.backward()
    assert float(loss) == pytest.approx(float(ref), rel=rtol * 1e-3)
    g, r = th.grad.cpu().numpy(), ref_th.grad.cpu().numpy()
    assert np.abs(r).max() > 0
    np.testing.assert_allclose(g, r, rtol=rtol, atol=rtol * 1e-3 * np.abs(r).max())


def test_adjoint_matches_central_differences_fp64():
    s = _small(torch.float64, K=16)
    theta = torch.tensor(design_field(s.shape, region=8, seed=3, sigma=1.5), device="cuda")
    target = s.forward(torch.zeros_like(theta), 50)[0] * 0.5
    th = theta.clone().requires_grad_(True)
    s.loss(th, target, 50).backward()
    rng = np.random.default_rng(0)
    h = 1e-3
    for _ in range(6):
        c = tuple(int(rng.integers(4, n - 4)) for n in s.shape)
        tp, tm = theta.clone(), theta.clone()
        tp[c] += h
        tm[c] -= h
        fd = (float(s.loss(tp, target, 50)) - float(s.loss(tm, target, 50))) / (2 * h)
        assert float(th.grad[c]) == pytest.approx(fd, rel=1e-5, abs=1e-14)


def test_differentiable_workload_against_fd():
    """The 128^3 workload: 10-cell PML, design field on the central 64^3,
    1.5 kHz source, 2000 steps, checkpoints every 100 steps.  Against FP64
    central differences (h = 1e-3) on 16 random cells of the design region,
    per cell: the default double-word adjoint rel 1e-4 (the target), the
    FP64 adjoint rel 1e-5 (O(h^2) truncation), the FP32 adjoint rel 2e-3
    (FP32 rounding of 2000 forward and 2000 adjoint steps); the double-word
    gradient also equals the FP64 one to 1e-6 in L2 over the region."""
    shape = (128, 128, 128)
    probes = [(100, 64, 64), (64, 100, 40)]

    def make(dtype):
        return DifferentiableSolver(shape, pml_depth=10, frequency=1500.0, source=(30, 64, 64),
                                    probes=probes, dtype=dtype, checkpoint_every=100)

    s64 = make(torch.float64)
    theta = torch.tensor(design_field(shape, 64, seed=0), device="cuda")
    target = s64.forward(torch.tensor(design_field(shape, 64, seed=1), device="cuda"), 2000)[0]
    grads = {}
    for name, dtype in (("dw", "dw"), ("f64", torch.float64), ("f32", torch.float32)):
        s = s64 if dtype == torch.float64 else make(dtype)
        th = theta.clone().to(s.ext_dtype).requires_grad_(True)
        s.loss(th, target.to(s.ext_dtype), 2000).backward()
        grads[name] = th.grad.double()
        del s, th
    rng = np.random.default_rng(5)
    h = 1e-3
    worst = {k: 0.0 for k in grads}
    for _ in range(16):
        c = tuple(int(v) for v in rng.integers(32, 96, size=3))
        tp, tm = theta.clone(), theta.clone()
        tp[c] += h
        tm[c] -= h
        fd = (float(s64.loss(tp, target, 2000)) - float(s64.loss(tm, target, 2000))) / (2 * h)
        for k, g in grads.items():
            worst[k] = max(worst[k], abs(float(g[c]) - fd) / abs(fd))
    region = (slice(32, 96),) * 3
    l2 = float(torch.linalg.norm(grads["dw"][region] - grads["f64"][region])
               / torch.linalg.norm(grads["f64"][region]))
    print("adjoint vs FD, worst rel per sampled cell: "
          + ", ".join(f"{k} {v:.3e}" for k, v in worst.items()) + f"; dw vs f64 L2 {l2:.3e}")
    assert worst["dw"] < 1e-4, worst
    assert worst["f64"] < 1e-5, worst
    assert worst["f32"] < 2e-3, worst
    assert l2 < 1e-6, l2


def test_probe_gather_paths_and_many_probe_gradients():
    """Up to 4 probes are sampled inside the forward kernel, more by a
    separate gather after each step: the traces of the probes both solvers
    share must be identical bit for bit, in every precision.  With 6 probes
    (the separate gather) the FP64 adjoint must match autograd through the
    plain PyTorch stepping (rel 1e-9); the FP32 adjoint, whose face sums are
    double-word float pairs, the FP64 adjoint to 1e-4 of the largest
    gradient entry (FP32 rounding of 60 forward and 60 adjoint steps), and
    the double-word adjoint to 1e-9."""
    pos = [(12, 7, 9), (8, 3, 14), (10, 10, 4), (4, 5, 6), (13, 11, 15), (6, 12, 3)]

    def make(dtype, probes):
        return DifferentiableSolver((16, 14, 18), pml_depth=3, frequency=20000.0,
                                    source=(5, 7, 9), probes=probes, dtype=dtype,
                                    checkpoint_every=25)

    theta = torch.tensor(design_field((16, 14, 18), region=8, seed=4, sigma=1.5), device="cuda")
    target64 = make(torch.float64, pos).forward(
        torch.tensor(design_field((16, 14, 18), region=8, seed=5, sigma=1.5), device="cuda"),
        60)[0]
    grads = {}
    for dtype in (torch.float32, torch.float64, "dw"):
        few, many = make(dtype, pos[:3]), make(dtype, pos)
        trace_few = few.forward(theta, 60)[0]
        trace_many = many.forward(theta, 60)[0]
        assert trace_many.shape == (60, 6)
        assert torch.equal(trace_few, trace_many[:, :3])
        assert float(trace_many.abs().max()) > 0
        target = target64.to(many.ext_dtype)
        th = theta.clone().to(many.ext_dtype).requires_grad_(True)
        loss = many.loss(th, target, 60)
        loss.backward()
        grads[dtype] = th.grad.double()
        if dtype == torch.float64:
            ref_th = theta.clone().requires_grad_(True)
            ref = reference_loss_torch(many, ref_th, target, 60)
            ref.backward()
            assert float(loss) == pytest.approx(float(ref), rel=1e-12)
            r = ref_th.grad.cpu().numpy()
            np.testing.assert_allclose(th.grad.cpu().numpy(), r, rtol=1e-9,
                                       atol=1e-12 * np.abs(r).max())
    g32, g64, gdw = grads[torch.float32], grads[torch.float64], grads["dw"]
    scale = float(g64.abs().max())
    assert scale > 0
    err = float((g32 - g64).abs().max()) / scale
    err_dw = float((gdw - g64).abs().max()) / scale
    print(f"6 probes, max abs err / max |g| against the fp64 adjoint: fp32 {err:.3e}, "
          f"dw {err_dw:.3e}")
    assert err < 1e-4, err
    assert err_dw < 1e-9, err_dw


def test_unit_decay_blocks_change_no_value():
    """Blocks whose cells and neighbours all have decay 1 skip the decay
    products in the forward and adjoint kernels: traces and gradients must
    equal, bit for bit, those of the same solve with that path switched off
    (empty unit-decay ranges), in every precision."""
    shape = (24, 28, 72)  # interior blocks of 32 k x 8 j exist at PML 3
    theta = torch.tensor(design_field(shape, region=12, seed=7, sigma=2.0), device="cuda")
    for dtype in (torch.float32, torch.float64, "dw"):
        out = []
        for unit in (True, False):
            s = DifferentiableSolver(shape, pml_depth=3, frequency=20000.0, source=(8, 14, 30),
                                     probes=[(16, 14, 50), (10, 20, 20)], dtype=dtype,
                                     checkpoint_every=20)
            if unit:
                assert s._unit[2][1] - s._unit[2][0] >= 40 and s._unit[1][1] - s._unit[1][0] >= 16
            else:
                s._unit = [(0, 0)] * 3
            th = theta.clone().to(s.ext_dtype).requires_grad_(True)
            target = torch.zeros((60, 2), dtype=s.ext_dtype, device="cuda")
            loss = s.loss(th, target, 60)
            loss.backward()
            out.append((s.forward(theta.to(s.ext_dtype), 60)[0], th.grad.clone(), loss.detach()))
        (t1, g1, l1), (t0, g0, l0) = out
        assert float(t1.abs().max()) > 0 and float(g1.abs().max()) > 0
        assert torch.equal(t1, t0) and torch.equal(g1, g0) and torch.equal(l1, l0), dtype


def _walled_geometry(shape=(20, 18, 22)):
    """A rigid slab across x = 10-11 with a 4x4 aperture, and a solid block
    beside the source: faces on every axis touch a solid cell."""
    g = np.ones(shape, dtype=bool)
    g[10:12] = False
    g[10:12, 7:11, 9:13] = True
    g[4:7, 12:15, 5:9] = False
    return g


def _walled(dtype, geometry, K=25, source=(5, 9, 11)):
    return DifferentiableSolver(geometry.shape, pml_depth=3, frequency=20000.0, source=source,
                                probes=[(15, 9, 11), (14, 4, 16)], dtype=dtype,
                                checkpoint_every=K, geometry=geometry)


@pytest.mark.parametrize("walls", [False, True])
def test_forward_matches_oracle_fp64(walls):
    """The differentiable forward at theta = 0 is the reference scheme with a
    scalar density: its FP64 probe traces against the oracle's FP64 build of
    the same solve (the oracle's samples as doubles, before get_probe_data
    rounds them to float32 as the reference stores them) (same PML, pulse, probes and, with
    walls, the same air mask through the reference's rigid pass and p = 0 in
    solids), rel-L2 1e-12 (the face coefficient is formed as
    (dt/dx)(1/rho + 1/rho)/2 instead of dt/(rho dx): rounding-level
    differences in FP64)."""
    from oracle import oracle as O

    g = _walled_geometry()
    s = DifferentiableSolver(g.shape, pml_depth=3, frequency=20000.0, source=(5, 9, 11),
                             probes=[(15, 9, 11), (14, 4, 16)], dtype=torch.float64,
                             checkpoint_every=25, geometry=g if walls else None)
    n = 150
    trace = s.forward(torch.zeros(g.shape, dtype=torch.float64, device="cuda"), n,
                      keep_checkpoints=False)[0].cpu().numpy()
    o = O.FDTDSolver(shape=g.shape, resolution=1e-3, c=343.0, rho=1.204, courant=0.5,
                     precision="f64")
    o.add_boundary(O.PML(depth=3))
    if walls:
        o.set_geometry(g)
    o.add_source(O.GaussianPulse(position=(5, 9, 11), frequency=20000.0))
    o.add_probe("a", (15, 9, 11))
    o.add_probe("b", (14, 4, 16))
    o.run_steps(n)
    for q, name in enumerate("ab"):
        r = np.asarray(o._probes[name].data, dtype=np.float64)
        assert np.abs(r).max() > 0
        err = np.linalg.norm(trace[:, q] - r) / np.linalg.norm(r)
        assert err < 1e-12, (name, err)


@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-9), ("dw", 1e-8)])
def test_walled_adjoint_matches_autograd(dtype, rtol):
    """With rigid walls the adjoint matches autograd through the plain
    PyTorch stepping (wall faces' coefficients held at zero), and the
    gradient is zero in every solid cell."""
    g = _walled_geometry()
    s = _walled(dtype, g)
    theta = torch.tensor(design_field(g.shape, region=10, seed=6, sigma=1.5), device="cuda")
    target = s.forward(torch.tensor(design_field(g.shape, region=10, seed=7, sigma=1.5),
                                    device="cuda"), 80)[0]
    th = theta.clone().requires_grad_(True)
    loss = s.loss(th, target, 80)
    loss.backward()
    ref_th = theta.clone().requires_grad_(True)
    ref = reference_loss_torch(_walled(torch.float64, g), ref_th, target, 80)
    ref.backward()
    assert float(loss) == pytest.approx(float(ref), rel=rtol * 1e-3)
    gr, r = th.grad.cpu().numpy(), ref_th.grad.cpu().numpy()
    assert np.abs(r).max() > 0
    np.testing.assert_allclose(gr, r, rtol=rtol, atol=rtol * 1e-3 * np.abs(r).max())
    assert not np.any(gr[~g]), "gradient in a solid cell"
    # cells next to a wall carry gradient through their open faces
    assert np.abs(gr[9, 7:11, 9:13]).max() > 0


def test_walled_adjoint_matches_central_differences():
    """FP64 and double-word adjoints with walls against FP64 central
    differences (h = 1e-3) on cells beside the walls, rel 1e-5."""
    g = _walled_geometry()
    cells = [(9, 8, 10), (12, 9, 11), (7, 13, 7), (4, 11, 6), (9, 3, 4), (13, 10, 12)]
    theta = torch.tensor(design_field(g.shape, region=10, seed=8, sigma=1.5), device="cuda")
    base = _walled(torch.float64, g, K=16)
    target = base.forward(torch.zeros_like(theta), 70)[0] * 0.5
    h = 1e-3
    fd = {}
    for c in cells:
        assert g[c]
        tp, tm = theta.clone(), theta.clone()
        tp[c] += h
        tm[c] -= h
        fd[c] = (float(base.loss(tp, target, 70)) - float(base.loss(tm, target, 70))) / (2 * h)
    for dtype in (torch.float64, "dw"):
        s = _walled(dtype, g, K=16)
        th = theta.clone().requires_grad_(True)
        s.loss(th, target, 70).backward()
        for c in cells:
            assert float(th.grad[c]) == pytest.approx(fd[c], rel=1e-5, abs=1e-14), (dtype, c)


def test_source_in_a_solid_cell_injects_nothing():
    g = _walled_geometry()
    s = _walled(torch.float64, g, source=(10, 2, 2))
    tr = s.forward(torch.zeros(g.shape, dtype=torch.float64, device="cuda"), 40)[0]
    assert float(tr.abs().max()) == 0.0


def _occupancy(shape, seed):
    """A smooth partial-solid field (0-0.6) on the central region plus the
    walled slab of _walled_geometry as fully solid cells."""
    phi = 0.6 * design_field(shape, region=10, seed=seed, sigma=1.5)
    phi[~_walled_geometry(shape)] = 1.0
    return phi


def test_full_occupancy_is_a_rigid_wall():
    """phi = 1 on the solid cells of the air mask, 0 elsewhere, gives the
    walled solve's traces bit for bit (every face it closes has a zero
    coefficient, the others keep theirs)."""
    g = _walled_geometry()
    phi = torch.tensor((~g).astype(np.float64), device="cuda")
    theta = torch.tensor(design_field(g.shape, region=10, seed=9, sigma=1.5), device="cuda")
    for dtype in (torch.float64, "dw", torch.float32):
        walled = _walled(dtype, g).forward(theta, 60, keep_checkpoints=False)[0]
        free = DifferentiableSolver(g.shape, pml_depth=3, frequency=20000.0, source=(5, 9, 11),
                                    probes=[(15, 9, 11), (14, 4, 16)], dtype=dtype,
                                    checkpoint_every=25)
        occ = free.forward(theta, 60, keep_checkpoints=False, occupancy=phi)[0]
        assert float(walled.abs().max()) > 0
        assert torch.equal(walled, occ), dtype


@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-9), ("dw", 1e-8)])
def test_occupancy_and_density_gradients_match_autograd(dtype, rtol):
    """Gradients with respect to both the density field theta and the
    occupancy field phi against autograd through the plain PyTorch stepping
    of the same scheme."""
    shape = (20, 18, 22)
    s = DifferentiableSolver(shape, pml_depth=3, frequency=20000.0, source=(5, 9, 11),
                             probes=[(15, 9, 11), (14, 4, 16)], dtype=dtype, checkpoint_every=25)
    theta = torch.tensor(design_field(shape, region=10, seed=12, sigma=1.5), device="cuda")
    phi = torch.tensor(_occupancy(shape, 13), device="cuda")
    target = s.forward(theta, 80, occupancy=torch.tensor(_occupancy(shape, 14), device="cuda"))[0]
    th = theta.clone().requires_grad_(True)
    ph = phi.clone().requires_grad_(True)
    loss = s.loss(th, target, 80, occupancy=ph)
    loss.backward()
    ref_s = DifferentiableSolver(shape, pml_depth=3, frequency=20000.0, source=(5, 9, 11),
                                 probes=[(15, 9, 11), (14, 4, 16)], dtype=torch.float64,
                                 checkpoint_every=25)
    rth = theta.clone().requires_grad_(True)
    rph = phi.clone().requires_grad_(True)
    ref = reference_loss_torch(ref_s, rth, target, 80, occupancy=rph)
    ref.backward()
    assert float(loss) == pytest.approx(float(ref), rel=rtol * 1e-3)
    for got, want in ((th.grad, rth.grad), (ph.grad, rph.grad)):
        w = want.cpu().numpy()
        assert np.abs(w).max() > 0
        np.testing.assert_allclose(got.cpu().numpy(), w, rtol=rtol, atol=rtol * 1e-3 * np.abs(w).max())


def test_occupancy_gradient_matches_central_differences():
    """dL/dphi of the FP64 and double-word adjoints against FP64 central
    differences (h = 1e-3) in partly open cells, rel 1e-5."""
    shape = (20, 18, 22)

    def make(dtype):
        return DifferentiableSolver(shape, pml_depth=3, frequency=20000.0, source=(5, 9, 11),
                                    probes=[(15, 9, 11), (14, 4, 16)], dtype=dtype,
                                    checkpoint_every=16)

    theta = torch.tensor(design_field(shape, region=10, seed=15, sigma=1.5), device="cuda")
    phi = torch.tensor(_occupancy(shape, 16), device="cuda")
    base = make(torch.float64)
    target = base.forward(theta, 70, occupancy=torch.zeros_like(phi))[0] * 0.5
    cells = [(9, 8, 10), (12, 9, 11), (8, 12, 8), (13, 10, 12), (7, 6, 14)]
    h = 1e-3
    fd = {}
    for c in cells:
        assert 0.0 < float(phi[c]) < 1.0
        pp, pm = phi.clone(), phi.clone()
        pp[c] += h
        pm[c] -= h
        fd[c] = (float(base.loss(theta, target, 70, occupancy=pp))
                 - float(base.loss(theta, target, 70, occupancy=pm))) / (2 * h)
    for dtype in (torch.float64, "dw"):
        s = make(dtype)
        ph = phi.clone().requires_grad_(True)
        s.loss(theta, target, 70, occupancy=ph).backward()
        for c in cells:
            assert float(ph.grad[c]) == pytest.approx(fd[c], rel=1e-5, abs=1e-14), (dtype, c)
