"""sf_plan_energy_noalloc: the energy reading for callers that cannot
allocate device memory (a process whose HBM another caching allocator holds,
or a real-time loop that must not call cudaMalloc / cudaFree).  Its scratch is
a fixed array in the library's device image, so its answers must equal the
allocating entry point's (sf_plan_energy, which takes caller scratch) -- here
on two calls in a row, each after more steps, so a stale value left in the
shared array would show.  Collected last; runs alone or after the others."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import strata_fdtd_gb300 as S  # noqa: E402
from strata_fdtd_gb300 import _native  # noqa: E402


def _energy_with_scratch(lib, s):
    need = int(lib.sf_energy_scratch_doubles(s._plan))
    scratch = torch.empty(need, dtype=torch.float64, device="cuda")
    out = ctypes.c_double()
    _native.check(lib.sf_plan_energy(s._plan, s.rho, s.c, s.dx, scratch.data_ptr(),
                                     ctypes.byref(out), torch.cuda.current_stream().cuda_stream),
                  "sf_plan_energy")
    return out.value


def _energy_no_alloc(lib, s):
    out = ctypes.c_double()
    _native.check(lib.sf_plan_energy_noalloc(s._plan, s.rho, s.c, s.dx, ctypes.byref(out),
                                             torch.cuda.current_stream().cuda_stream),
                  "sf_plan_energy_noalloc")
    return out.value


@pytest.mark.parametrize("shape,geometry", [((100, 100, 100), False), ((64, 48, 80), True)])
def test_energy_noalloc_matches_allocating_entry_point(shape, geometry):
    lib = _native.load()
    s = S.FDTDSolver(shape=shape, resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
    s.add_boundary(S.PML(depth=6))
    if geometry:
        g = np.ones(shape, dtype=bool)
        g[20:30, 10:30, 30:50] = False
        s.set_geometry(g)
    s.add_source(S.GaussianPulse(position=(shape[0] // 8, shape[1] // 2, shape[2] // 2),
                                 frequency=20000.0))  # in air, outside the solid block
    s.run_steps(60)
    s.device_fields()  # push any host edits; the state now lives on the GPU
    first = [_energy_no_alloc(lib, s), _energy_with_scratch(lib, s)]
    s.run_steps(25)
    second = [_energy_no_alloc(lib, s), _energy_with_scratch(lib, s)]
    assert first[0] > 0 and second[0] > 0 and first[0] != second[0]
    # same kernels, same block count, same summation order: equal to 1e-12
    assert first[0] == pytest.approx(first[1], rel=1e-12)
    assert second[0] == pytest.approx(second[1], rel=1e-12)
    torch.cuda.synchronize()
