"""Host side of the GPU voxeliser: the CSG stack programs.  An n-ary union,
intersection or difference is emitted as a left fold of two-operand steps
(the order of the reference's np.minimum.reduce / np.maximum.reduce /
Difference loop, geometry/sdf.py:549-733), so the evaluation stack grows
with the tree depth only; the kernel's stack holds 32 distances and 12
points."""
import strata_fdtd_gb300 as S
from strata_fdtd_gb300 import sdf as SD


def _depths(prog, n):
    d = p = dmax = pmax = 0
    for q in range(n):
        op, k = prog[q].op, prog[q].n
        if op in (SD.OP_BOX, SD.OP_SPHERE, SD.OP_CYLINDER):
            d += 1
        elif op in (SD.OP_UNION, SD.OP_INTERSECTION, SD.OP_DIFFERENCE):
            assert 0 <= k <= d or k == 0
            d = d - k + 1
        elif op in (SD.OP_PUSH_TRANSLATE, SD.OP_PUSH_SCALE):
            p += 1
        elif op == SD.OP_POP_POINT:
            p -= 1
        dmax, pmax = max(dmax, d), max(pmax, p)
    assert d == 1 and p == 0
    return dmax, pmax


def test_wide_union_keeps_a_shallow_stack():
    boxes = [S.Box(center=(0.01 * q, 0.0, 0.0), size=(0.005, 0.005, 0.005)) for q in range(64)]
    prog, n = S.Union(*boxes).program()
    assert n == 64 + 63
    assert _depths(prog, n)[0] == 2


def test_resonator_block_and_nested_csg_fit_the_kernel_stacks():
    res = [S.HelmholtzResonator(position=(0.01 * q, 0.01, 0.01), cavity_shape="box",
                                cavity_size=(0.004,) * 3, neck_length=0.002, neck_radius=0.001)
           for q in range(32)]
    walls = S.Difference(S.Box(center=(0.1, 0.1, 0.1), size=(0.2, 0.2, 0.2)),
                         S.Box(center=(0.1, 0.1, 0.1), size=(0.18, 0.18, 0.18)),
                         *[S.Sphere(center=(0.02 * q, 0.1, 0.1), radius=0.004) for q in range(10)])
    shape = S.Intersection(S.Union(walls, *res), S.Box(center=(0.1, 0.1, 0.1), size=(0.3,) * 3))
    prog, n = shape.program()
    dmax, pmax = _depths(prog, n)
    assert dmax <= 6 and pmax <= 2


def test_single_and_empty_operands():
    one = S.Union(S.Sphere(center=(0, 0, 0), radius=1.0))
    prog, n = one.program()
    assert [prog[q].op for q in range(n)] == [SD.OP_SPHERE, SD.OP_UNION]
    prog, n = S.Union().program()
    assert n == 1 and prog[0].op == SD.OP_UNION and prog[0].n == 0
