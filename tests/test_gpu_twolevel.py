"""The two-level preconditioner of the flexible mixed solve
(sipg_apply_twolevel_f32) against its CPU restatement (tests/twolevel_ref.py,
FP64), and the properties the inner CG relies on: symmetry and positivity,
and an iteration count that does not grow with the mesh.

Tolerance: M r in FP32 within 2e-4 of the FP64 restatement, relative to
max |M r| (FP32 rounding through the V-cycle and the element blocks)."""
import numpy as np
import pytest

import twolevel_ref

pytestmark = pytest.mark.gpu

RTOL = 2e-4


@pytest.fixture(scope="module")
def torch():
    import torch as t

    return t


@pytest.mark.parametrize("p,dim", [(1, 1), (2, 2), (3, 5), (4, 8), (4, 9), (6, 12), (8, 17), (2, 33), (5, 20), (3, 65), (2, 70)])
def test_twolevel_matches_cpu_restatement(sipg, oracle, torch, p, dim):
    pen = float(p * p)
    op = sipg.Operator(dim, p, pen)
    r = np.random.default_rng(10 * p + dim).uniform(-1.0, 1.0, op.ndof).astype(np.float32)
    z = op.apply_twolevel(torch.from_numpy(r).cuda()).cpu().numpy().astype(np.float64)
    ref = twolevel_ref.TwoLevel(oracle, p, dim, pen).apply(r.astype(np.float64))
    err = np.max(np.abs(z - ref)) / np.max(np.abs(ref))
    assert err <= RTOL, (p, dim, err)
    op.close()


@pytest.mark.parametrize("p,dim", [(2, 40), (4, 64), (6, 48), (8, 30)])
def test_twolevel_is_symmetric_and_positive(sipg, torch, p, dim):
    op = sipg.Operator(dim, p, float(p * p))
    g = torch.Generator(device="cuda").manual_seed(p + dim)
    x = torch.rand(op.ndof, device="cuda", generator=g, dtype=torch.float64) * 2 - 1
    y = torch.rand(op.ndof, device="cuda", generator=g, dtype=torch.float64) * 2 - 1
    mx = op.apply_twolevel(x.float()).double()
    my = op.apply_twolevel(y.float()).double()
    a, b = torch.dot(y, mx).item(), torch.dot(x, my).item()
    assert abs(a - b) <= 1e-4 * (x.norm() * my.norm()).item(), (a, b)
    assert torch.dot(x, mx).item() > 0 and torch.dot(y, my).item() > 0
    op.close()


def test_flexible_twolevel_iterations_do_not_grow_with_the_mesh(sipg, torch):
    # FP32 inner iterations of the whole solve to a true 1e-10 (p = 4): flat
    # in dim, where plain CG's count doubles from 64^2 to 256^2
    counts = {}
    for dim in (64, 128, 256):
        op = sipg.Operator(dim, 4, 16.0)
        b = op.rhs("sinsin")
        x = torch.zeros_like(b)
        st, rm = op.solve_mixed(x, b, inner_tol=1e-2, outer_tol=1e-10)
        assert st == 0 and rm.inner_kind == 4 and rm.outer_kind == 2
        assert (b - op.apply(x)).norm().item() / b.norm().item() <= 1.01e-10
        counts[dim] = rm.inner_iterations
        op.close()
    assert counts[256] <= 1.5 * counts[64], counts
    assert counts[256] <= 400, counts
