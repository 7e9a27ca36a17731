"""Batched mixed-precision solves (sipg_batch_*): many right-hand sides on one
mesh and uneven (dim, p) problems in one batch must give, problem by problem,
what the single-problem FP64 CG gives: FP64 relative residual <= 1e-10, the
solution within 1e-7 relative of the FP64 CG solution (both stop at 1e-10),
and the L2 error within 1.05x of the FP64 solve's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t

    return t


def _modes(sipg, rng):
    return sipg.Modes.make(rng.normal(size=4), rng.integers(1, 9, 4), rng.integers(1, 9, 4))


def _fp64_reference(sipg, torch, op, b):
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-10, relative=True)
    assert st == 0
    return x


def test_batch_many_rhs_shared_mesh(sipg, torch):
    rng = np.random.default_rng(1)
    dim, p, pen = 24, 3, 9.0
    nrhs = 6
    batch = sipg.Batch([(dim, p, pen)] * nrhs)
    bs, refs = [], []
    single = sipg.Operator(dim, p, pen)
    for k in range(nrhs):
        m = _modes(sipg, rng)
        b = batch.op(k).rhs("modes", m)
        bs.append(b)
        refs.append(_fp64_reference(sipg, torch, single, b))
    xs = [torch.zeros_like(b) for b in bs]
    st, res = batch.solve_mixed(xs, bs)
    assert st == 0
    for k in range(nrhs):
        assert res[k].converged == 1 and res[k].rel_residual <= 1e-10
        assert (xs[k] - refs[k]).abs().max().item() <= 1e-7 * refs[k].abs().max().item()
    single.close()
    batch.close()


def test_batch_uneven_problems(sipg, torch):
    probs = [(16, 2, 4.0), (37, 5, 25.0), (20, 8, 64.0), (33, 3, 9.0), (8, 7, 49.0), (45, 4, 16.0)]
    batch = sipg.Batch(probs)
    bs = [batch.op(k).rhs("sinsin") for k in range(len(probs))]
    xs = [torch.zeros_like(b) for b in bs]
    st, res = batch.solve_mixed(xs, bs)
    assert st == 0
    for k, (d, p, pen) in enumerate(probs):
        op = sipg.Operator(d, p, pen)
        ref = _fp64_reference(sipg, torch, op, bs[k])
        assert res[k].converged == 1 and res[k].rel_residual <= 1e-10
        assert (xs[k] - ref).abs().max().item() <= 1e-7 * ref.abs().max().item(), k
        e_ref = op.err_norms("sinsin", ref)
        e_b = op.err_norms("sinsin", xs[k])
        # both stop at relative residual 1e-10; where the discretisation error
        # is below what that allows (p = 5 on 37 x 37: 3e-13), the difference of
        # the two solutions bounds the difference of their errors
        slack = 2.0 * (xs[k] - ref).abs().max().item()
        assert e_b[0] <= 1.05 * e_ref[0] + slack, (k, e_b, e_ref)
        op.close()
    batch.close()


def test_batch_retires_converged_problems(sipg, torch):
    # a zero right-hand side converges before any iteration; the others go on
    probs = [(12, 2, 4.0), (12, 2, 4.0), (30, 6, 36.0)]
    batch = sipg.Batch(probs)
    bs = [torch.zeros(batch.op(0).ndof, dtype=torch.float64, device="cuda"), batch.op(1).rhs("A"),
          batch.op(2).rhs("E")]
    xs = [torch.zeros_like(b) for b in bs]
    st, res = batch.solve_mixed(xs, bs)
    assert st == 0
    assert res[0].converged == 1 and res[0].inner_iterations == 0 and res[0].outer_iterations == 0
    assert res[1].inner_iterations < res[2].inner_iterations
    assert all(r.rel_residual <= 1e-10 for r in res[1:])
    # solving again reuses the resident state and graph
    xs2 = [torch.zeros_like(b) for b in bs]
    st, res2 = batch.solve_mixed(xs2, bs)
    assert st == 0 and all(torch.equal(a, c) for a, c in zip(xs, xs2))
    batch.close()
