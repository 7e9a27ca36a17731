"""Batched mixed-precision solves (sipg_batch_*: flexible CG in FP64 around an
FP32 inner CG): many right-hand sides on one mesh and uneven (dim, p) problems
in one batch must give, problem by problem, what the single-problem FP64 CG
gives: FP64 relative residual <= 1e-10 (recomputed from the solution), the
solution within 1e-7 relative of the FP64 CG solution (both stop at 1e-10),
and the L2 error within 1.05x of the FP64 solve's; at the 64-right-hand-side,
256 x 256, p = 4 shape one instance is checked against the oracle's CG."""
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


def _true_rel(op, x, b):
    # b - A x in FP64 with the operator's zero-sum contractions over differences
    return op.true_residual(x, b)


def test_batch_reports_the_flexible_fp32_scheme(sipg, torch):
    probs = [(20, 4, 16.0), (28, 6, 36.0)]
    batch = sipg.Batch(probs)
    bs = [batch.op(k).rhs("sinsin") for k in range(len(probs))]
    xs = [torch.zeros_like(b) for b in bs]
    st, res = batch.solve_mixed(xs, bs)
    assert st == 0
    for k, r in enumerate(res):
        assert r.inner_kind == 4 and r.outer_kind == 2 and r.converged == 1
        # one FP64 apply per outer step, the initial residual and the final check(s)
        assert r.outer_iterations + 2 <= r.fp64_applies <= r.outer_iterations + 5
        assert _true_rel(batch.op(k), xs[k], bs[k]) <= 1.01e-10
    with pytest.raises(sipg.SipgError):
        # batches run the flexible scheme only
        o = sipg.MixedOpts(0.1, 1e-10, 200, 0, sipg.INNER["pairs"], sipg.OUTER["reliable"])
        px = (sipg.C.c_void_p * 2)(*[x.data_ptr() for x in xs])
        pb = (sipg.C.c_void_p * 2)(*[b.data_ptr() for b in bs])
        sipg._check(sipg.lib().sipg_batch_solve_mixed(batch._h, sipg.C.cast(px, sipg.C.c_void_p),
                                                       sipg.C.cast(pb, sipg.C.c_void_p), sipg.C.byref(o), None,
                                                       sipg._stream()), "batch")
    batch.close()


def test_batch_64_rhs_256_p4_against_the_oracle(sipg, oracle, torch):
    # the shared-mesh batch at full shape: 64 right-hand sides of 4 sine modes
    # (seed 1) on 256 x 256, p = 4 (104.9 M DoF in all)
    import workloads

    probs = workloads.shared_mesh_rhs(64, 256, 4, seed=1)
    batch = sipg.Batch([(d, p, pen) for d, p, pen, _ in probs])
    ms = [sipg.Modes.make(*m) for _, _, _, m in probs]
    bs = [batch.op(k).rhs("modes", ms[k]) for k in range(len(probs))]
    xs = [torch.zeros_like(b) for b in bs]
    st, res = batch.solve_mixed(xs, bs)
    assert st == 0
    op = batch.op(0)
    for k in range(len(probs)):
        assert res[k].converged == 1
        assert _true_rel(op, xs[k], bs[k]) <= 1.01e-10, k
    # instance 0 against the oracle (the reference's CG restated in C) to 1e-12
    d, p, pen, _ = probs[0]
    it_ref, x_ref, _ = oracle.cg(p, d, pen, bs[0].cpu().numpy(), 1e-12, rel=True, nthreads=16)
    diff = np.max(np.abs(xs[0].cpu().numpy() - x_ref)) / np.max(np.abs(x_ref))
    assert diff <= 1e-7, diff
    # the discretisation error of instance 0 against the analytic solution
    x64 = torch.from_numpy(x_ref).cuda()
    e_ref = op.err_norms("modes", x64, ms[0])
    e_b = op.err_norms("modes", xs[0], ms[0])
    assert e_b[0] <= 1.05 * e_ref[0], (e_b, e_ref)
    batch.close()
