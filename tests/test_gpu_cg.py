"""CUDA conjugate gradient, RHS and error norms against the reference.

Iteration counts must be within +-1 of the reference's own CG on the same
problem (its dots are cuBLAS, order unspecified); solutions agree to the CG
tolerance; error norms reproduce the reference's and the thesis's values.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t

    assert t.cuda.is_available()
    return t


def test_rhs_matches_oracle(sipg, oracle, torch):
    for sol in (1, 2, 3, 4, 5, 6):
        for p, d in ((2, 4), (4, 7), (3, 1), (6, 33)):
            pen = float(p * p)
            op = sipg.Operator(d, p, pen)
            b = op.rhs(sol).cpu().numpy()
            op.close()
            ref = oracle.rhs(p, d, pen, sol)
            assert np.max(np.abs(b - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref))), (sol, p, d)


def test_rhs_modes_matches_oracle(sipg, oracle, torch):
    amps, ks, ls = [0.3, -1.2, 0.7, 2.0], [1, 3, 8, 5], [2, 7, 1, 5]
    p, d, pen = 4, 20, 16.0
    op = sipg.Operator(d, p, pen)
    b = op.rhs("modes", sipg.Modes.make(amps, ks, ls)).cpu().numpy()
    ref = oracle.rhs(p, d, pen, 7, oracle.modes(amps, ks, ls))
    assert np.max(np.abs(b - ref)) <= 1e-13 * np.max(np.abs(ref))
    op.close()


def test_cg_matches_reference_solves(sipg, golden, torch):
    for i, row in enumerate(golden["solve_table"]):
        sol, p, d, pen, tol = int(row[0]), int(row[1]), int(row[2]), float(row[3]), float(row[4])
        it_ref, l2_ref, h1_ref, mx_ref = row[5:9]
        op = sipg.Operator(d, p, pen)
        b = torch.from_numpy(golden["solve_rhs_%d" % i]).cuda()
        x = torch.zeros_like(b)
        st, res = op.cg(x, b, tol)
        assert st == 0, (i, st)
        assert abs(res.iterations - int(it_ref)) <= 1, (i, res.iterations, it_ref)
        u_ref = golden["solve_u_%d" % i]
        assert np.max(np.abs(x.cpu().numpy() - u_ref)) <= 1e-8 * np.max(np.abs(u_ref)), i
        l2, h1, mx = op.err_norms(sol, x)
        assert l2 == pytest.approx(l2_ref, rel=1e-6) and h1 == pytest.approx(h1_ref, rel=1e-6)
        assert mx == pytest.approx(mx_ref, rel=1e-6)
        op.close()


def test_poisson16_relative_tolerance(sipg, golden, torch):
    # 16x16, p = 4, sin-sin, pen = p^2, CG from 0 to ||r|| <= 1e-12 ||b||
    p, d, pen, tol_abs, it_ref, l2_ref, h1_ref, mx_ref = golden["poisson16_stats"]
    op = sipg.Operator(int(d), int(p), pen)
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-12, relative=True)
    assert st == 0
    assert abs(res.iterations - int(it_ref)) <= 1
    assert res.stop == pytest.approx(tol_abs, rel=1e-12)
    l2, h1, mx = op.err_norms("sinsin", x)
    assert l2 == pytest.approx(l2_ref, rel=1e-4) and h1 == pytest.approx(h1_ref, rel=1e-4)
    op.close()


@pytest.mark.parametrize("p,d", [(2, 16), (3, 16), (4, 16), (5, 8), (6, 8)])
def test_thesis_table_4_10_on_gpu(sipg, torch, p, d):
    from test_oracle_golden import THESIS_T4_10

    H1, L2, LI = THESIS_T4_10[(p, d)]
    op = sipg.Operator(d, p, 100.0 * p * p)
    b = op.rhs("E")
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-15)
    l2, h1, mx = op.err_norms("E", x)
    assert h1 == pytest.approx(H1, rel=1e-5) and l2 == pytest.approx(L2, rel=1e-5)
    op.close()


def test_cg_larger_mesh_vs_oracle_iterations(sipg, oracle, torch):
    p, d, pen = 4, 48, 16.0
    b_np = oracle.rhs(p, d, pen, 1)
    it_ref, x_ref, _ = oracle.cg(p, d, pen, b_np, 1e-10, rel=True, nthreads=8)
    op = sipg.Operator(d, p, pen)
    b = torch.from_numpy(b_np).cuda()
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-10, relative=True)
    assert st == 0 and abs(res.iterations - it_ref) <= 1
    assert np.max(np.abs(x.cpu().numpy() - x_ref)) <= 1e-8 * np.max(np.abs(x_ref))
    op.close()


def test_cg_max_it_and_breakdown_statuses(sipg, torch):
    op = sipg.Operator(8, 3, 9.0)
    b = op.rhs("A")
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-30, max_it=5)
    assert st == 3 and res.iterations == 5 and res.converged == 0
    # a negative penalty makes the operator indefinite: CG reports breakdown
    bad = sipg.Operator(8, 3, -50.0)
    x2 = torch.zeros_like(b)
    st2, res2 = bad.cg(x2, b, 1e-12, max_it=500)
    assert st2 in (3, 4)
    op.close()
    bad.close()


def test_cg_zero_rhs_returns_immediately(sipg, torch):
    op = sipg.Operator(4, 2, 4.0)
    b = torch.zeros(op.ndof, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-12, relative=False)
    assert st == 0 and res.iterations == 0
    op.close()


def test_cg_f32(sipg, oracle, torch):
    p, d, pen = 3, 24, 9.0
    op = sipg.Operator(d, p, pen)
    b = op.rhs("A")
    x = torch.zeros_like(b, dtype=torch.float32)
    st, res = op.cg(x, b.float(), 1e-5, relative=True)
    assert st == 0
    it_ref, x_ref, _ = oracle.cg(p, d, pen, b.cpu().numpy(), 1e-12, rel=True, nthreads=4)
    assert np.max(np.abs(x.double().cpu().numpy() - x_ref)) <= 1e-3 * np.max(np.abs(x_ref))
    op.close()


def test_mixed_precision_reaches_fp64_accuracy(sipg, oracle, torch):
    # a problem whose discretisation error (~1e-8) is far above round-off, so
    # "L2 error within 1.05x of the FP64 solve" is a meaningful comparison
    p, d, pen = 3, 32, 9.0
    op = sipg.Operator(d, p, pen)
    b = op.rhs("sinsin")
    x64 = torch.zeros_like(b)
    st, r64 = op.cg(x64, b, 1e-10, relative=True)
    assert st == 0
    xm = torch.zeros_like(b)
    st, rm = op.solve_mixed(xm, b, inner_tol=0.1, outer_tol=1e-10, inner="f32", outer="reliable")
    assert st == 0 and rm.converged == 1 and rm.rel_residual <= 1e-10 and rm.inner_kind == 1
    assert rm.outer_kind == 1
    assert rm.outer_iterations >= 2 and rm.inner_iterations > 0
    # reliable updates keep the Krylov space: the FP32 iteration count stays within
    # a small factor of the FP64 one (a restarted inner solve needs orders of magnitude more)
    assert rm.inner_iterations <= 3 * r64.iterations
    e64 = op.err_norms("sinsin", x64)
    em = op.err_norms("sinsin", xm)
    assert em[0] <= 1.05 * e64[0]
    # both solves stop at ||b - Ax|| <= 1e-10 ||b||: their difference is bounded by the residuals
    assert (xm - x64).abs().max().item() <= 1e-7 * x64.abs().max().item()
    op.close()


def test_mixed_pairs_on_an_ill_conditioned_problem(sipg, torch):
    # 256 x 256, p = 6: condition number ~5e6, a quarter of 1 / eps_32 -- FP32
    # vectors cannot carry the iteration; double-float pairs reach a TRUE FP64
    # relative residual of 1e-10.  (The FP64 CG stops on its iterated residual;
    # here its true residual stalls near 3e-10, so its iteration count is only
    # a yardstick.)
    p, d, pen = 6, 256, 36.0
    op = sipg.Operator(d, p, pen)
    b = op.rhs("sinsin")
    bn = b.norm().item()
    x64 = torch.zeros_like(b)
    st, r64 = op.cg(x64, b, 1e-10, relative=True)
    assert st == 0
    xm = torch.zeros_like(b)
    st, rm = op.solve_mixed(xm, b, inner_tol=0.1, outer_tol=1e-10, inner="pairs")  # reliable updates
    assert st == 0 and rm.converged == 1 and rm.rel_residual <= 1e-10
    assert rm.inner_kind == 2 and rm.outer_kind == 1
    true_rel = op.true_residual(xm, b)
    assert true_rel <= 1.01e-10, true_rel
    assert rm.inner_iterations <= 3 * r64.iterations, (rm.inner_iterations, r64.iterations)
    e64 = op.err_norms("sinsin", x64)
    em = op.err_norms("sinsin", xm)
    slack = 2.0 * (xm - x64).abs().max().item()
    assert em[0] <= 1.05 * e64[0] + slack, (em, e64)
    assert (xm - x64).abs().max().item() <= 1e-7 * x64.abs().max().item()
    op.close()


def test_mixed_auto_picks_flexible_twolevel(sipg, torch):
    op = sipg.Operator(16, 2, 4.0)
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, rm = op.solve_mixed(x, b)
    assert st == 0 and rm.inner_kind == 4 and rm.outer_kind == 2 and rm.rel_residual <= 1e-10
    # the reliable-update loop with auto inner still picks FP32 vectors on a well-conditioned problem
    x.zero_()
    st, rm = op.solve_mixed(x, b, outer="reliable")
    assert st == 0 and rm.inner_kind == 1 and rm.outer_kind == 1 and rm.rel_residual <= 1e-10
    op.close()


def _true_rel(op, x, b):
    # b - A x in FP64 with the operator's zero-sum contractions over differences
    return op.true_residual(x, b)


@pytest.mark.parametrize("inner,inner_tol", [("twolevel", 1e-1), ("twolevel", 1e-3), ("twolevel", 1e-5),
                                             ("f32", 1e-1)])
def test_flexible_fp32_inner_on_an_ill_conditioned_problem(sipg, oracle, torch, inner, inner_tol):
    # 256 x 256, p = 6: condition number ~5e6 (kappa * eps_32 ~ 0.3), where FP32
    # vectors stall a unit-step defect correction.  Flexible CG in FP64 with a
    # pure FP32 inner CG (FP32 values, FP32 accumulation) reaches a TRUE FP64
    # relative residual of 1e-10, L2 error within 1.05x of the FP64 solve's.
    p, d, pen = 6, 256, 36.0
    op = sipg.Operator(d, p, pen)
    b = op.rhs("sinsin")
    x64 = torch.zeros_like(b)
    st, rr = op.solve_mixed(x64, b, inner_tol=0.1, outer_tol=1e-10, inner="f64", outer="reliable")
    # (the all-FP64 yardstick checks itself with the plain FP64 sums, those of its inner apply)
    assert st == 0 and rr.rel_residual <= 1e-10
    xm = torch.zeros_like(b)
    st, rm = op.solve_mixed(xm, b, inner_tol=inner_tol, outer_tol=1e-10, inner=inner, outer="flexible")
    assert st == 0 and rm.converged == 1 and rm.inner_kind == sipg.INNER[inner] and rm.outer_kind == 2
    assert rm.rel_residual <= 1e-10
    true_rel = _true_rel(op, xm, b)
    assert true_rel <= 1.01e-10, true_rel
    # one FP64 apply per outer step, plus the residual checks
    assert rm.outer_iterations + 1 <= rm.fp64_applies <= rm.outer_iterations + 4
    e64 = op.err_norms("sinsin", x64)
    em = op.err_norms("sinsin", xm)
    # here the discretisation error (~1.5e-12) is below what a relative
    # residual of 1e-10 pins down: the difference of the two solutions
    # bounds the difference of their errors
    slack = 2.0 * (xm - x64).abs().max().item()
    assert em[0] <= 1.05 * e64[0] + slack, (em, e64)
    assert (xm - x64).abs().max().item() <= 1e-7 * x64.abs().max().item()
    op.close()


def test_flexible_matches_the_oracle_solution(sipg, oracle, torch):
    # a small mesh where the oracle's CG to 1e-13 is the answer: the flexible
    # mixed solve to 1e-11 lands within the residual bound of it
    p, d, pen = 4, 24, 16.0
    op = sipg.Operator(d, p, pen)
    b = op.rhs("sinsin")
    it_ref, x_ref, _ = oracle.cg(p, d, pen, b.cpu().numpy(), 1e-13, rel=True, nthreads=4)
    x = torch.zeros_like(b)
    st, rm = op.solve_mixed(x, b, inner_tol=1e-2, outer_tol=1e-11, outer="flexible")
    assert st == 0 and rm.outer_kind == 2 and rm.rel_residual <= 1e-11
    diff = np.max(np.abs(x.cpu().numpy() - x_ref)) / np.max(np.abs(x_ref))
    assert diff <= 1e-8, diff
    op.close()


def test_flexible_rejects_a_pairs_inner(sipg, torch):
    op = sipg.Operator(8, 3, 9.0)
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    with pytest.raises(sipg.SipgError):
        op.solve_mixed(x, b, inner="pairs", outer="flexible")
    op.close()


def test_flexible_reports_not_converged_at_max_outer(sipg, torch):
    op = sipg.Operator(64, 4, 16.0)
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, rm = op.solve_mixed(x, b, inner_tol=0.5, outer_tol=1e-12, max_outer=2, outer="flexible")
    assert st == 3 and rm.converged == 0 and rm.outer_iterations == 2
    op.close()


def test_persistent_cg_barrier_gives_up_and_device_stays_usable(sipg, torch):
    """The persistent small-mesh CG's grid barrier with a target no arrival
    count reaches: every CTA's bounded wait runs out and reports it (no fault,
    no hang), and the next solve runs normally."""
    assert sipg.selftest_barrier_timeout()
    op = sipg.Operator(16, 4, 16.0)
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-12, relative=True)
    assert st == 0 and res.converged == 1 and abs(res.iterations - 136) <= 1
    op.close()
