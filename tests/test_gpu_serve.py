"""The continuous-batching server (sipg_server_*): requests of mixed sizes,
degrees, precisions and tolerances submitted while others are mid-solve all
retire with ||b - Ax|| <= tol ||b||, and each result is the same alone and in
the mix: within 1e-6 relative of the single-problem FP64 CG solution to 1e-12
(the served solves stop at 1e-8 / 1e-10).  Admission respects the memory
budget and rejects requests larger than it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t

    return t


def _requests(sipg, rng, n):
    out = []
    for _ in range(n):
        dim = int(np.exp(rng.uniform(np.log(8), np.log(40))))
        p = int(rng.integers(2, 9))
        modes = sipg.Modes.make(rng.normal(size=4), rng.integers(1, 9, 4), rng.integers(1, 9, 4))
        tol = float(rng.choice([1e-8, 1e-10]))
        prec = int(rng.integers(0, 2))
        out.append((dim, p, float(p * p), tol, modes, prec))
    return out


def _reference(sipg, torch, dim, p, pen, modes):
    op = sipg.Operator(dim, p, pen)
    b = op.rhs("modes", modes)
    x = torch.zeros_like(b)
    st, _ = op.cg(x, b, 1e-12, relative=True)
    assert st == 0
    op.close()
    return x.cpu().numpy()


def test_server_mixed_stream_matches_single_solves(sipg, torch):
    rng = np.random.default_rng(3)
    reqs = _requests(sipg, rng, 24)
    sv = sipg.Server(budget_bytes=2 << 30, max_active=8, iters_per_step=8)
    ids = []
    pending = list(reqs)
    # submit a few, step, submit more while the first are mid-solve
    for _ in range(3):
        ids.append(sv.submit(*pending.pop(0)[:4], modes=reqs[len(ids)][4], precision=reqs[len(ids)][5])[0])
    sv.step()
    while pending:
        d, p, pen, tol, modes, prec = pending.pop(0)
        ids.append(sv.submit(d, p, pen, tol, modes=modes, precision=prec)[0])
        sv.step()
    for _ in range(100000):
        active, _ = sv.step()
        if active == 0 and sv.stats().queued == 0:
            break
    assert sv.stats().completed == len(reqs)
    for rid, (d, p, pen, tol, modes, prec) in zip(ids, reqs):
        res = sv.poll(rid)
        assert res.done == 1 and res.status == 0, (d, p, prec, res.status)
        assert res.rel_residual <= tol
        x = sv.solution(rid, d * d * (p + 1) ** 2)
        ref = _reference(sipg, torch, d, p, pen, modes)
        assert np.max(np.abs(x - ref)) <= (1e-4 if tol == 1e-8 else 1e-6) * np.max(np.abs(ref)), (d, p, tol, prec)
        sv.release(rid)
    assert sv.stats().bytes_in_use == 0
    sv.close()


def test_server_alone_equals_in_mix(sipg, torch):
    rng = np.random.default_rng(5)
    d, p, pen, tol = 24, 5, 25.0, 1e-10
    modes = sipg.Modes.make([1.0, -0.5, 0.25, 2.0], [1, 2, 5, 3], [3, 1, 4, 6])
    alone = sipg.Server(max_active=1)
    rid, _ = alone.submit(d, p, pen, tol, modes=modes)
    while alone.step()[0] or alone.stats().queued:
        pass
    xa = alone.solution(rid, d * d * (p + 1) ** 2)
    mix = sipg.Server(max_active=16)
    others = _requests(sipg, rng, 10)
    for o in others[:5]:
        mix.submit(*o[:4], modes=o[4], precision=o[5])
    rid2, _ = mix.submit(d, p, pen, tol, modes=modes)
    for o in others[5:]:
        mix.submit(*o[:4], modes=o[4], precision=o[5])
    while mix.step()[0] or mix.stats().queued:
        pass
    xm = mix.solution(rid2, d * d * (p + 1) ** 2)
    # the batched kernels give every request the same arithmetic whatever runs beside it
    assert np.array_equal(xa, xm)
    alone.close()
    mix.close()


def test_server_budget_admission_and_rejection(sipg, torch):
    sv = sipg.Server(budget_bytes=64 << 20, max_active=64)
    modes = sipg.Modes.make([1.0], [1], [1])
    big, st = sv.submit(512, 8, 64.0, 1e-8, modes=modes)
    assert st == 7 and sv.poll(big).status == 7  # SIPG_ERR_REJECTED
    ids = [sv.submit(48, 4, 16.0, 1e-8, modes=modes)[0] for _ in range(12)]
    peak = 0
    while True:
        active, _ = sv.step()
        peak = max(peak, sv.stats().bytes_in_use)
        if active == 0 and sv.stats().queued == 0:
            break
    assert peak <= 64 << 20
    assert all(sv.poll(i).status == 0 for i in ids)
    sv.close()


def test_server_small_request_not_held_behind_a_large_one(sipg, torch):
    """Requests run in size-class lanes stepped independently: a small solve
    submitted after a large one retires while the large one is still running
    (in lockstep it would advance one iteration per large-solve iteration)."""
    sv = sipg.Server(max_active=8, iters_per_step=8)
    modes = sipg.Modes.make([1.0, 0.5], [1, 3], [2, 1])
    big, _ = sv.submit(400, 8, 64.0, 1e-10, modes=modes)  # ~13 M DoF: the large lane
    sv.step()
    small, _ = sv.submit(16, 3, 9.0, 1e-10, modes=modes)  # 4096 DoF: the small lane
    for _ in range(100000):
        sv.step()
        if sv.poll(small).done:
            break
    rs, rb = sv.poll(small), sv.poll(big)
    assert rs.done == 1 and rs.status == 0 and rs.rel_residual <= 1e-10
    assert rb.done == 0, "the small request waited for the large one"
    x = sv.solution(small, 16 * 16 * 16)
    ref = _reference(sipg, torch, 16, 3, 9.0, modes)
    assert np.max(np.abs(x - ref)) <= 1e-6 * np.max(np.abs(ref))
    sv.close()  # the large request is dropped unfinished


def test_server_interleaved_precisions_against_the_oracle(sipg, oracle, torch):
    """Mixed-precision (flexible CG in FP64 around an FP32 inner CG) and plain
    FP64 requests on 64^2..128^2 meshes, interleaved in one server: every
    result reaches a true relative residual under its tolerance (recomputed
    here in FP64) and agrees with the oracle's CG (the reference's algorithm
    restated in C) to 1e-12 within the bound the two residuals allow."""
    cases = [(64, 4, 1e-10, sipg.F32), (96, 3, 1e-10, sipg.F64), (128, 2, 1e-8, sipg.F32),
             (80, 6, 1e-10, sipg.F32), (64, 5, 1e-8, sipg.F64), (112, 4, 1e-10, sipg.F32)]
    modes = sipg.Modes.make([1.0, -0.7, 0.3, 1.5], [1, 4, 7, 2], [2, 3, 1, 8])
    sv = sipg.Server(max_active=8, iters_per_step=8)
    ids = []
    for d, p, tol, prec in cases:
        ids.append(sv.submit(d, p, float(p * p), tol, modes=modes, precision=prec)[0])
        sv.step()
    for _ in range(1000000):
        active, _ = sv.step()
        if active == 0 and sv.stats().queued == 0:
            break
    for rid, (d, p, tol, prec) in zip(ids, cases):
        res = sv.poll(rid)
        assert res.done == 1 and res.status == 0, (d, p, prec, res.status)
        n = d * d * (p + 1) ** 2
        x = sv.solution(rid, n)
        op = sipg.Operator(d, p, float(p * p))
        b = op.rhs("modes", modes)
        xt = torch.from_numpy(x).cuda()
        true_rel = op.true_residual(xt, b)
        assert true_rel <= 1.01 * tol, (d, p, prec, true_rel)
        it_ref, x_ref, _ = oracle.cg(p, d, float(p * p), b.cpu().numpy(), 1e-12, rel=True, nthreads=8)
        bound = 1e-4 if tol == 1e-8 else 1e-6
        assert np.max(np.abs(x - x_ref)) <= bound * np.max(np.abs(x_ref)), (d, p, prec)
        if prec == sipg.F32:
            assert res.corrections >= 1 and res.iterations > 0
        op.close()
        sv.release(rid)
    sv.close()


def test_server_closes_with_preparations_pending(sipg, torch):
    """Mixed requests start their preparation (operator and two-level
    preconditioner, on the server's preparation threads) at submission; a
    server closed before any step joins those threads and frees everything,
    and a fresh server then serves the same requests."""
    reqs = [(d, p, float(p * p)) for d, p in ((64, 4), (40, 6), (96, 3), (33, 8), (71, 2), (128, 5))]
    srv = sipg.Server(budget_bytes=8 << 30, max_active=16, iters_per_step=8)
    for d, p, pen in reqs:
        _, st = srv.submit(d, p, pen, 1e-8, "sinsin", None, precision=sipg.F32)
        assert st == 0
    srv.close()
    srv = sipg.Server(budget_bytes=8 << 30, max_active=16, iters_per_step=8)
    ids = [srv.submit(d, p, pen, 1e-8, "sinsin", None, precision=sipg.F32)[0] for d, p, pen in reqs]
    done = {}
    import time

    t_end = time.time() + 120
    while time.time() < t_end:
        srv.step()
        for rid in ids:
            if rid not in done:
                r = srv.poll(rid)
                if r.done:
                    done[rid] = (r.status, r.rel_residual)
        if len(done) == len(ids):
            break
    assert len(done) == len(ids)
    for status, rel in done.values():
        assert status == 0 and rel <= 1e-8
    assert srv.stats().prep_ms > 0
    srv.close()
