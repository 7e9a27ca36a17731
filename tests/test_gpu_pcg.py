"""The block-Jacobi preconditioner and the preconditioned CG (the reference's
USE_PRECONDITIONER path) against the oracle, which is pinned bit for bit to
the reference's own code built with that macro (tests/golden/).

Tolerances: the preconditioner apply to 1e-13 relative (max |z - z_ref| /
max |z_ref|: the same 2p+1 products per value, in FP64); preconditioned
solves: iteration counts within max(1, 1 %) of the reference's (its dots are
cuBLAS, order unspecified) -- within 40 % where the tolerance sits at the
rounding floor of the residual -- solutions to 1e-8 relative, error norms to
1e-6 relative."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cuda-sipg-matrix-free_gb300")


@pytest.fixture(scope="module")
def torch():
    import torch as t

    return t


def _close_iterations(it, it_ref, tol):
    if tol < 1e-14:
        return abs(it - it_ref) <= max(2, int(0.4 * it_ref))
    return abs(it - it_ref) <= max(1, int(0.01 * it_ref))


@pytest.mark.parametrize("p", range(1, 9))
def test_prec_apply_matches_oracle(sipg, oracle, torch, p):
    d = 9
    for pen in (float(p * p), 100.0 * p * p, 37.9):
        op = sipg.Operator(d, p, pen)
        x = np.random.default_rng(p).uniform(-1, 1, op.ndof)
        z = op.apply_prec(torch.from_numpy(x).cuda()).cpu().numpy()
        zr = oracle.prec_apply(p, d, oracle.prec_rows(p, pen), x)
        assert np.max(np.abs(z - zr)) <= 1e-13 * np.max(np.abs(zr)), (p, pen)
        op.close()


def test_pcg_matches_reference_solves(sipg, golden, torch):
    for i, row in enumerate(golden["pcg_table"]):
        sol, p, d, pen, tol = int(row[0]), int(row[1]), int(row[2]), float(row[3]), float(row[4])
        op = sipg.Operator(d, p, pen)
        b = torch.from_numpy(golden["pcg_rhs_%d" % i]).cuda()
        x = torch.zeros_like(b)
        st, res = op.pcg(x, b, tol)
        assert st in (0, 3), (i, st)
        assert _close_iterations(res.iterations, int(row[5]), tol), (i, res.iterations, row[5])
        u = golden["pcg_u_%d" % i]
        assert np.max(np.abs(x.cpu().numpy() - u)) <= 1e-8 * np.max(np.abs(u)), i
        l2, h1, mx = op.err_norms(sol, x)
        assert l2 == pytest.approx(row[6], rel=1e-6) and h1 == pytest.approx(row[7], rel=1e-6)
        op.close()


def test_pcg_relative_tolerance_and_zero_rhs(sipg, oracle, torch):
    p, d, pen = 4, 16, 16.0
    op = sipg.Operator(d, p, pen)
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, res = op.pcg(x, b, 1e-10, relative=True)
    it_ref, x_ref, _ = oracle.pcg(p, d, pen, b.cpu().numpy(), 1e-10, rel=True)
    assert st == 0 and res.converged == 1 and _close_iterations(res.iterations, it_ref, 1e-10)
    assert np.max(np.abs(x.cpu().numpy() - x_ref)) <= 1e-8 * np.max(np.abs(x_ref))
    # b = 0: r = 0, nothing to do
    z = torch.zeros_like(b)
    st, res = op.pcg(z, torch.zeros_like(b), 1e-12)
    assert st == 0 and res.iterations == 0 and float(z.abs().max()) == 0.0
    op.close()


@pytest.fixture(scope="module")
def pcg_driver_output(sipg, tmp_path_factory):
    sipg.lib()
    exe = str(tmp_path_factory.mktemp("cpp") / "host_api_pcg_driver")
    subprocess.check_call(["nvcc", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                           os.path.join(PKG, "host"), os.path.join(ROOT, "tests", "cpp", "host_api_pcg_driver.cpp"),
                           "-L", os.path.join(PKG, "lib"), "-lsipg_gb300", "-Xlinker",
                           "-rpath=" + os.path.join(PKG, "lib"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    return [json.loads(line) for line in out.stdout.splitlines() if line.startswith("{")]


def test_host_api_with_use_preconditioner(pcg_driver_output, oracle):
    from test_oracle_golden import THESIS_T4_10

    rows = [r for r in pcg_driver_output if r["case"] == "pcg"]
    assert len(rows) == 9
    seen = 0
    for r in rows:
        p, d, pen, tol = r["p"], r["dim"], r["pen"], r["tol"]
        b = oracle.rhs(p, d, pen, 5)
        it, x, _ = oracle.pcg(p, d, pen, b, tol)
        l2, h1, _ = oracle.err_norms(p, d, 5, x)
        assert _close_iterations(r["it"], it, tol), (r, it)
        assert r["L2"] == pytest.approx(l2, rel=1e-6) and r["H1"] == pytest.approx(h1, rel=1e-6)
        if (p, d) in THESIS_T4_10:
            H1, L2, _ = THESIS_T4_10[(p, d)]
            assert r["H1"] == pytest.approx(H1, rel=1e-5) and r["L2"] == pytest.approx(L2, rel=1e-5)
            seen += 1
    assert seen >= 6
    gen = next(r for r in pcg_driver_output if r["case"] == "generic")
    assert abs(gen["it_generic"] - gen["it_fused"]) <= 1 and gen["rel_diff"] <= 1e-9


def _laplacian_rows(oracle, p):
    """host_laplacian_matrix (mode_matrix.hpp:419-466) rows from the oracle's
    element Laplacian: the diagonal, then (i1, j != i2), then (j != i1, i2)."""
    n = p + 1
    L = oracle.laplace2d(p).reshape(n, n, n, n)  # [i1, i2, j1, j2]
    rows = []
    for i1 in range(n):
        for i2 in range(n):
            rows.append(L[i1, i2, i1, i2])
            rows += [L[i1, i2, i1, j] for j in range(n) if j != i2]
            rows += [L[i1, i2, j, i2] for j in range(n) if j != i1]
    return np.array(rows)


@pytest.mark.parametrize("p", range(1, 9))
def test_stored_operator_apply_matches_reference(sipg, oracle, golden, torch, p):
    # the reference's volume_mvm<T,1> with the Laplacian mode matrix, on the
    # golden inputs (tests/golden: its outputs, from the reference's code)
    rows = torch.from_numpy(sipg.laplacian_rows(p)).cuda()  # the product's builder
    assert np.max(np.abs(rows.cpu().numpy() - _laplacian_rows(oracle, p))) <= 1e-13 * rows.abs().max().item()
    for d in (1, 2, 3):
        x = golden["apply_in_%d_%d" % (p, d)]
        y = sipg.volume_mvm(d, p, rows, torch.from_numpy(x).cuda()).cpu().numpy()
        ref = golden["volume_mvm_out_%d_%d" % (p, d)]
        assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref)), (p, d)


def test_stored_operator_per_element(sipg, torch):
    # volume_mvm<T,0>: a different operator per element, mode_matrix layout
    p, d = 3, 5
    n, R, noe = p + 1, 2 * p + 1, d * d
    rng = np.random.default_rng(7)
    mat = rng.normal(size=(n * n, R, noe))  # [row k][entry r][element e]
    x = rng.normal(size=(n * n, noe))
    ref = np.zeros_like(x)
    for i1 in range(n):
        for i2 in range(n):
            k = i1 * n + i2
            cols = [k] + [i1 * n + j for j in range(n) if j != i2] + [j * n + i2 for j in range(n) if j != i1]
            ref[k] = sum(mat[k, r] * x[c] for r, c in enumerate(cols))
    y = sipg.volume_mvm(d, p, torch.from_numpy(mat.ravel()).cuda(), torch.from_numpy(x.ravel()).cuda())
    assert np.max(np.abs(y.cpu().numpy().reshape(n * n, noe) - ref)) <= 1e-13 * np.max(np.abs(ref))
