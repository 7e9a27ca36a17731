"""The oracle (oracle/sipg_oracle.c) against the reference's own outputs.

tests/golden/reference_golden.npz holds outputs of paogor/CUDA-SIPG-matrix-free's
own code (its headers compiled for a CPU by oracle/build_ref.py, generated by
tests/golden/make_golden.py).  The oracle restates the same arithmetic in the
same order, so everything here is bit-exact except where noted.  The thesis
table at the end is the reference's published SIPG error table.
"""
import numpy as np
import pytest

import oracle_lib


def test_lgl_tables_bit_exact(oracle, golden):
    for n in range(2, 34):
        x, w = oracle.lgl(n)
        assert np.array_equal(x, golden["lgl_nodes_%d" % n]), n
        assert np.array_equal(w, golden["lgl_weights_%d" % n]), n


def test_lgl_closed_forms(oracle):
    # GLL_nodes_analytical_validation_test.cpp:11-52 (degrees 2..6)
    s = np.sqrt
    cases = {
        2: [-1, 0, 1],
        3: [-1, -1 / s(5), 1 / s(5), 1],
        4: [-1, -s(3) / s(7), 0, s(3) / s(7), 1],
        5: [-1, -s(2 * s(7) + 7) / s(21), -s(7 - 2 * s(7)) / s(21), s(7 - 2 * s(7)) / s(21), s(2 * s(7) + 7) / s(21), 1],
        6: [-1, -s(2 * s(15) + 15) / s(33), -s(15 - 2 * s(15)) / s(33), 0, s(15 - 2 * s(15)) / s(33),
            s(2 * s(15) + 15) / s(33), 1],
    }
    for deg, want in cases.items():
        x, _ = oracle.lgl(deg + 1)
        np.testing.assert_allclose(x, want, rtol=0, atol=4e-16)


def test_lgl_quadrature_exactness(oracle):
    # GLL_nodes_weights_validation_test.cpp:22-93: exact on [1,2] up to degree 2n-3
    a, b = 1.0, 2.0
    for n in range(2, 10):
        x, w = oracle.lgl(n)
        for deg in range(0, 2 * n - 2):
            q = np.sum(0.5 * (b - a) * w * (0.5 * (b - a) * x + 0.5 * (a + b)) ** deg)
            exact = (b ** (deg + 1) - a ** (deg + 1)) / (deg + 1)
            assert abs(q - exact) <= 1e-13 * max(1.0, abs(exact)), (n, deg)


def test_dphi_and_laplacian_bit_exact(oracle, golden):
    for p in range(1, 17):
        assert np.array_equal(oracle.dphi(p), golden["dphi_%d" % p]), p
    for p in range(1, 9):
        assert np.array_equal(oracle.laplace2d(p), golden["laplace2d_%d" % p]), p


def test_dphi_known_values(oracle):
    # p = 4: corner derivatives -N(N+1)/4 and the LGL weight w0 = 2/(N(N+1))
    D = oracle.dphi(4).reshape(5, 5)
    assert D[0, 0] == -5.0 and D[4, 4] == 5.0 and D[2, 2] == 0.0
    x, w = oracle.lgl(5)
    assert w[0] == pytest.approx(0.1, rel=1e-15)
    assert x[1] == pytest.approx(-0.6546536707079772, rel=1e-15)


def test_mesh_coords_bit_exact(oracle, golden):
    for d in (1, 2, 3, 16):
        x, y = oracle.mesh_coords(d)
        assert np.array_equal(x, golden["mesh_x_%d" % d])
        assert np.array_equal(y, golden["mesh_y_%d" % d])


def _apply_cases(golden):
    return sorted({tuple(int(v) for v in k.split("_")[2:4]) for k in golden.files if k.startswith("apply_in_")})


def test_apply_bit_exact(oracle, golden):
    for (p, d) in _apply_cases(golden):
        x = golden["apply_in_%d_%d" % (p, d)]
        y = oracle.apply(p, d, float(p * p), x, nthreads=1)
        assert np.array_equal(y, golden["apply_out_ref_%d_%d" % (p, d)]), (p, d)
        if "apply_out_thesis_%d_%d" % (p, d) in golden.files:
            y = oracle.apply(p, d, 100.0 * p * p, x, nthreads=3)
            assert np.array_equal(y, golden["apply_out_thesis_%d_%d" % (p, d)]), (p, d)


def test_apply_f32_bit_exact(oracle, golden):
    for (p, d) in _apply_cases(golden):
        k = "apply_out_f32_%d_%d" % (p, d)
        if k not in golden.files:
            continue
        x = golden["apply_in_%d_%d" % (p, d)].astype(np.float32)
        y = oracle.apply_f32(p, d, float(p * p), x, nthreads=2)
        assert np.array_equal(y, golden[k]), (p, d)


def test_volume_matches_stored_operator_path(oracle, golden):
    # volume_mvm<T,1> sums the same operator in another order: equal to rounding
    for (p, d) in _apply_cases(golden):
        k = "volume_mvm_out_%d_%d" % (p, d)
        if k not in golden.files:
            continue
        x = golden["apply_in_%d_%d" % (p, d)]
        y = oracle.volume(p, d, x)
        ref = golden[k]
        assert np.max(np.abs(y - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref))), (p, d)


def test_rhs_and_full_solve_bit_exact(oracle, golden):
    table = golden["solve_table"]
    for i, row in enumerate(table):
        sol, p, d, pen, tol = int(row[0]), int(row[1]), int(row[2]), float(row[3]), float(row[4])
        it_ref, l2_ref, h1_ref, mx_ref = row[5:9]
        b = oracle.rhs(p, d, pen, sol)
        assert np.array_equal(b, golden["solve_rhs_%d" % i]), i
        it, x, _ = oracle.cg(p, d, pen, b, tol)
        assert it == int(it_ref), (i, it, it_ref)
        assert np.array_equal(x, golden["solve_u_%d" % i]), i
        e = oracle.err_norms(p, d, sol, x)
        assert (e[0], e[1], e[2]) == (l2_ref, h1_ref, mx_ref), i


def test_poisson16_case(oracle, golden):
    # 16x16, p = 4, u = sin(2 pi x) sin(2 pi y), pen = p^2, CG to 1e-12 relative
    p, d, pen, tol, it_ref, l2, h1, mx = golden["poisson16_stats"]
    p, d = int(p), int(d)
    b = oracle.rhs(p, d, pen, 6)
    assert np.array_equal(b, golden["poisson16_rhs"])
    it, x, _ = oracle.cg(p, d, pen, b, 1e-12, rel=True)
    assert it == int(it_ref)
    assert np.array_equal(x, golden["poisson16_u"])
    e = oracle.err_norms(p, d, 6, x)
    assert (e[0], e[1], e[2]) == (l2, h1, mx)


def test_cg_threaded_same_iterations(oracle, golden):
    # the chunked (multi-thread) dot order changes rounding only
    i = 1
    row = golden["solve_table"][i]
    sol, p, d, pen, tol = int(row[0]), int(row[1]), int(row[2]), float(row[3]), float(row[4])
    b = oracle.rhs(p, d, pen, sol)
    it1, x1, _ = oracle.cg(p, d, pen, b, tol, nthreads=1)
    it4, x4, _ = oracle.cg(p, d, pen, b, tol, nthreads=4)
    assert abs(it1 - it4) <= 1
    assert np.max(np.abs(x1 - x4)) <= 1e-10 * np.max(np.abs(x1))


# Thesis_TEXT.pdf p.51, Table 4.10: SIPG errors for solution E with penalty
# 100 p^2 and an absolute CG tolerance of 1e-15; (p, 1/h): (H1, L2, Linf).
THESIS_T4_10 = {
    (2, 4): (100.257, 18.1742, 30.1482), (2, 8): (17.4574, 0.221405, 0.530548),
    (2, 16): (3.65441, 0.0117439, 0.0222896), (3, 4): (26.3858, 1.82256, 3.08348),
    (3, 8): (1.89155, 0.0204869, 0.0372516), (3, 16): (0.46087, 0.000446633, 0.000906137),
    (4, 4): (6.50855, 0.126711, 0.302995), (4, 8): (0.91651, 0.000576389, 0.00122825),
    (4, 16): (0.0447112, 1.78395e-05, 3.39006e-05), (5, 4): (3.47723, 0.0078239, 0.013923),
    (5, 8): (0.0344363, 0.00012172, 0.000221666), (6, 4): (0.382002, 0.00200687, 0.00443417),
    (6, 8): (0.0192741, 1.99282e-06, 3.75147e-06),
}


@pytest.mark.parametrize("key", sorted(THESIS_T4_10))
def test_thesis_table_4_10(oracle, key):
    p, d = key
    pen = 100.0 * p * p
    b = oracle.rhs(p, d, pen, 5)
    it, x, _ = oracle.cg(p, d, pen, b, 1e-15, nthreads=4)
    l2, h1, mx = oracle.err_norms(p, d, 5, x)
    H1, L2, LI = THESIS_T4_10[key]
    # the table prints six significant digits
    assert h1 == pytest.approx(H1, rel=1e-5)
    assert l2 == pytest.approx(L2, rel=1e-5)
    assert mx == pytest.approx(LI, rel=1e-5)


def test_convergence_rates_h(oracle):
    # measured rates of the reference: H1 ~ p, L2 ~ p+2 (nodal superconvergence)
    p, pen = 3, 9.0
    errs = []
    for d in (4, 8, 16):
        b = oracle.rhs(p, d, pen, 1)
        it, x, _ = oracle.cg(p, d, pen, b, 1e-14, nthreads=4)
        errs.append(oracle.err_norms(p, d, 1, x))
    r_h1 = np.log2(errs[1][1] / errs[2][1])
    r_l2 = np.log2(errs[1][0] / errs[2][0])
    assert r_h1 == pytest.approx(p, abs=0.25)
    assert r_l2 > p + 0.8


# ---- block-Jacobi preconditioner and preconditioned CG (USE_PRECONDITIONER) ----

@pytest.mark.parametrize("p", range(1, 9))
def test_prec_rows_match_reference(oracle, golden, p):
    # the reference's penalty parameter is an int: 37.9 acts as 37
    for k, pen in enumerate((float(p * p), 100.0 * p * p, 37.9)):
        assert np.array_equal(oracle.prec_rows(p, pen), golden["prec_rows_%d_%d" % (p, k)]), (p, k)


@pytest.mark.parametrize("p", [3, 8])
def test_prec_block_and_inverse_match_reference(oracle, golden, p):
    blk = oracle.prec_block(p, float(p * p))
    assert np.array_equal(blk, golden["prec_block_%d" % p])
    assert np.array_equal(oracle.invert(blk), golden["prec_inverse_%d" % p])
    # and it is an inverse
    nn = (p + 1) ** 2
    prod = blk.reshape(nn, nn) @ golden["prec_inverse_%d" % p].reshape(nn, nn)
    assert np.max(np.abs(prod - np.eye(nn))) < 1e-12


def test_pcg_matches_reference_solves(oracle, golden):
    for i, row in enumerate(golden["pcg_table"]):
        sol, p, d, pen, tol = int(row[0]), int(row[1]), int(row[2]), float(row[3]), float(row[4])
        b = oracle.rhs(p, d, pen, sol)
        assert np.array_equal(b, golden["pcg_rhs_%d" % i])
        it, x, _ = oracle.pcg(p, d, pen, b, tol)
        assert it == int(row[5]), (i, it, row[5])
        assert np.array_equal(x, golden["pcg_u_%d" % i]), i
        l2, h1, mx = oracle.err_norms(p, d, sol, x)
        assert (l2, h1, mx) == (row[6], row[7], row[8])


def test_pcg_reproduces_thesis_rows(oracle, golden):
    # solution E, penalty 100 p^2, tolerance 1e-15: the h-adaptivity driver's
    # preconditioned solves give the thesis's Table 4.10 errors
    seen = 0
    for row in golden["pcg_table"]:
        sol, p, d, pen, tol = int(row[0]), int(row[1]), int(row[2]), float(row[3]), float(row[4])
        if sol == 5 and pen == 100.0 * p * p and (p, d) in THESIS_T4_10:
            H1, L2, _ = THESIS_T4_10[(p, d)]
            assert row[7] == pytest.approx(H1, rel=1e-5) and row[6] == pytest.approx(L2, rel=1e-5)
            seen += 1
    assert seen >= 3
