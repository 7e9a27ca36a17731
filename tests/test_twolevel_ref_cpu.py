"""The CPU restatement of the two-level preconditioner (tests/twolevel_ref.py)
on its own, without a GPU: preconditioned CG with it needs a number of
iterations that does not grow with the mesh (the property the FP32 inner solve
of the flexible mixed solve relies on), far fewer than plain CG."""
import numpy as np

import twolevel_ref


def _pcg(orc, p, dim, pen, b, M, tol=1e-10):
    x = np.zeros_like(b)
    r = b.copy()
    z = M(r)
    pv = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    for it in range(1, 5000):
        Ap = orc.apply(p, dim, pen, pv, nthreads=4)
        a = rz / (pv @ Ap)
        x += a * pv
        r -= a * Ap
        if np.linalg.norm(r) <= tol * bn:
            return it
        z = M(r)
        rz2 = r @ z
        pv = z + rz2 / rz * pv
        rz = rz2
    return 5000


def test_twolevel_pcg_iterations_flat_in_the_mesh(oracle):
    p, pen = 4, 16.0
    counts = {}
    for dim in (8, 24):
        b = oracle.rhs(p, dim, pen, 6)
        counts[dim] = _pcg(oracle, p, dim, pen, b, twolevel_ref.TwoLevel(oracle, p, dim, pen).apply)
    plain = _pcg(oracle, p, 24, pen, oracle.rhs(p, 24, pen, 6), lambda r: r.copy())
    assert abs(counts[24] - counts[8]) <= 0.15 * counts[8], counts
    assert counts[24] <= 0.35 * plain, (counts, plain)


def test_twolevel_coarsening_of_odd_levels():
    # m cells -> ceil(m/2): coarse vertices at the even fine vertices and at m
    for m in (9, 16, 17, 33):
        P, mc = twolevel_ref.interp1d(m)
        assert mc == (m + 1) // 2 and P.shape == (m + 1, mc + 1)
        xs_f = np.arange(m + 1, dtype=float)
        xs_c = np.array([min(2 * J, m) for J in range(mc + 1)], dtype=float)
        assert np.allclose(P @ xs_c, xs_f)  # linear functions are reproduced
        assert np.allclose(P.sum(axis=1), 1.0)


def _stamp_class(v, m, ms=6):
    if v <= 2:
        return v
    if v >= m - 2:
        return ms - (m - v)
    return ms // 2


def test_vertex_operator_rows_repeat_past_the_boundary(oracle):
    """The set-up copies a large mesh's level-0 vertex operator P^T A P from a
    6 x 6 mesh's (the two vertices at each end of an axis keep their rows,
    every other vertex takes the middle one): the bilinear vertex functions
    are continuous, so only boundary vertices see the Nitsche terms and the
    element and face terms do not depend on the element size.  The probed
    operators agree exactly."""
    for p in (1, 2, 4, 6):
        pen = float(p * p)
        small = twolevel_ref.level0(oracle, p, 6, pen, twolevel_ref.prolongation(oracle, p, 6)).toarray()
        for dim in (7, 11):
            A = twolevel_ref.level0(oracle, p, dim, pen, twolevel_ref.prolongation(oracle, p, dim)).toarray()
            n1 = dim + 1
            for vy in range(n1):
                for vx in range(n1):
                    cy, cx = _stamp_class(vy, dim), _stamp_class(vx, dim)
                    for dy in (-1, 0, 1):
                        for dx in (-1, 0, 1):
                            ux, uy = vx + dx, vy + dy
                            if not (0 <= ux <= dim and 0 <= uy <= dim):
                                continue
                            got = A[vy * n1 + vx, uy * n1 + ux]
                            want = small[cy * 7 + cx, (cy + dy) * 7 + cx + dx]
                            assert got == want, (p, dim, vx, vy, dx, dy, got, want)
