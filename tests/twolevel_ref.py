"""CPU restatement (numpy, FP64) of the two-level preconditioner of the
flexible mixed-precision solve, the checker of sipg_apply_twolevel_f32 (test
infrastructure; the preconditioner has no counterpart in the reference).

M r = B^-1 r + P V(P^T r):
- B^-1: the inverse of every element's diagonal block, probed from the
  operator (the oracle's matvec) on a mesh of min(dim, 3) elements per side
  with a checkerboard colouring; blocks are keyed by which faces lie on the
  domain boundary (bit 0 LEFT, 1 RIGHT, 2 DOWN, 3 UP; row 0 is the top row).
  It is formed from the block's generalised eigenvectors (B V = W V mu, W the
  nodal quadrature weights), leaving out null modes, |mu| <= 1e-12 max |mu|.
- P: bilinear hat functions of the (dim + 1)^2 vertices (bottom-up vertex rows)
  at each element's LGL nodes (node (i1, i2): i1 along x, i2 along y).
- V: one V-cycle for A_0 = P^T A P (probed with nine vertex colours),
  Galerkin levels P_l^T A_l P_l (m cells -> ceil(m / 2): coarse vertices at the
  even fine vertices and at m) down to at most 8 cells, two damped-Jacobi
  sweeps from zero before and two after each coarse correction with omega =
  1.6 / (1.05 lambda_max(D^-1 A)) from 40 power iterations started at
  sin(0.7 v + 0.3) + 0.5, the coarsest level by its dense inverse.
"""
import numpy as np
import scipy.linalg
import scipy.sparse as sp

COARSEST = 8
NULL_REL = 1e-12


def elem_type(row, col, dim):
    return (col == 0) * 1 | (col == dim - 1) * 2 | (row == dim - 1) * 4 | (row == 0) * 8


def blocks(orc, p, pen, dim):
    n1 = p + 1
    nn = n1 * n1
    dm = min(dim, 3)
    noe = dm * dm
    out = {}
    for color in (0, 1):
        for k in range(nn):
            x = np.zeros(nn * noe)
            for e in range(noe):
                if (e // dm + e % dm) % 2 == color:
                    x[k * noe + e] = 1.0
            y = orc.apply(p, dm, pen, x, nthreads=1).reshape(nn, noe)
            for e in range(noe):
                if (e // dm + e % dm) % 2 != color:
                    continue
                t = elem_type(e // dm, e % dm, dm)
                out.setdefault(t, np.zeros((nn, nn)))[:, k] = y[:, e]
    xi, w = orc.lgl(n1)
    W = np.kron(np.diag(w), np.diag(w))
    return {t: block_inverse(b, W) for t, b in out.items()}


def block_inverse(B, W):
    """V diag(1/mu) V^T from B V = W V diag(mu), V^T W V = I: the inverse of
    B, with the modes of |mu| <= 1e-12 max |mu| left out (a singular block)."""
    mu, V = scipy.linalg.eigh(B, W)
    keep = np.abs(mu) > NULL_REL * np.abs(mu).max()
    inv = np.zeros_like(mu)
    inv[keep] = 1.0 / mu[keep]
    return (V * inv) @ V.T


def prolongation(orc, p, dim):
    n1 = p + 1
    noe = dim * dim
    xi, _ = orc.lgl(n1)
    hat = [(1 - xi) / 2, (1 + xi) / 2]
    rows, cols, vals = [], [], []
    for e in range(noe):
        row, col = divmod(e, dim)
        R = dim - 1 - row
        for a in (0, 1):
            for b in (0, 1):
                v = (R + b) * (dim + 1) + col + a
                for i1 in range(n1):
                    for i2 in range(n1):
                        rows.append((i1 * n1 + i2) * noe + e)
                        cols.append(v)
                        vals.append(hat[a][i1] * hat[b][i2])
    return sp.csr_matrix((vals, (rows, cols)), shape=(n1 * n1 * noe, (dim + 1) ** 2))


def level0(orc, p, dim, pen, P):
    n1v = dim + 1
    nv = n1v * n1v
    vx, vy = np.arange(nv) % n1v, np.arange(nv) // n1v
    A = sp.lil_matrix((nv, nv))
    for cy in range(3):
        for cx in range(3):
            ind = ((vx % 3 == cx) & (vy % 3 == cy)).astype(float)
            y = P.T @ orc.apply(p, dim, pen, P @ ind, nthreads=4)
            for v in range(nv):
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        ux, uy = vx[v] + dx, vy[v] + dy
                        if 0 <= ux <= dim and 0 <= uy <= dim and ux % 3 == cx and uy % 3 == cy:
                            A[v, uy * n1v + ux] = y[v]
    return A.tocsr()


def interp1d(m):
    mc = (m + 1) // 2
    R, C, V = [], [], []
    for i in range(m + 1):
        if i % 2 == 0 or i == m:
            R.append(i)
            C.append((i + 1) // 2)
            V.append(1.0)
        else:
            R += [i, i]
            C += [(i - 1) // 2, (i + 1) // 2]
            V += [0.5, 0.5]
    return sp.csr_matrix((V, (R, C)), shape=(m + 1, mc + 1)), mc


def omega(A):
    D = A.diagonal()
    x = np.sin(0.7 * np.arange(A.shape[0]) + 0.3) + 0.5
    lam = 1.0
    for _ in range(40):
        y = (A @ x) / D
        lam = np.linalg.norm(y) / np.linalg.norm(x)
        x = y / np.linalg.norm(y)
    return 1.6 / (1.05 * lam)


def hierarchy(A0, m):
    levels = []
    A = A0
    while True:
        lv = {"A": A, "m": m, "D": A.diagonal()}
        levels.append(lv)
        if m <= COARSEST:
            lv["inv"] = np.linalg.inv(A.toarray())
            return levels
        lv["w"] = omega(A)
        P1, mc = interp1d(m)
        lv["P"] = sp.kron(P1, P1).tocsr()
        A = (lv["P"].T @ A @ lv["P"]).tocsr()
        m = mc


def vcycle(levels, l, b):
    L = levels[l]
    if "inv" in L:
        return L["inv"] @ b
    A, wd = L["A"], L["w"] / L["D"]
    x1 = wd * b
    x = x1 + wd * (b - A @ x1)
    x = x + L["P"] @ vcycle(levels, l + 1, L["P"].T @ (b - A @ x))
    y = x + wd * (b - A @ x)
    return y + wd * (b - A @ y)


class TwoLevel:
    def __init__(self, orc, p, dim, pen):
        self.p, self.dim = p, dim
        self.binv = blocks(orc, p, pen, dim)
        self.P = prolongation(orc, p, dim)
        self.levels = hierarchy(level0(orc, p, dim, pen, self.P), dim)

    def apply(self, r):
        p, dim = self.p, self.dim
        nn, noe = (p + 1) ** 2, dim * dim
        R = np.asarray(r, dtype=np.float64).reshape(nn, noe)
        Z = np.empty_like(R)
        types = np.array([elem_type(e // dim, e % dim, dim) for e in range(noe)])
        for t, B in self.binv.items():
            mask = types == t
            Z[:, mask] = B @ R[:, mask]
        return Z.reshape(-1) + self.P @ vcycle(self.levels, 0, self.P.T @ R.reshape(-1))
