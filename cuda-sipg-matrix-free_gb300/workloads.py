"""Seeded synthetic workloads of the solver's benchmark configurations.

Every generator is deterministic in its seed (numpy PCG64) so that two runs,
or the library and a comparison against the plain FP64 solver, see the same
problems.  A right-hand side of the "modes" kind is
f = sum_k A_k sin(k_k pi x) sin(l_k pi y) (up to 8 terms, sipg_modes).
"""
import math

import numpy as np

DEGREES = tuple(range(2, 9))


def random_modes(rng, nmodes=4, kmax=8):
    """nmodes terms with A ~ N(0, 1) and k, l uniform in {1..kmax}."""
    amps = rng.normal(size=nmodes)
    ks = rng.integers(1, kmax + 1, nmodes)
    ls = rng.integers(1, kmax + 1, nmodes)
    return [float(a) for a in amps], [int(k) for k in ks], [int(l) for l in ls]


def log_uniform_int(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def shared_mesh_rhs(count=64, dim=256, degree=4, seed=1):
    """Many right-hand sides on one mesh: [(dim, degree, pen, modes)]."""
    rng = np.random.default_rng(seed)
    pen = float(degree * degree)
    return [(dim, degree, pen, random_modes(rng)) for _ in range(count)]


def uneven_problems(count=200, dim_lo=16, dim_hi=256, seed=2):
    """Independent problems: dim log-uniform in [dim_lo, dim_hi], p uniform in 2..8."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        dim = log_uniform_int(rng, dim_lo, dim_hi)
        p = int(rng.choice(DEGREES))
        out.append((dim, p, float(p * p), random_modes(rng)))
    return out


def request_stream(count=10000, rate=200.0, dim_lo=8, dim_hi=512, tols=(1e-8, 1e-10), seed=3):
    """Solve requests with Poisson arrivals at `rate` per second:
    [(t_arrival_s, dim, degree, pen, modes, tol)]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        dim = log_uniform_int(rng, dim_lo, dim_hi)
        p = int(rng.choice(DEGREES))
        tol = float(tols[int(rng.integers(0, len(tols)))])
        out.append((t, dim, p, float(p * p), random_modes(rng), tol))
    return out


def ndof(dim, degree):
    return dim * dim * (degree + 1) ** 2
