"""The fused CUDA apply against the reference's outputs and the oracle.

Tolerance: FP64 results agree with the reference's matvec to 1e-12 relative
(max |y - y_ref| / max |y_ref|); the FP32 operator agrees with the FP64
reference to 2e-6 relative (a few FP32 ulps of the largest entry).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12
RTOL32 = 2e-6


def rel_err(y, ref):
    return float(np.max(np.abs(y - ref)) / max(np.max(np.abs(ref)), 1e-300))


def _cases(golden):
    return sorted({tuple(int(v) for v in k.split("_")[2:4]) for k in golden.files if k.startswith("apply_in_")})


@pytest.fixture(scope="module")
def torch():
    import torch as t

    assert t.cuda.is_available()
    return t


def test_apply_f64_matches_reference_golden(sipg, golden, torch):
    for (p, d) in _cases(golden):
        x = golden["apply_in_%d_%d" % (p, d)]
        xt = torch.from_numpy(x).cuda()
        for name, pen in (("ref", float(p * p)), ("thesis", 100.0 * p * p)):
            k = "apply_out_%s_%d_%d" % (name, p, d)
            if k not in golden.files:
                continue
            op = sipg.Operator(d, p, pen)
            y = op.apply(xt).cpu().numpy()
            op.close()
            assert rel_err(y, golden[k]) <= RTOL64, (p, d, name, rel_err(y, golden[k]))


def test_apply_f32_matches_reference_golden(sipg, golden, torch):
    for (p, d) in _cases(golden):
        k = "apply_out_ref_%d_%d" % (p, d)
        x = golden["apply_in_%d_%d" % (p, d)]
        op = sipg.Operator(d, p, float(p * p))
        y = op.apply(torch.from_numpy(x.astype(np.float32)).cuda()).cpu().numpy().astype(np.float64)
        op.close()
        assert rel_err(y, golden[k]) <= RTOL32, (p, d, rel_err(y, golden[k]))


@pytest.mark.parametrize("p", range(1, 9))
def test_apply_f64_vs_oracle_multi_tile(sipg, oracle, torch, p):
    # sizes that are not multiples of the 32 x TY tile, several CTAs in both directions
    rng = np.random.default_rng(7 + p)
    for d in (37, 70):
        x = rng.uniform(-1, 1, d * d * (p + 1) ** 2)
        pen = float(p * p)
        op = sipg.Operator(d, p, pen)
        y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        op.close()
        ref = oracle.apply(p, d, pen, x)
        assert rel_err(y, ref) <= RTOL64, (p, d, rel_err(y, ref))


@pytest.mark.parametrize("p", range(1, 9))
def test_apply_f32_vs_oracle_multi_tile(sipg, oracle, torch, p):
    # the FP32 apply over several 32-element tiles in x and y, sizes that are
    # not tile multiples: its register-resident nodal blocks (p <= 6), halo
    # reads and face ownership across tile edges, against the FP64 oracle on
    # the same (FP32-representable) input
    rng = np.random.default_rng(17 + p)
    for d in (37, 70):
        x = rng.uniform(-1, 1, d * d * (p + 1) ** 2).astype(np.float32)
        pen = float(p * p)
        op = sipg.Operator(d, p, pen)
        y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy().astype(np.float64)
        op.close()
        ref = oracle.apply(p, d, pen, x.astype(np.float64))
        assert rel_err(y, ref) <= RTOL32, (p, d, rel_err(y, ref))


@pytest.mark.parametrize("p", [4, 6])
def test_apply_f32_full_size_vs_oracle(sipg, oracle, torch, p):
    # full size: 1024 x 1024 (p = 4, 26.2 M DoF) and 571 x 571 (p = 6, the
    # ~16 M DoF sweep size), input U[-1,1] seed 0 rounded to FP32
    d = 1024 if p == 4 else 571
    pen = float(p * p)
    x = np.random.default_rng(0).uniform(-1.0, 1.0, d * d * (p + 1) ** 2).astype(np.float32)
    op = sipg.Operator(d, p, pen)
    y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy().astype(np.float64)
    op.close()
    ref = oracle.apply(p, d, pen, x.astype(np.float64), nthreads=8)
    assert rel_err(y, ref) <= RTOL32, rel_err(y, ref)


def test_apply_full_size_vs_oracle(sipg, oracle, torch):
    # the 1024 x 1024, p = 4 throughput case (26.2 M DoF), input U[-1,1] seed 0
    p, d, pen = 4, 1024, 16.0
    x = np.random.default_rng(0).uniform(-1.0, 1.0, d * d * (p + 1) ** 2)
    op = sipg.Operator(d, p, pen)
    y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    op.close()
    ref = oracle.apply(p, d, pen, x)
    assert rel_err(y, ref) <= RTOL64


def test_apply_properties_full_size(sipg, torch):
    # symmetry <Ax, z> = <x, Az> and linearity, on 1024^2 p=4 without a CPU reference
    p, d = 4, 1024
    op = sipg.Operator(d, p, 16.0)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(op.ndof, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    z = torch.rand(op.ndof, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    Ax, Az = op.apply(x), op.apply(z)
    lhs, rhs = torch.dot(Ax, z).item(), torch.dot(x, Az).item()
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + abs(rhs))
    Alin = op.apply(2.5 * x - 0.75 * z)
    assert (Alin - (2.5 * Ax - 0.75 * Az)).abs().max().item() <= 1e-11 * Ax.abs().max().item()
    # positive definite on random vectors for pen = p^2
    assert torch.dot(Ax, x).item() > 0
    op.close()


def test_apply_host_buffers(sipg, oracle):
    p, d = 3, 40
    x = np.random.default_rng(11).uniform(-1, 1, d * d * (p + 1) ** 2)
    op = sipg.Operator(d, p, 9.0)
    y = op.apply_host(x)
    op.close()
    assert rel_err(y, oracle.apply(p, d, 9.0, x)) <= RTOL64


@pytest.mark.parametrize("p,d,tile", [(4, 300, None), (1, 1030, None), (6, 389, 2), (3, 260, "pernode"),
                                      (2, 515, 8), (8, 129, None)])
def test_apply_host_buffers_banded_equals_device_apply(sipg, torch, p, d, tile):
    """The host-buffer apply runs in bands of element rows (copy-in, apply and
    copy-out overlapped); every band reads its halo rows from the next band's
    copy.  Its result equals the device apply's bit for bit, with the element
    tiles and the per-node tile, including ragged last bands."""
    op = sipg.Operator(d, p, float(p * p) + 0.5)
    if tile == "pernode":
        op.set_pernode(1)
    elif tile is not None:
        op.set_tile("f64", tile)
    x = np.random.default_rng(d).uniform(-1, 1, op.ndof)
    xp = torch.from_numpy(x).pin_memory()
    yp = torch.empty_like(xp).pin_memory()
    y_host = op.apply_host(xp.numpy(), out=yp.numpy())
    y_dev = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.array_equal(y_host, y_dev)
    y_again = op.apply_host(x)  # pageable buffers: the same result
    assert np.array_equal(y_again, y_dev)
    op.close()


def test_apply_on_side_stream_and_counts_launches(sipg, torch):
    p, d = 2, 64
    op = sipg.Operator(d, p, 4.0)
    x = torch.rand(op.ndof, dtype=torch.float64, device="cuda")
    ref = op.apply(x)
    s = torch.cuda.Stream()
    n0 = sipg.launch_count()
    with torch.cuda.stream(s):
        y = op.apply(x)
    s.synchronize()
    assert sipg.launch_count() - n0 == 1
    assert torch.equal(y, ref)  # deterministic
    op.close()


def test_invalid_degree_raises(sipg):
    with pytest.raises(sipg.SipgError):
        sipg.Operator(8, 9, 1.0)


def _rel_l2(y, ref):
    return float(((y - ref).norm() / ref.norm()).item())


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 7, 8])
def test_apply_pairs_matches_f64_random(sipg, torch, p):
    # double-float pair vectors, compensated arithmetic: the FP64 apply of the
    # same value (hi + lo, exact in FP64) to the FP64 parity bar, 1e-12
    d = 37
    g = torch.Generator(device="cuda").manual_seed(p)
    op = sipg.Operator(d, p, 100.0 * p * p + 0.3)  # a penalty with a non-zero FP32 remainder
    xp = sipg.to_pairs(torch.rand(op.ndof, device="cuda", generator=g, dtype=torch.float64) * 2 - 1)
    y64 = op.apply(sipg.from_pairs(xp))
    y = sipg.from_pairs(op.apply_pairs(xp))
    assert (y - y64).abs().max().item() <= 1e-12 * y64.abs().max().item(), p
    op.close()


def test_apply_pairs_on_smooth_vector(sipg, torch):
    # A x for the discrete solution x of a fine mesh is b: the terms cancel to
    # about 1 part in the condition number (~1e6 here).  The FP32 apply of the
    # rounded vector loses that many of its 24 bits; pairs keep ~48.
    d, p = 128, 6
    op = sipg.Operator(d, p, float(p * p))
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, _ = op.cg(x, b, 1e-12, relative=True)
    assert st == 0
    e_pairs = _rel_l2(sipg.from_pairs(op.apply_pairs(sipg.to_pairs(x))), op.apply(x))
    e_32 = _rel_l2(op.apply(x.float()).double(), op.apply(x))
    assert e_pairs <= 3e-8, e_pairs
    assert e_32 >= 1000 * e_pairs, (e_32, e_pairs)
    op.close()
