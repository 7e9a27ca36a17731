"""The tile-shape autotuner (sipg_op_autotune / set_tile / get_tile): every
tile shape gives the same apply result bit for bit (each output is the same
operations in the same order whatever the tiling), the tuner keeps a shape
that launches, and operators created later for the same (degree, dim) start
with the tuned shape."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t

    return t


@pytest.mark.parametrize("p,d", [(2, 45), (5, 37), (8, 21)])
def test_every_tile_shape_gives_identical_applies(sipg, torch, p, d):
    op = sipg.Operator(d, p, float(p * p) + 0.25)
    g = torch.Generator(device="cuda").manual_seed(p)
    x64 = torch.rand(op.ndof, device="cuda", dtype=torch.float64, generator=g) * 2 - 1
    x32 = x64.float()
    xp = sipg.to_pairs(x64)
    outs = {}

    def run(f, *args):
        try:
            return f(*args)
        except sipg.SipgError:
            # p = 8 with 8 rows needs more than 227 KB of shared memory (FP64
            # and pair vectors): refused at launch, never run
            assert p == 8 and rows == 8
            return None

    for rows in (2, 4, 8):
        for kind in ("f64", "f32", "pairs"):
            op.set_tile(kind, rows)
            assert op.get_tile(kind) == rows
        outs[rows] = (run(op.apply, x64), run(op.apply, x32), run(op.apply_pairs, xp))
    for rows in (4, 8):
        for k in range(3):
            a, b = outs[2][k], outs[rows][k]
            if a is not None and b is not None:
                assert torch.equal(a, b), (rows, k)
    op.close()


def test_autotune_picks_a_launchable_shape_and_is_remembered(sipg, torch):
    p, d = 6, 96
    op = sipg.Operator(d, p, 36.0)
    choice = op.autotune()
    for kind, (rows, ms) in choice.items():
        assert rows in (2, 4, 8) and ms > 0, (kind, rows, ms)
        assert op.get_tile(kind) == rows
    # a later operator of the same degree and size starts from the tuned shapes
    op2 = sipg.Operator(d, p, 36.0)
    for kind, (rows, _) in choice.items():
        assert op2.get_tile(kind) == rows
    # and a CG solve after re-tuning re-captures its graphs and still converges
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-10, relative=True)
    assert st == 0 and res.converged == 1
    op.set_tile("f64", 2 if op.get_tile("f64") != 2 else 4)
    x2 = torch.zeros_like(b)
    st, res2 = op.cg(x2, b, 1e-10, relative=True)
    assert st == 0 and abs(res2.iterations - res.iterations) <= 1
    assert (x2 - x).abs().max().item() <= 1e-8 * x.abs().max().item()
    op.close()
    op2.close()
