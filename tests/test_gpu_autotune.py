"""The tile-shape autotuner (sipg_op_autotune / set_tile / get_tile): every
tile shape -- rows per tile, and one or two threads per element for the pairs
apply -- gives the same apply result bit for bit (each output is the same
operations in the same order whatever the tiling), the tuner keeps a shape
that launches, and operators created later for the same (degree, dim) start
with the tuned shape."""
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(2, 1), (4, 1), (8, 1), (2, 2), (4, 2)]


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

    for rows, tpe in SHAPES:
        kinds = ("pairs",) if tpe == 2 else ("f64", "f32", "pairs")
        for kind in kinds:
            op.set_tile(kind, rows, tpe)
            assert op.get_tile(kind) == (rows, tpe)
        if tpe == 2:
            outs[(rows, tpe)] = (None, None, run(op.apply_pairs, xp))
        else:
            outs[(rows, tpe)] = (run(op.apply, x64), run(op.apply, x32), run(op.apply_pairs, xp))
    base = outs[(2, 1)]
    for shape in SHAPES[1:]:
        for k in range(3):
            a, b = base[k], outs[shape][k]
            if a is not None and b is not None:
                assert torch.equal(a, b), (shape, k)
    op.close()


def test_two_threads_per_element_rejected_where_not_compiled(sipg):
    op = sipg.Operator(8, 3, 9.0)
    for kind, rows in (("f64", 4), ("f32", 4), ("pairs", 8)):
        with pytest.raises(sipg.SipgError):
            op.set_tile(kind, rows, 2)
    op.close()


def test_autotune_picks_a_launchable_shape_and_is_remembered(sipg, torch):
    p, d = 6, 96
    op = sipg.Operator(d, p, 36.0)
    choice = op.autotune()
    for kind, (rows, tpe, ms) in choice.items():
        assert (rows, tpe) in SHAPES and ms > 0, (kind, rows, tpe, ms)
        assert tpe == 1 or kind == "pairs"
        assert op.get_tile(kind) == (rows, tpe)
    # a later operator of the same degree and size starts from the tuned shapes
    op2 = sipg.Operator(d, p, 36.0)
    for kind, (rows, tpe, _) in choice.items():
        assert op2.get_tile(kind) == (rows, tpe)
    # and a CG solve after re-tuning re-captures its graphs and still converges
    b = op.rhs("sinsin")
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, 1e-10, relative=True)
    assert st == 0 and res.converged == 1
    op.set_tile("f64", 2 if op.get_tile("f64")[0] != 2 else 4)
    x2 = torch.zeros_like(b)
    st, res2 = op.cg(x2, b, 1e-10, relative=True)
    assert st == 0 and abs(res2.iterations - res.iterations) <= 1
    assert (x2 - x).abs().max().item() <= 1e-8 * x.abs().max().item()
    # the pairs mixed solve with two threads per element
    op.set_tile("pairs", 4, 2)
    xm = torch.zeros_like(b)
    st, rm = op.solve_mixed(xm, b, inner="pairs")
    assert st == 0 and rm.rel_residual <= 1e-10
    op.close()
    op2.close()
