"""The tile-shape autotuner (sipg_op_autotune / set_tile / get_tile): every
tile shape -- rows per tile, one or two threads per element for the pairs
apply, the per-node FP64 tile -- gives the same apply result bit for bit (each output is the same
operations in the same order whatever the tiling), the tuner keeps a shape
that launches, and operators created later for the same (degree, dim) start
with the tuned shape."""
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(2, 1), (4, 1), (8, 1), (2, 2), (4, 2)]
SHAPES3 = [(32, r, t) for r, t in SHAPES]


def pernode(p, shape=0):
    """The per-node FP64 tile of degree p: (elements per row, rows, (p+1)^2)."""
    return (4 if p <= 2 else 2) * (2 if shape else 1), 4 if p == 1 else 2, (p + 1) ** 2


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
    for kind, rows in (("f32", 4), ("pairs", 4), ("f64", 2)):
        with pytest.raises(sipg.SipgError):
            op.set_tile(kind, rows, 1, elements_per_row=8)
    # the per-node tile: FP64 only, its two compiled shapes only
    ex, ey, tpe = pernode(3)
    for kind in ("f32", "pairs"):
        with pytest.raises(sipg.SipgError):
            op.set_tile(kind, ey, tpe, elements_per_row=ex)
    for bad in ((ex, ey + 2), (3 * ex, ey), (32, 4)):
        with pytest.raises(sipg.SipgError):
            op.set_tile("f64", bad[1], tpe, elements_per_row=bad[0])
    op.close()


# every degree; meshes that fill no tile, fill tiles exactly, and leave ragged
# tiles in x and y (including a single element: four boundary faces); and
# meshes with more tiles than resident CTAs, where each CTA works through
# several tiles
PERNODE_CASES = [(1, 1), (1, 13), (2, 9), (2, 16), (3, 1), (3, 16), (4, 16), (4, 37), (5, 7), (6, 11), (7, 5),
                 (8, 3), (8, 20), (1, 1025), (4, 301), (8, 150)]


@pytest.mark.parametrize("p,d", PERNODE_CASES)
def test_pernode_tile_gives_identical_applies(sipg, torch, p, d):
    """The per-node FP64 tile computes each output with the operations of the
    element-per-thread kernel, in the same order: bit-identical applies."""
    op = sipg.Operator(d, p, float(p * p) + 0.25)
    if d <= sipg.PERNODE_DEFAULT_DIM:
        assert op.get_shape("f64") == pernode(p, 0 if d <= sipg.PERNODE_WIDE_DIM else 1)
    else:
        assert op.get_shape("f64") == (32, {1: 8, 2: 8, 3: 8, 4: 8, 5: 4, 6: 2, 7: 4, 8: 2}[p], 1)
    op.set_pernode(0)
    g = torch.Generator(device="cuda").manual_seed(100 + p)
    x = torch.rand(op.ndof, device="cuda", dtype=torch.float64, generator=g) * 2 - 1
    y0 = op.apply(x)
    op.set_pernode(1)
    assert op.get_shape("f64") == pernode(p, 1)
    y1 = op.apply(x)
    op.set_tile("f64", 4)
    assert op.get_shape("f64") == (32, 4, 1)
    y = op.apply(x)
    assert torch.equal(y0, y) and torch.equal(y1, y)
    op.close()


@pytest.mark.parametrize("p,d", [(4, 16), (2, 23), (7, 9), (4, 128)])
def test_pernode_cg_matches_element_tile_cg(sipg, torch, p, d):
    """CG with the per-node tile (direction fused into the apply: two kernels
    an iteration) against CG with the element tile (three kernels): the same
    iterates up to the grouping of the dot-product sums."""
    op = sipg.Operator(d, p, float(p * p))
    b = op.rhs("sinsin")
    xs, its = [], []
    for shape in ("pernode", "element"):
        if shape == "element":
            op.set_tile("f64", 4)
        else:
            op.set_pernode(0)
        x = torch.zeros_like(b)
        st, res = op.cg(x, b, 1e-12, relative=True)
        assert st == 0 and res.converged == 1
        xs.append(x)
        its.append(res.iterations)
    assert abs(its[0] - its[1]) <= 1
    assert (xs[0] - xs[1]).abs().max().item() <= 1e-9 * xs[1].abs().max().item()
    op.close()


def test_autotune_picks_a_launchable_shape_and_is_remembered(sipg, torch):
    p, d = 6, 96
    op = sipg.Operator(d, p, 36.0)
    choice = op.autotune()
    for kind, (tx, rows, tpe, ms) in choice.items():
        allowed = SHAPES3 + ([pernode(p, 0), pernode(p, 1)] if kind == "f64" else [])
        assert (tx, rows, tpe) in allowed and ms > 0, (kind, tx, rows, tpe, ms)
        assert tpe == 1 or kind == "pairs" or (kind == "f64" and tpe == (p + 1) ** 2)
        assert tx == 32 or kind == "f64"
        assert op.get_shape(kind) == (tx, rows, tpe)
    # a later operator of the same degree and size starts from the tuned shapes
    op2 = sipg.Operator(d, p, 36.0)
    for kind, (tx, rows, tpe, _) in choice.items():
        assert op2.get_shape(kind) == (tx, rows, tpe)
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
