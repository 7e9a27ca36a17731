"""The fused CUDA apply and CG against the reference's own CUDA kernels on the
same GPU (oracle/_ref/ref_kernels.cubin, the reference headers compiled
unchanged for sm_103a; built where the reference checkout exists).

Matvec: within 1e-12 relative (max |y - y_ref| / max |y_ref|) on the same mesh,
degree and input vectors, up to the full 1024 x 1024, p = 4 size.  CG:
iteration counts within +-1 of the reference's CG (cuBLAS dots)."""
import numpy as np
import pytest

import oracle_lib

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not oracle_lib.ref_gpu_available(),
                                 reason="reference cubin not built (needs the reference checkout)")]


@pytest.fixture(scope="module")
def torch():
    import torch as t

    return t


def rel(a, b):
    return float((a - b).abs().max().item() / b.abs().max().item())


@pytest.mark.parametrize("p", range(1, 9))
def test_apply_matches_reference_kernels(sipg, torch, p):
    ref = oracle_lib.ref_gpu()
    for d in (5, 64, 129):
        op = sipg.Operator(d, p, float(p * p))
        g = torch.Generator(device="cuda").manual_seed(100 * p + d)
        x = torch.rand(op.ndof, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        y_ref = torch.empty_like(x)
        ref.apply(p, d, float(p * p), x.data_ptr(), y_ref.data_ptr())
        torch.cuda.synchronize()
        y = op.apply(x)
        assert rel(y, y_ref) <= 1e-12, (p, d, rel(y, y_ref))
        op.close()


def test_apply_full_size_matches_reference_kernels(sipg, torch):
    p, d, pen = 4, 1024, 16.0
    ref = oracle_lib.ref_gpu()
    x_np = np.random.default_rng(0).uniform(-1.0, 1.0, d * d * (p + 1) ** 2)
    x = torch.from_numpy(x_np).cuda()
    y_ref = torch.empty_like(x)
    ref.apply(p, d, pen, x.data_ptr(), y_ref.data_ptr())
    torch.cuda.synchronize()
    op = sipg.Operator(d, p, pen)
    y = op.apply(x)
    assert rel(y, y_ref) <= 1e-12
    op.close()


@pytest.mark.parametrize("p", range(1, 9))
def test_apply_sweep_sizes_match_reference_kernels(sipg, torch, p):
    # the constant ~16 M DoF sweep: dim = round(4000 / (p + 1)) (2000^2 at p = 1
    # ... 444^2 at p = 8), input U[-1,1] from seed 0 as the throughput bench
    # uses, each degree's default tile shape (and the p = 8 shared-memory
    # coefficient path) against the reference's kernels on the same vector
    d = round(4000 / (p + 1))
    pen = float(p * p)
    ref = oracle_lib.ref_gpu()
    op = sipg.Operator(d, p, pen)
    x = torch.from_numpy(np.random.default_rng(0).uniform(-1.0, 1.0, op.ndof)).cuda()
    y_ref = torch.empty_like(x)
    ref.apply(p, d, pen, x.data_ptr(), y_ref.data_ptr())
    torch.cuda.synchronize()
    y = op.apply(x)
    assert rel(y, y_ref) <= 1e-12, (p, d, rel(y, y_ref))
    op.close()


@pytest.mark.parametrize("p,d,pen,sol", [(4, 16, 16.0, "sinsin"), (2, 64, 4.0, "E"), (6, 32, 3600.0, "E")])
def test_cg_iterations_match_reference_cg(sipg, torch, p, d, pen, sol):
    ref = oracle_lib.ref_gpu()
    op = sipg.Operator(d, p, pen)
    b = op.rhs(sol)
    tol = 1e-12 * b.norm().item()
    x_ref = torch.zeros_like(b)
    it_ref, _ = ref.cg(p, d, pen, x_ref.data_ptr(), b.data_ptr(), tol)
    x = torch.zeros_like(b)
    st, res = op.cg(x, b, tol)
    assert st == 0
    assert abs(res.iterations - it_ref) <= 1, (res.iterations, it_ref)
    assert rel(x, x_ref) <= 1e-9
    op.close()
