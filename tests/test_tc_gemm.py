"""The sm_103a tensor-core GEMM (cpg_gemm_f32_tc) against an FP64 torch GEMM.

Each operand row is scaled by a power of two and split into FP16 hi and lo; the kernel sums
Ah Bh + Ah Bl + Al Bh in FP32.  Per product that leaves a relative error of a few 2^-22, so the
bound checked is elementwise:

    |C - C64| <= 4e-6 (|A| |B|)_ij + 1e-30

(|A| |B| the product of the magnitudes), which an FP32 GEMM of inner dimension k would also
meet only up to its own k 2^-24 accumulation bound.  Shapes are odd on purpose: partial 128-row
and 256-column tiles, k not a multiple of 64, a single column.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(cg, A, B, Cm=None, alpha=1.0, beta=0.0, sm_budget=0):
    import torch
    m, k = A.shape
    n = B.shape[1]
    dA = A.t().contiguous()  # column-major storage: the transpose, row-major
    dB = B.t().contiguous()
    dC = (Cm.t().contiguous() if Cm is not None else torch.zeros((n, m), dtype=torch.float32, device="cuda"))
    ctx = cg.Context.default()
    torch.cuda.synchronize()
    rc = ctx.L.cpg_gemm_f32_tc(ctx.h, m, n, k, C.c_float(alpha), C.c_void_p(dA.data_ptr()), m,
                               C.c_void_p(dB.data_ptr()), k, C.c_float(beta), C.c_void_p(dC.data_ptr()), m, sm_budget)
    ctx.check(rc, "tensor-core gemm")
    return dC.t()


def _check(A, B, Cm, got, alpha, beta, tol=4e-6):
    A64, B64 = A.double(), B.double()
    ref = alpha * (A64 @ B64) + (beta * Cm.double() if beta != 0 else 0)
    bound = tol * abs(alpha) * (A64.abs() @ B64.abs()) + 1e-30
    if beta != 0:
        bound = bound + 1e-7 * abs(beta) * Cm.double().abs()
    err = (got.double() - ref).abs()
    worst = float((err / bound).max())
    assert worst <= 1.0, "error %.3g of the bound" % worst


@pytest.mark.parametrize("m,n,k", [(300, 520, 200), (1000, 257, 1024), (129, 1, 64), (128, 256, 64),
                                   (2050, 3000, 1024), (77, 700, 5)])
def test_gemm_matches_fp64(built, m, n, k):
    import torch
    import cpanel_gb300 as cg
    g = torch.Generator(device="cuda").manual_seed(m * 7919 + n * 31 + k)
    A = torch.randn((m, k), generator=g, device="cuda", dtype=torch.float32)
    B = torch.randn((k, n), generator=g, device="cuda", dtype=torch.float32)
    got = _gemm(cg, A, B)
    _check(A, B, None, got, 1.0, 0.0)


@pytest.mark.parametrize("alpha,beta", [(-1.0, 1.0), (0.5, -2.0)])
def test_gemm_accumulates_into_c(built, alpha, beta):
    """C = alpha A B + beta C, as the factorization's trailing update uses it (alpha -1, beta 1)."""
    import torch
    import cpanel_gb300 as cg
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn((700, 384), generator=g, device="cuda")
    B = torch.randn((384, 900), generator=g, device="cuda")
    Cm = torch.randn((700, 900), generator=g, device="cuda")
    got = _gemm(cg, A, B, Cm, alpha, beta)
    _check(A, B, Cm, got, alpha, beta)


def test_gemm_row_scales(built):
    """Rows and columns spanning 1e-12 .. 1e6 in magnitude keep their relative accuracy (each
    row of A and column of B has its own power-of-two scale), and zero rows give zeros."""
    import torch
    import cpanel_gb300 as cg
    g = torch.Generator(device="cuda").manual_seed(11)
    m, n, k = 513, 300, 256
    A = torch.randn((m, k), generator=g, device="cuda") * torch.logspace(-12, 6, m, device="cuda")[:, None]
    B = torch.randn((k, n), generator=g, device="cuda") * torch.logspace(4, -10, n, device="cuda")[None, :]
    A[17] = 0
    B[:, 5] = 0
    got = _gemm(cg, A, B)
    _check(A, B, None, got, 1.0, 0.0)
    assert float(got[17].abs().max()) == 0.0 and float(got[:, 5].abs().max()) == 0.0


def test_gemm_sm_budget(built):
    """A grid limited to a few SMs (the rest left to other streams) gives the same bits."""
    import torch
    import cpanel_gb300 as cg
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn((1500, 512), generator=g, device="cuda")
    B = torch.randn((512, 1300), generator=g, device="cuda")
    full = _gemm(cg, A, B)
    few = _gemm(cg, A, B, sm_budget=7)
    assert torch.equal(full, few)
