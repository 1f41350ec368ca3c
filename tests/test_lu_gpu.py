"""The FP32 LU and its block substitutions (cpg_lu_solve_f32) against an FP64 solve.

The mixed precision factors A32 once without pivoting (1,024-column panels, tensor-core products
for the off-diagonal factors and the trailing updates) and solves by forward and backward block
substitutions with the diagonal blocks' inverses: skinny products with one kernel per column
count (groups of at most 32 columns), split along K into per-tile partials when a step has too
few rows to fill the GPU.  The matrices here are R / sqrt(n) + 2 I,
R standard normal, for which elimination without pivoting is stable.  Sizes cover a matrix below
one 1,024-column panel, whole panels followed by a ragged 128-column tail, and tall steps whose
products switch to 64-row tiles; the right-hand side counts cover single columns, odd counts and
more than one column group.  Bounds, normwise:

    ||A X - B|| <= 1e-5 ||A|| ||X||        (backward error of an FP32 factorization)
    ||X - X64|| <= 1e-4 ||X64||            (the condition number here is below 10)
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg(built):
    import cpanel_gb300
    return cpanel_gb300


def _lu_solve(cg, A, B):
    import torch
    n = A.shape[0]
    k = B.shape[1]
    # column-major storage: the transpose, row-major; copies, as the call overwrites both (for
    # one column B.t().contiguous() would be B itself)
    dA = A.t().contiguous().clone()
    dX = B.t().contiguous().clone()
    ctx = cg.Context.default()
    torch.cuda.synchronize()
    rc = ctx.L.cpg_lu_solve_f32(ctx.h, n, C.c_void_p(dA.data_ptr()), k, C.c_void_p(dX.data_ptr()))
    ctx.check(rc, "lu solve")
    return dX.t(), dA.t()


def _system(n, k, seed):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = torch.randn(n, n, generator=g, dtype=torch.float64) / np.sqrt(n) + 2 * torch.eye(n, dtype=torch.float64)
    B = torch.randn(n, k, generator=g, dtype=torch.float64)
    return A.float().cuda(), B.float().cuda()


@pytest.mark.parametrize("n,k", [(300, 1), (1100, 17), (2100, 40), (2500, 8), (2600, 33), (6000, 17), (5000, 3)])
def test_lu_solve_matches_fp64(cg, n, k):
    import torch
    A, B = _system(n, k, 100 + n + k)
    X, _ = _lu_solve(cg, A, B)
    A64, B64, X64 = A.double(), B.double(), X.double()
    back = float(torch.linalg.norm(A64 @ X64 - B64) / (torch.linalg.norm(A64) * torch.linalg.norm(X64)))
    assert back <= 1e-5, back
    ref = torch.linalg.solve(A64, B64)
    fwd = float(torch.linalg.norm(X64 - ref) / torch.linalg.norm(ref))
    assert fwd <= 1e-4, fwd


def test_lu_factors_reproduce_a(cg):
    import torch
    n = 1300
    A, B = _system(n, 1, 7)
    _, LU = _lu_solve(cg, A, B)
    LU = LU.double()
    L = torch.tril(LU, -1) + torch.eye(n, dtype=torch.float64, device=LU.device)
    U = torch.triu(LU)
    err = float(torch.linalg.norm(L @ U - A.double()) / torch.linalg.norm(A.double()))
    assert err <= 1e-5, err


def test_lu_solve_is_deterministic(cg):
    """The split products add their partials in a fixed order: two runs agree bit for bit."""
    import torch
    A, B = _system(3000, 17, 11)
    X1, _ = _lu_solve(cg, A, B)
    X2, _ = _lu_solve(cg, A, B)
    assert torch.equal(X1, X2)


def test_lu_zero_pivot_is_reported(cg):
    import torch
    A = torch.ones(64, 64, dtype=torch.float32, device="cuda")  # rank one: the second pivot is zero
    B = torch.ones(64, 1, dtype=torch.float32, device="cuda")
    with pytest.raises(cg.CpgError) as e:
        _lu_solve(cg, A, B)
    assert e.value.code == 1
