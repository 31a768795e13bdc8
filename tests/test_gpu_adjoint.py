"""Adjoint of the batched solve (differentiable-solve workload: 2,048 matrices
n=64, A = 4 I + uniform(-1,1), nrhs=4, upstream gradient N(0,1)).

Checks: the transposed solve and the outer product are bit-identical to the
oracle; the gradient agrees with torch's FP64 autograd through
torch.linalg.solve (the reference gradient) and with FP64 central finite
differences (h = 1e-6); torch.autograd.gradcheck passes on small sizes; the
FP32 form agrees with the FP64 gradient to FP32 accuracy."""
import numpy as np
import pytest
import torch

import oracle
from magma_gb300.autograd import solve, solve_with_info

pytestmark = pytest.mark.gpu


def _inputs(batch, n, nrhs, seed, dtype=torch.float64, dev="cuda"):
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = 4.0 * torch.eye(n, dtype=torch.float64) + (torch.rand((batch, n, n), generator=g,
                                                              dtype=torch.float64) * 2 - 1)
    B = torch.rand((batch, n, nrhs), generator=g, dtype=torch.float64) * 2 - 1
    gX = torch.randn((batch, n, nrhs), generator=g, dtype=torch.float64)
    return A.to(dev, dtype), B.to(dev, dtype), gX.to(dev, dtype)


def test_adjoint_bitexact_vs_oracle(cuda):
    A, B, gX = _inputs(64, 64, 4, seed=1)
    A.requires_grad_(True)
    B.requires_grad_(True)
    X = solve(A, B)
    X.backward(gX)
    torch.cuda.synchronize()
    # oracle: forward LU, then adjoint
    S = A.detach().transpose(1, 2).contiguous().cpu().numpy()
    Xs = B.detach().transpose(1, 2).contiguous().cpu().numpy()
    ipiv, info = oracle.dgesv_batched(S, Xs)
    G = gX.transpose(1, 2).contiguous().cpu().numpy()
    GA = oracle.gesv_adjoint_batched(S, ipiv, Xs, G)
    assert np.array_equal(X.detach().transpose(1, 2).cpu().numpy(), Xs)
    assert np.array_equal(B.grad.transpose(1, 2).cpu().numpy(), G)
    assert np.array_equal(A.grad.transpose(1, 2).cpu().numpy(), GA)


def test_adjoint_matches_torch_autograd_fp64(cuda):
    """2,048 matrices n=64 nrhs=4: against torch's FP64 autograd of linalg.solve."""
    A, B, gX = _inputs(2048, 64, 4, seed=2)
    A1, B1 = A.clone().requires_grad_(True), B.clone().requires_grad_(True)
    X1 = solve(A1, B1)
    X1.backward(gX)
    A2, B2 = A.clone().requires_grad_(True), B.clone().requires_grad_(True)
    X2 = torch.linalg.solve(A2, B2)
    X2.backward(gX)
    torch.cuda.synchronize()
    # two FP64 LU solvers agree to about cond(A) * eps; 4I + U(-1,1) at n = 64 has
    # condition numbers up to ~1e4 in this batch
    cond = torch.linalg.cond(A).max().item()
    tol = 64 * cond * 2.0 ** -52
    rel = lambda a, b: float((a - b).detach().abs().max() / b.detach().abs().max())
    assert rel(X1, X2) < tol
    assert rel(B1.grad, B2.grad) < tol
    assert rel(A1.grad, A2.grad) < 2 * tol


def test_adjoint_central_differences(cuda):
    """Directional derivatives of L = <gx, x(A, b)> against (L(+h) - L(-h)) / 2h."""
    A, B, gX = _inputs(8, 64, 4, seed=3)
    A1, B1 = A.clone().requires_grad_(True), B.clone().requires_grad_(True)
    solve(A1, B1).backward(gX)
    g = torch.Generator(device="cpu").manual_seed(4)
    h = 1e-6
    for _ in range(3):
        EA = torch.randn(A.shape, generator=g, dtype=torch.float64).to(A.device)
        EB = torch.randn(B.shape, generator=g, dtype=torch.float64).to(B.device)
        Lp = (gX * solve(A + h * EA, B + h * EB)).sum()
        Lm = (gX * solve(A - h * EA, B - h * EB)).sum()
        fd = float((Lp - Lm) / (2 * h))
        an = float((A1.grad * EA).sum() + (B1.grad * EB).sum())
        assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (fd, an)


def test_gradcheck_small(cuda):
    A, B, _ = _inputs(3, 7, 2, seed=5)
    A.requires_grad_(True)
    B.requires_grad_(True)
    assert torch.autograd.gradcheck(lambda a, b: solve(a, b), (A, B), eps=1e-6, atol=1e-7,
                                    rtol=1e-6)


def test_adjoint_fp32(cuda):
    A, B, gX = _inputs(2048, 64, 4, seed=6)
    A32, B32 = A.float().requires_grad_(True), B.float().requires_grad_(True)
    solve(A32, B32).backward(gX.float())
    A64, B64 = A.clone().requires_grad_(True), B.clone().requires_grad_(True)
    solve(A64, B64).backward(gX)
    torch.cuda.synchronize()
    rel = float((A32.grad.double() - A64.grad).abs().max() / A64.grad.abs().max())
    cond = torch.linalg.cond(A).max().item()
    assert rel < max(1e-4, 64 * cond * 2.0 ** -23)
    # FP32 path is bit-identical to the FP32 oracle too
    S = A32.detach().transpose(1, 2).contiguous().cpu().numpy()
    Xs = B32.detach().transpose(1, 2).contiguous().cpu().numpy()
    ipiv, _ = oracle.sgesv_batched(S, Xs)
    G = gX.float().transpose(1, 2).contiguous().cpu().numpy()
    GA = oracle.gesv_adjoint_batched(S, ipiv, Xs, G)
    assert np.array_equal(A32.grad.transpose(1, 2).cpu().numpy(), GA)


def test_info_reports_singular(cuda):
    A, B, _ = _inputs(4, 16, 1, seed=7)
    A[2] = 0.0
    X, info = solve_with_info(A, B)
    assert info.tolist() == [0, 0, 1, 0]
