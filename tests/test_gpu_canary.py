"""Out-of-bounds writes, checked without a sanitizer.

Every matrix, right-hand side, pivot vector and info array is placed inside a
larger device buffer whose other cells hold a sentinel bit pattern: guard
columns before and after each matrix, padding rows between m and ld, guard
entries around each pivot vector and around the info array.  After a call, every
sentinel cell must still hold its pattern (no kernel wrote outside its operand)
and the operands must equal the oracle's bit for bit (no kernel read outside
its operand in a way that changed a result).  Sizes are the ragged edges of the
kernels' tiles and panels (1, 2, 3, 7, 31-33, 63-65, 127-129, 255-257, 300) at
batch counts 1, 2 and 33, plus one batch large enough for the FP32 band kernel
and the refinement solve.
"""
import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle

pytestmark = pytest.mark.gpu

GUARD = 5                         # guard columns / entries on each side
SENT64 = 0x7FF80000DEADBEEF       # a NaN payload no kernel produces
SENT32 = 0x7FC0BEEF
SENTI = -777777


def _guarded(host: np.ndarray, pad_rows: int, cuda):
    """(batch, ncols, m) host storage -> guarded device buffer and the view the
    library works on: (batch, ncols, m + pad_rows) with GUARD sentinel columns
    before and after each matrix."""
    b, nc, m = host.shape
    ld = m + pad_rows
    dt = torch.float64 if host.dtype == np.float64 else torch.float32
    it = torch.int64 if dt == torch.float64 else torch.int32
    big = torch.empty((b, nc + 2 * GUARD, ld), dtype=dt, device=cuda)
    big.view(it).fill_(SENT64 if dt == torch.float64 else SENT32)
    view = big[:, GUARD:GUARD + nc, :]
    view[:, :, :m] = torch.from_numpy(host).to(cuda)
    return big, view


def _sentinels_intact(big: torch.Tensor, nc: int, m: int) -> bool:
    it = torch.int64 if big.dtype == torch.float64 else torch.int32
    s = SENT64 if big.dtype == torch.float64 else SENT32
    bits = big.view(it)
    mask = torch.ones_like(bits, dtype=torch.bool)
    mask[:, GUARD:GUARD + nc, :m] = False
    return bool((bits[mask] == s).all().item()) if mask.any() else True


def _guarded_ints(b: int, k: int, cuda):
    big = torch.full((b, k + 2 * GUARD), SENTI, dtype=torch.int32, device=cuda)
    return big, big[:, GUARD:GUARD + k]


def _ints_intact(big: torch.Tensor, k: int) -> bool:
    mask = torch.ones_like(big, dtype=torch.bool)
    mask[:, GUARD:GUARD + k] = False
    return bool((big[mask] == SENTI).all().item())


SIZES = [1, 2, 3, 7, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257, 300]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("batch", [1, 2, 33])
def test_gesv_writes_stay_inside(cuda, dtype, batch):
    rng = np.random.default_rng(batch * 7 + (dtype == np.float32))
    for n in SIZES:
        for nrhs in (1, 3):
            A = rng.uniform(-1, 1, (batch, n, n)).astype(dtype)
            B = rng.uniform(-1, 1, (batch, nrhs, n)).astype(dtype)
            bigA, S = _guarded(A, 3, cuda)
            bigB, X = _guarded(B, 2, cuda)
            bigP, ipiv = _guarded_ints(batch, n, cuda)
            bigI, info = _guarded_ints(1, batch, cuda)
            mg.gesv_batched(S, X, ipiv=ipiv, info=info[0])
            torch.cuda.synchronize()
            rA, rB = A.copy(), B.copy()
            rp, ri = (oracle.dgesv_batched if dtype == np.float64 else oracle.sgesv_batched)(rA, rB)
            where = f"n={n} nrhs={nrhs} batch={batch} {np.dtype(dtype).name}"
            assert _sentinels_intact(bigA, n, n), where
            assert _sentinels_intact(bigB, nrhs, n), where
            assert _ints_intact(bigP, n), where
            assert _ints_intact(bigI, batch), where
            assert np.array_equal(S[:, :, :n].cpu().numpy(), rA), where
            assert np.array_equal(X[:, :, :n].cpu().numpy(), rB, equal_nan=True), where
            assert np.array_equal(ipiv.cpu().numpy(), rp[:, :n]), where
            assert np.array_equal(info[0].cpu().numpy(), ri), where


@pytest.mark.parametrize("m,n,batch", [(257, 257, 320), (300, 129, 320), (129, 300, 320)])
def test_fp32_band_and_two_level_writes_stay_inside(cuda, m, n, batch):
    rng = np.random.default_rng(m + n)
    A = rng.uniform(-1, 1, (batch, n, m)).astype(np.float32)   # storage (batch, ncols, m)
    bigA, S = _guarded(A, 5, cuda)
    bigP, ipiv = _guarded_ints(batch, min(m, n), cuda)
    mg.getrf_batched(S, m, ipiv=ipiv)
    torch.cuda.synchronize()
    rA = A.copy()
    rp, _ = oracle.sgetrf_batched(rA, m)
    assert _sentinels_intact(bigA, n, m)
    assert _ints_intact(bigP, min(m, n))
    assert np.array_equal(S[:, :, :m].cpu().numpy(), rA)
    assert np.array_equal(ipiv.cpu().numpy(), rp[:, :min(m, n)])


@pytest.mark.parametrize("n,batch", [(33, 33), (129, 40), (300, 33), (512, 8)])
def test_refinement_writes_stay_inside(cuda, n, batch):
    rng = np.random.default_rng(n)
    nrhs = 2
    A = rng.uniform(-1, 1, (batch, n, n))
    A[0] = 0.0                              # a singular matrix: the FP64 fallback writes A
    B = rng.uniform(-1, 1, (batch, nrhs, n))
    bigA, S = _guarded(A, 3, cuda)
    bigB, Bd = _guarded(B, 1, cuda)
    bigX, X = _guarded(np.zeros_like(B), 4, cuda)
    bigP, ipiv = _guarded_ints(batch, n, cuda)
    _, _, info, iters = mg.dsgesv_batched(S, Bd, X=X, ipiv=ipiv, tol=30.0)
    torch.cuda.synchronize()
    rS = A.copy()
    rX, rp, rinfo, riters = oracle.dsgesv_batched(rS, B.copy(), tol=30.0)
    assert _sentinels_intact(bigA, n, n)
    assert _sentinels_intact(bigB, nrhs, n)
    assert _sentinels_intact(bigX, nrhs, n)
    assert _ints_intact(bigP, n)
    assert np.array_equal(iters.cpu().numpy(), riters)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    assert np.array_equal(X[:, :, :n].cpu().numpy(), rX, equal_nan=True)   # the singular one: inf/NaN
    assert np.array_equal(S[:, :, :n].cpu().numpy(), rS)
