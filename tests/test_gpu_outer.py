"""GPU parity of the two-level blocked FP32 LU (128-column blocks of 32-column
panels, one rank-128 update right of each block: csrc/lu_outer.cu), through the
C ABI, bit-identical to the CPU oracle.

The shapes cover full and partial blocks (min(m, n) not a multiple of 128 or 32),
tall and wide matrices (blocks with no rows below them, columns right of the
last block), padded leading dimensions, singular columns and NaN entries, large
batches (the inner steps in the fused band kernel) and small ones (the per-tile
kernels), and variable-size batches through the per-step kernels.
"""
import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, VBatch, _vp
from tests.util import to_storage

pytestmark = pytest.mark.gpu


def _gpu_getrf(S, m, cuda):
    dS = torch.from_numpy(S).to(cuda)
    ipiv, info = mg.getrf_batched(dS, m)
    torch.cuda.synchronize()
    return dS.cpu().numpy(), ipiv.cpu().numpy(), info.cpu().numpy()


@pytest.mark.parametrize("m,n,batch", [(512, 512, 320), (300, 700, 64), (900, 300, 40),
                                       (1024, 1024, 3), (257, 257, 7), (160, 161, 5),
                                       (129, 300, 6), (700, 129, 5), (200, 260, 310),
                                       (1000, 999, 2), (65, 640, 4)])
def test_sgetrf_two_level_bitexact(cuda, m, n, batch):
    rng = np.random.default_rng(m * 31 + n * 7 + batch)
    S = to_storage(rng.uniform(-1, 1, (batch, m, n)).astype(np.float32))
    rS = S.copy()
    ripiv, rinfo = oracle.sgetrf_batched(rS, m)
    gS, gipiv, ginfo = _gpu_getrf(S, m, cuda)
    k = min(m, n)
    assert np.array_equal(ginfo, rinfo)
    assert np.array_equal(gipiv[:, :k], ripiv[:, :k])
    assert np.array_equal(gS, rS)


def test_sgetrf_two_level_padded_singular_nan(cuda):
    rng = np.random.default_rng(5)
    n, ld, batch = 300, 321, 330
    A = rng.uniform(-1, 1, (batch, n, n)).astype(np.float32)
    A[1, :, 130] = 0.0             # zero column inside the second block
    A[2, :, 5] = 0.0               # inside the first block
    A[3] = 0.0
    A[4, :, 299] = 0.0             # the last column
    A[5, 17, 200] = np.nan         # NaN below a later block
    A[6, 250, 3] = np.inf
    A[7, :, 128:256] *= 1e-30      # tiny trailing columns
    S = to_storage(A, ld)
    S[:, :, n:] = 7.0
    rS = S.copy()
    ripiv, rinfo = oracle.sgetrf_batched(rS, n)
    gS, gipiv, ginfo = _gpu_getrf(S, n, cuda)
    assert np.array_equal(ginfo, rinfo)
    assert list(ginfo[1:5]) == [131, 6, 1, 300]
    assert np.array_equal(gipiv, ripiv)
    assert np.array_equal(gS, rS, equal_nan=True)
    assert np.all(gS[:, :, n:] == 7.0)


@pytest.mark.parametrize("batch", [5, 320])
def test_sgesv_two_level_solution_bitexact(cuda, batch):
    rng = np.random.default_rng(batch)
    n, nrhs = 384, 3
    A = rng.uniform(-1, 1, (batch, n, n)).astype(np.float32)
    B = rng.uniform(-1, 1, (batch, n, nrhs)).astype(np.float32)
    S, X = to_storage(A), to_storage(B)
    rS, rX = S.copy(), X.copy()
    ripiv, rinfo = oracle.sgesv_batched(rS, rX)
    dS, dX = torch.from_numpy(S).to(cuda), torch.from_numpy(X).to(cuda)
    ipiv, info = mg.gesv_batched(dS, dX)
    torch.cuda.synchronize()
    assert np.array_equal(ipiv.cpu().numpy(), ripiv)
    assert np.array_equal(dS.cpu().numpy(), rS)
    assert np.array_equal(dX.cpu().numpy(), rX)


def test_sgetrf_vbatched_two_level(cuda):
    """Variable-size FP32 batch above the persistent kernel's sizes (per-step kernels with
    per-matrix sizes, largest matrix <= 1024 rows): each matrix's blocks end at its own
    min(m, n)."""
    rng = np.random.default_rng(44)
    shapes = [(700, 300), (300, 700), (513, 513), (1, 900), (900, 1), (64, 64), (1000, 1000),
              (257, 256), (33, 40), (0, 5), (600, 600), (130, 1000), (1000, 131), (200, 200)]
    shapes += [(int(a), int(b)) for a, b in rng.integers(100, 800, (290, 2))]
    ms = [m for m, _ in shapes]
    mats = [rng.uniform(-1, 1, (n, m + 3)).astype(np.float32) for m, n in shapes]
    A = VBatch([a.shape for a in mats], ms, torch.float32, cuda).load(mats)
    mn = [max(min(m, n), 1) for m, n in shapes]
    ipiv = torch.zeros((sum(mn),), dtype=torch.int32, device=cuda)
    offs = np.concatenate([[0], np.cumsum(mn)[:-1]])
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=cuda) * 4
    info = torch.full((len(shapes),), -7, dtype=torch.int32, device=cuda)
    rc = L.load().magma_sgetrf_vbatched(_vp(A.rows), _vp(A.ncols), _vp(A.ptrs), _vp(A.ld), _vp(dP),
                                        _vp(info), len(shapes), Queue.current(cuda).handle)
    torch.cuda.synchronize()
    assert rc == 0
    P = ipiv.cpu().numpy()
    inf = info.cpu().numpy()
    for k, (m, n) in enumerate(shapes):
        ref = mats[k].copy()
        rp, rinfo = oracle.sgetrf(ref, m)
        assert inf[k] == rinfo, k
        assert np.array_equal(A.view(k).cpu().numpy(), ref, equal_nan=True), k
        assert np.array_equal(P[offs[k]:offs[k] + min(m, n)], rp[:min(m, n)]), k
