"""Tensor-core trailing update (tcgen05 + TMEM, TMA-fed) of the FP32
factorisation, magma_sgetrf_batched_tc.

Exactness test: A = [[I, U12], [L21, A22]] with I of order 128 (one block of
the two-level factorisation), L21 and U12 multiples of 1/8 in (-1, 1) --
exactly representable in BF16 and FP16 -- and A22 multiples of 1/64 makes the
first 128 columns pivot-free with L21 as multipliers and U12 unchanged, and
every partial sum of the rank-128 tensor-core update exact in FP32.
Everything else (the panels, the updates inside a block, the U12 solves) runs
on the FP32 kernels.  So the result must equal the FP32 SIMT factorisation bit
for bit -- which checks the TMA maps, the swizzled operand descriptors of the
four 32-deep slices, the MMA instruction descriptor (including the negated A),
the TMEM read-back, the tile indexing, and the rows below the block that the
interchange step moves in place.  Then a random-matrix test bounds the
backward error."""
import ctypes as C

import numpy as np
import pytest
import torch

import magma_gb300 as mg
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, ptr_array
from tests.util import lu_error, to_storage, from_storage

pytestmark = pytest.mark.gpu
PREC = {"fp16": 905, "bf16": 930}


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _tc_getrf(S, m, prec, cuda):
    b, n, ld = S.shape
    lib = L.load()
    lw = C.c_size_t(0)
    assert lib.magma_sgetrf_batched_tc(PREC[prec], m, n, None, ld, None, None, None, C.byref(lw),
                                       b, None) == 0
    work = torch.empty((lw.value,), dtype=torch.uint8, device=cuda)
    ipiv = torch.empty((b, min(m, n)), dtype=torch.int32, device=cuda)
    info = torch.empty((b,), dtype=torch.int32, device=cuda)
    dA, dP = ptr_array(S), ptr_array(ipiv)
    q = Queue.current(cuda)
    rc = lib.magma_sgetrf_batched_tc(PREC[prec], m, n, _vp(dA), ld, _vp(dP), _vp(info), _vp(work),
                                     C.byref(lw), b, q.handle)
    assert rc == 0
    st = lib.magma_sgetrf_batched_tc_status(m, n, _vp(work), b, q.handle)
    assert st == 0, f"tensor-core pipeline reported error {st}"
    return ipiv, info


def _structured(rng, batch, m, n, w=128):
    # A22 in multiples of 1/64 too: every partial sum of the first update is then
    # exact in FP32, whichever order the FP32 or the tensor-core path adds in
    A = (rng.integers(-63, 64, (batch, m, n)) / 64.0).astype(np.float32)
    A[:, :w, :w] = np.eye(w, dtype=np.float32)
    A[:, w:, :w] = rng.integers(-7, 8, (batch, m - w, w)) / 8.0     # L21, |l| < 1
    A[:, :w, w:] = rng.integers(-7, 8, (batch, w, n - w)) / 8.0     # U12
    return A


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
@pytest.mark.parametrize("m,n", [(160, 160), (288, 160), (160, 288)])
def test_tc_update_exact_first_step(cuda, prec, m, n):
    rng = np.random.default_rng(m * 7 + n)
    A = _structured(rng, 6, m, n)
    S1 = torch.from_numpy(to_storage(A)).to(cuda)
    S2 = S1.clone()
    ipiv1, info1 = _tc_getrf(S1, m, prec, cuda)
    ipiv2, info2 = mg.getrf_batched(S2, m)
    torch.cuda.synchronize()
    assert torch.equal(ipiv1, ipiv2[:, :min(m, n)])
    assert torch.equal(S1, S2)


@pytest.mark.parametrize("prec,tol", [("bf16", 2.0 ** -8), ("fp16", 2.0 ** -11)])
def test_tc_getrf_backward_error(cuda, prec, tol):
    rng = np.random.default_rng(3)
    n = 512
    A = rng.uniform(-1, 1, (4, n, n)).astype(np.float32)
    S = torch.from_numpy(to_storage(A)).to(cuda)
    ipiv, info = _tc_getrf(S, n, prec, cuda)
    torch.cuda.synchronize()
    LU = from_storage(S.cpu().numpy(), n)
    err = lu_error(A.astype(np.float64), LU, ipiv.cpu().numpy())
    # normwise backward error of an LU whose updates use unit roundoff `tol`
    assert np.all(err < 4 * tol), err
    assert np.all(info.cpu().numpy() == 0)
