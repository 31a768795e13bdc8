"""GPU parity for the batched mixed-precision iterative refinement
(magma_dsgesv_batched_work) against the oracle's restatement of
magma_dsgesv_gpu: iterates, iteration counts (ITER codes), pivots and info are
bit-identical; solutions are FP64-accurate.

Edge cases follow src/zcgesv_gpu.cpp: FP32 overflow (iter -2), singular FP32
factor (iter -3), no convergence (iter -itermax-1), each followed by the FP64
re-solve."""
import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from magma_gb300.testing import svd_batch_torch
from tests.util import from_storage, scaled_residual, to_storage

pytestmark = pytest.mark.gpu


def _svd(batch, n, kappas, seed):
    return svd_batch_torch(batch, n, kappas, seed, device="cpu").numpy()


def _run_both(A, Bm, cuda, itermax=30, tol=0.0, fallback=True):
    n = A.shape[1]
    S, Bs = to_storage(A), to_storage(Bm)
    rS = S.copy()
    rX, ripiv, rinfo, riters = oracle.dsgesv_batched(rS, Bs, itermax=itermax, tol=tol,
                                                     fallback=fallback)
    dS = torch.from_numpy(S).to(cuda)
    dB = torch.from_numpy(Bs).to(cuda)
    X, ipiv, info, iters = mg.dsgesv_batched(dS, dB, itermax=itermax, tol=tol, fallback=fallback)
    torch.cuda.synchronize()
    gpu = (X.cpu().numpy(), ipiv.cpu().numpy(), info.cpu().numpy(), iters.cpu().numpy(),
           dS.cpu().numpy())
    ref = (rX, ripiv, rinfo, riters, rS)
    return gpu, ref


def _assert_same(gpu, ref, n):
    X, ipiv, info, iters, S = gpu
    rX, ripiv, rinfo, riters, rS = ref
    assert np.array_equal(iters, riters), (iters, riters)
    assert np.array_equal(info, rinfo)
    assert np.array_equal(ipiv[:, :n], ripiv[:, :n])
    assert np.array_equal(X, rX, equal_nan=True)     # singular matrices give inf/NaN
    assert np.array_equal(S, rS, equal_nan=True)


@pytest.mark.parametrize("tol", [0.0, 30.0])
@pytest.mark.parametrize("n,nrhs", [(20, 1), (64, 4), (100, 9), (160, 16)])
def test_dsgesv_matches_oracle(cuda, n, nrhs, tol):
    kappas = [1e2, 1e4, 1e6] * 3
    A = _svd(9, n, kappas, seed=n)
    Bm = np.random.default_rng(n).uniform(-1, 1, (9, n, nrhs))
    gpu, ref = _run_both(A, Bm, cuda, tol=tol)
    _assert_same(gpu, ref, n)
    assert np.all(gpu[3] >= 0)
    res = scaled_residual(A, from_storage(gpu[0], n), Bm)
    assert res.max() <= 30


def test_dsgesv_n512_kappa_mix(cuda):
    """The refinement workload's shape (n=512, nrhs=4, kappa 1e2/1e4/1e6) on a small batch."""
    A = _svd(3, 512, [1e2, 1e4, 1e6], seed=5)
    Bm = np.random.default_rng(5).uniform(-1, 1, (3, 512, 4))
    gpu, ref = _run_both(A, Bm, cuda, tol=30.0)
    _assert_same(gpu, ref, 512)
    assert scaled_residual(A, from_storage(gpu[0], 512), Bm).max() <= 30


def test_dsgesv_no_convergence_falls_back(cuda):
    A = _svd(2, 48, [1e12, 1e2], seed=9)
    Bm = np.random.default_rng(9).uniform(-1, 1, (2, 48, 2))
    gpu, ref = _run_both(A, Bm, cuda, itermax=3)
    _assert_same(gpu, ref, 48)
    assert gpu[3][0] == -4 and gpu[3][1] >= 0
    assert not np.array_equal(gpu[4][0], to_storage(A)[0])    # A_0 now holds its FP64 LU
    assert np.array_equal(gpu[4][1], to_storage(A)[1])        # A_1 untouched


def test_dsgesv_overflow_and_singular(cuda):
    rng = np.random.default_rng(4)
    A = rng.uniform(-1, 1, (3, 40, 40))
    A[0, 3, 7] = 1e39          # not representable in FP32
    A[1, :, 5] = 0.0           # singular in both precisions
    Bm = rng.uniform(-1, 1, (3, 40, 1))
    gpu, ref = _run_both(A, Bm, cuda)
    _assert_same(gpu, ref, 40)
    assert list(gpu[3][:2]) == [-2, -3]
    assert gpu[2][1] == 6 and gpu[3][2] >= 0


def test_dsgesv_without_fallback_never_syncs_and_reports(cuda):
    A = _svd(2, 48, [1e12, 1e3], seed=3)
    Bm = np.random.default_rng(3).uniform(-1, 1, (2, 48, 1))
    gpu, ref = _run_both(A, Bm, cuda, itermax=2, tol=30.0, fallback=False)
    _assert_same(gpu, ref, 48)
    assert gpu[3][0] < 0 and gpu[3][1] >= 0
    assert np.array_equal(gpu[4], to_storage(A))             # A untouched without fallback


def test_dsgesv_public_entry_uses_queue_workspace(cuda):
    """magma_dsgesv_batched (no _work) grows the queue's workspace itself."""
    import ctypes as C
    from magma_gb300 import lib as L
    from magma_gb300.batched import Queue, ptr_array
    n, nrhs, b = 70, 3, 5
    A = _svd(b, n, [1e3] * b, seed=2)
    Bm = np.random.default_rng(2).uniform(-1, 1, (b, n, nrhs))
    S, Bs = to_storage(A), to_storage(Bm)
    rX, ripiv, rinfo, riters = oracle.dsgesv_batched(S.copy(), Bs)
    dS = torch.from_numpy(S).to(cuda)
    dB = torch.from_numpy(Bs).to(cuda)
    dX = torch.empty_like(dB)
    ipiv = torch.empty((b, n), dtype=torch.int32, device=cuda)
    info = torch.empty((b,), dtype=torch.int32, device=cuda)
    iters = torch.empty((b,), dtype=torch.int32, device=cuda)
    q = Queue.current(cuda)
    pa, pp, pb, px = ptr_array(dS), ptr_array(ipiv), ptr_array(dB), ptr_array(dX)
    rc = L.load().magma_dsgesv_batched(n, nrhs, C.c_void_p(pa.data_ptr()), n,
                                       C.c_void_p(pp.data_ptr()), C.c_void_p(pb.data_ptr()), n,
                                       C.c_void_p(px.data_ptr()), n, C.c_void_p(info.data_ptr()),
                                       C.c_void_p(iters.data_ptr()), b, q.handle)
    torch.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(dX.cpu().numpy(), rX)
    assert np.array_equal(iters.cpu().numpy(), riters)


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
def test_dxgesv_tensor_core_factorisation(cuda, precision):
    """FP32 factorisation with tensor-core (BF16 / FP16) trailing updates + FP64
    refinement: every solve ends FP64-accurate; the well-conditioned third
    converges by refinement alone."""
    n, nrhs = 320, 4
    A = _svd(6, n, [1e2, 1e2, 1e4, 1e4, 1e6, 1e6], seed=21)
    Bm = np.random.default_rng(21).uniform(-1, 1, (6, n, nrhs))
    dS = torch.from_numpy(to_storage(A)).to(cuda)
    dB = torch.from_numpy(to_storage(Bm)).to(cuda)
    X, ipiv, info, iters = mg.dsgesv_batched(dS, dB, tol=30.0, precision=precision)
    torch.cuda.synchronize()
    it = iters.cpu().numpy()
    assert np.all(it[:2] >= 0), it
    res = scaled_residual(A, from_storage(X.cpu().numpy(), n), Bm)
    assert res.max() <= 30, (res, it)


def test_dxgesv_fp32_equals_dsgesv(cuda):
    """Precision 900 of the general entry is the FP32 refinement, bit for bit."""
    A = _svd(3, 100, [1e3] * 3, seed=8)
    Bm = np.random.default_rng(8).uniform(-1, 1, (3, 100, 2))
    gpu, ref = _run_both(A, Bm, cuda)
    _assert_same(gpu, ref, 100)


def _vb_case(seed, count, nmax, rmax, kappa_hi=1e6, kappa_fixed=None):
    rng = np.random.default_rng(seed)
    ns = [int(x) for x in rng.integers(1, nmax + 1, count)]
    rs = [int(x) for x in rng.integers(1, rmax + 1, count)]
    kap = 10.0 ** rng.uniform(0, np.log10(kappa_hi), count)
    if kappa_fixed is not None:
        kap[:] = kappa_fixed
    As, Bs = [], []
    for k, (n, r) in enumerate(zip(ns, rs)):
        A = _svd(1, n, [float(kap[k])], seed=seed * 1000 + k)[0]
        As.append(np.ascontiguousarray(A.T))                     # storage (ncols, ld = n)
        Bs.append(rng.uniform(-1, 1, (r, n)))
    return ns, rs, As, Bs


@pytest.mark.parametrize("tol", [0.0, 30.0])
def test_dxgesv_vbatched_matches_oracle(cuda, tol):
    """Variable-size refinement (FP32 persistent factorisation): solutions, pivots, info and
    iteration counts bit-identical to the oracle matrix by matrix, including matrices with
    kappa 1e9 that fall back to the FP64 re-solve."""
    ns, rs, As, Bs = _vb_case(3, 40, 200, 16)
    extra = _vb_case(4, 3, 90, 4, kappa_fixed=1e10)       # these do not converge in FP32
    ns, rs, As, Bs = ns + extra[0], rs + extra[1], As + extra[2], Bs + extra[3]
    ns.append(1); rs.append(1); As.append(np.array([[3.0]])); Bs.append(np.array([[1.5]]))
    A = mg.VBatch([a.shape for a in As], ns, torch.float64, cuda).load(As)
    B = mg.VBatch([b.shape for b in Bs], ns, torch.float64, cuda).load(Bs)
    X, ipiv, offs, info, iters, _ = mg.dxgesv_vbatched(A, B, tol=tol)
    torch.cuda.synchronize()
    rA = [a.copy() for a in As]
    rX, rp, rinfo, riters = oracle.dsgesv_vbatched(rA, Bs, tol=tol)
    it = iters.cpu().numpy()
    assert np.array_equal(it, riters), (it, riters)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    P = ipiv.cpu().numpy()
    for k, n in enumerate(ns):
        assert np.array_equal(P[offs[k]:offs[k] + n], rp[k]), k
        assert np.array_equal(X.view(k).cpu().numpy(), rX[k], equal_nan=True), k
        assert np.array_equal(A.view(k).cpu().numpy(), rA[k], equal_nan=True), k
    assert (it < 0).any() and (it >= 0).any()


def test_dxgesv_vbatched_band_path_matches_oracle(cuda):
    """Variable-size refinement with matrices above 256 and a large batch: the FP32
    factorisation runs through the per-step kernels with per-matrix sizes and the band
    kernel; bit-identical to the oracle matrix by matrix."""
    ns, rs, As, Bs = _vb_case(5, 320, 400, 4)
    A = mg.VBatch([a.shape for a in As], ns, torch.float64, cuda).load(As)
    B = mg.VBatch([b.shape for b in Bs], ns, torch.float64, cuda).load(Bs)
    X, ipiv, offs, info, iters, _ = mg.dxgesv_vbatched(A, B, tol=30.0)
    torch.cuda.synchronize()
    rA = [a.copy() for a in As]
    rX, rp, rinfo, riters = oracle.dsgesv_vbatched(rA, Bs, tol=30.0)
    assert max(ns) > 256
    assert np.array_equal(iters.cpu().numpy(), riters)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    P = ipiv.cpu().numpy()
    for k, n in enumerate(ns):
        assert np.array_equal(P[offs[k]:offs[k] + n], rp[k]), k
        assert np.array_equal(X.view(k).cpu().numpy(), rX[k], equal_nan=True), k


def test_dsgesv_adjoint_matches_oracle(cuda):
    """Adjoint of the refinement solve: GB = A^{-T} G refined with the forward's FP32
    factors, GA = -GB X^T; bit-identical to the oracle, including matrices whose forward
    solve fell back to FP64 (kappa 1e10) and use their FP64 factors."""
    n, nrhs, b = 64, 4, 8
    kappas = [1e2, 1e4, 1e6, 1e10, 1e3, 1e5, 1e10, 1e1]
    A = _svd(b, n, kappas, seed=77)
    Bm = np.random.default_rng(77).uniform(-1, 1, (b, n, nrhs))
    dS = torch.from_numpy(to_storage(A)).to(cuda)
    dB = torch.from_numpy(to_storage(Bm)).to(cuda)
    work = torch.empty((mg.dsgesv_workspace_bytes(n, nrhs, b),), dtype=torch.uint8, device=cuda)
    X, ipiv, info, iters = mg.dsgesv_batched(dS, dB, work=work)
    torch.cuda.synchronize()
    S_fwd, P_fwd, X_h, it_h = dS.cpu().numpy().copy(), ipiv.cpu().numpy(), X.cpu().numpy(), \
        iters.cpu().numpy()
    assert (it_h < 0).sum() == 2
    G = torch.from_numpy(np.random.default_rng(78).standard_normal((b, nrhs, n))).to(cuda)
    GB, GA, it2 = mg.dsgesv_adjoint_batched(dS, ipiv, X, G, iters, work, info)
    torch.cuda.synchronize()
    G_h = G.cpu().numpy()
    for k in range(b):
        rGB, rGA, rinfo, rit, _ = oracle.dsgesv_adjoint(S_fwd[k].copy(), P_fwd[k], X_h[k], G_h[k],
                                                        it_h[k])
        assert int(it2[k]) == rit, k
        assert np.array_equal(GB[k].cpu().numpy(), rGB), k
        assert np.array_equal(GA[k].cpu().numpy(), rGA), k
    # against an FP64 reference gradient
    Ad = torch.from_numpy(A)
    gb_ref = torch.linalg.solve(Ad.transpose(1, 2), torch.from_numpy(G_h).transpose(1, 2))
    err = (GB.cpu().transpose(1, 2) - gb_ref).abs().amax() / gb_ref.abs().amax()
    assert float(err) < 1e-6


def test_dxgesv_adjoint_vbatched_matches_oracle(cuda):
    ns, rs, As, Bs = _vb_case(9, 30, 160, 8, kappa_hi=1e5)
    extra = _vb_case(10, 2, 60, 3, kappa_fixed=1e12)     # forward falls back to FP64
    ns, rs, As, Bs = ns + extra[0], rs + extra[1], As + extra[2], Bs + extra[3]
    A = mg.VBatch([a.shape for a in As], ns, torch.float64, cuda).load(As)
    B = mg.VBatch([b.shape for b in Bs], ns, torch.float64, cuda).load(Bs)
    X, ipiv, offs, info, iters, work = mg.dxgesv_vbatched(A, B)
    torch.cuda.synchronize()
    A_fwd = [A.view(k).cpu().numpy().copy() for k in range(len(ns))]
    P = ipiv.cpu().numpy()
    it_h = iters.cpu().numpy()
    rng = np.random.default_rng(11)
    Gs = [rng.standard_normal(b.shape) for b in Bs]
    G = mg.VBatch([g.shape for g in Gs], ns, torch.float64, cuda).load(Gs)
    GB, GA, it2 = mg.dxgesv_adjoint_vbatched(A, ipiv, offs, X, G, iters, info, work)
    torch.cuda.synchronize()
    it2 = it2.cpu().numpy()
    for k, n in enumerate(ns):
        rGB, rGA, rinfo, rit, _ = oracle.dsgesv_adjoint(A_fwd[k].copy(), P[offs[k]:offs[k] + n],
                                                        X.view(k).cpu().numpy(), Gs[k], it_h[k])
        assert it2[k] == rit, k
        assert np.array_equal(GB.view(k).cpu().numpy(), rGB), k
        assert np.array_equal(GA.view(k).cpu().numpy(), rGA), k
