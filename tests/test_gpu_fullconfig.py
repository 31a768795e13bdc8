"""GPU parity at the benchmark's full sizes, bit for bit against the oracle.

* The mixed-precision refinement workload: 512 FP64 matrices of order 512, four
  right-hand sides, A = U diag(s) V^T with kappa 1e2/1e4/1e6 (one third each),
  the FP32 factorisation through the two-level blocked path with the fused band
  kernel (a batch this large), stop at scaled residual <= 30 -- solutions,
  iteration codes, pivots and info identical to the oracle's restatement of
  magma_dsgesv_gpu.
* The variable-size workload: 4,096 matrices of order 8..256 with 1..16
  right-hand sides, factored and solved in one CUDA graph replay of
  magma_dgesv_vbatched_max_nocheck_work -- identical to the oracle.
* The serving workload: 64 of its matrices (orders 128..1024, kappa up to 1e4,
  eight right-hand sides), forward refinement and the refined adjoint,
  identical to the oracle matrix by matrix.

Inputs are built as bench.py builds them (same constructions and seeds).
"""
import ctypes as C

import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, VBatch, _vp
from magma_gb300.testing import svd_batch_torch

pytestmark = pytest.mark.gpu


def test_refinement_workload_full_size(cuda):
    batch, n, nrhs, seed = 512, 512, 4, 20240603
    kap = ([1e2, 1e4, 1e6] * (batch // 3 + 1))[:batch]
    A = svd_batch_torch(batch, n, kap, seed, device=cuda)            # (batch, n, n) on the GPU
    g = torch.Generator(device="cpu").manual_seed(seed + 1)
    Bm = torch.rand((batch, n, nrhs), generator=g, dtype=torch.float64) * 2 - 1
    S = A.transpose(1, 2).contiguous()
    Bs = Bm.transpose(1, 2).contiguous()
    S_h, Bs_h = S.cpu().numpy(), Bs.numpy().copy()
    X, ipiv, info, iters = mg.dsgesv_batched(S, Bs.to(cuda), tol=30.0)
    torch.cuda.synchronize()
    rS = S_h.copy()
    rX, ripiv, rinfo, riters = oracle.dsgesv_batched(rS, Bs_h, tol=30.0)
    it = iters.cpu().numpy()
    assert np.array_equal(it, riters)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    assert np.array_equal(ipiv.cpu().numpy(), ripiv)
    assert np.array_equal(X.cpu().numpy(), rX)
    assert np.all(it >= 1) and np.all(it <= 3)       # kappa 1e2, 1e4, 1e6: 1, 2, 3 iterations


def test_vbatched_workload_full_size_in_graph(cuda):
    batch, seed = 4096, 20240602
    rng = np.random.default_rng(seed)
    ns = [int(x) for x in rng.integers(8, 257, batch)]
    rs = [int(x) for x in rng.integers(1, 17, batch)]
    rng = np.random.default_rng(seed + 1)
    As = [rng.uniform(-1, 1, (n, n)) for n in ns]
    Bs = [rng.uniform(-1, 1, (r, n)) for n, r in zip(ns, rs)]
    A = VBatch([a.shape for a in As], ns, torch.float64, cuda).load(As)
    B = VBatch([b.shape for b in Bs], ns, torch.float64, cuda).load(Bs)
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]])
    ipiv = torch.zeros((sum(ns),), dtype=torch.int32, device=cuda)
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=cuda) * 4
    info = torch.empty((batch,), dtype=torch.int32, device=cuda)
    lib = L.load()
    lw = C.c_int(-1)
    lib.magma_dgesv_vbatched_max_nocheck_work(None, None, max(ns), max(rs), None, None, None, None,
                                              None, None, None, C.byref(lw), batch, None)
    work = torch.empty((lw.value,), dtype=torch.uint8, device=cuda)
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()

    def call(q):
        return lib.magma_dgesv_vbatched_max_nocheck_work(
            _vp(A.ncols), _vp(B.ncols), max(ns), max(rs), _vp(A.ptrs), _vp(A.ld), _vp(dP),
            _vp(B.ptrs), _vp(B.ld), _vp(info), _vp(work), C.byref(lw), batch, q.handle)
    with torch.cuda.stream(s):
        q = Queue(cuda.index or 0, s.cuda_stream)
        assert call(q) == 0                       # eager once (kernel attributes)
        s.synchronize()
        with torch.cuda.graph(graph, stream=s):
            assert call(q) == 0
    A.load(As)
    B.load(Bs)
    torch.cuda.synchronize()
    graph.replay()
    torch.cuda.synchronize()
    rA = [a.copy() for a in As]
    rB = [b.copy() for b in Bs]
    rp, rinfo = oracle.dgesv_vbatched(ns, rs, rA, rB)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    P = ipiv.cpu().numpy()
    for k in range(batch):
        assert np.array_equal(P[offs[k]:offs[k] + ns[k]], rp[k]), k
        assert np.array_equal(A.view(k).cpu().numpy(), rA[k]), k
        assert np.array_equal(B.view(k).cpu().numpy(), rB[k]), k


def test_serving_workload_forward_and_adjoint(cuda):
    seed, nrhs, take = 20240605, 8, 64
    rng = np.random.default_rng(seed)
    ns_all = [int(x) for x in rng.integers(128, 1025, 256)]
    kap_all = [float(x) for x in 10.0 ** rng.uniform(0.0, 4.0, 256)]
    ns, As, Bs, Gs = [], [], [], []
    for k in range(take):
        n, kp = ns_all[k], kap_all[k]
        r = np.random.default_rng(seed * 7919 + k)
        U = np.linalg.qr(r.standard_normal((n, n)))[0]
        V = np.linalg.qr(r.standard_normal((n, n)))[0]
        sv = np.geomspace(1.0, 1.0 / kp, n)
        As.append(np.ascontiguousarray(((U * sv) @ V.T).T))
        Bs.append(r.standard_normal((nrhs, n)))
        Gs.append(r.standard_normal((nrhs, n)))
        ns.append(n)
    assert max(ns) > 256                          # the per-step kernels, two-level blocked
    A = VBatch([a.shape for a in As], ns, torch.float64, cuda).load(As)
    B = VBatch([b.shape for b in Bs], ns, torch.float64, cuda).load(Bs)
    X, ipiv, offs, info, iters, work = mg.dxgesv_vbatched(A, B, tol=30.0)
    torch.cuda.synchronize()
    rA = [a.copy() for a in As]
    rX, rp, rinfo, riters = oracle.dsgesv_vbatched(rA, Bs, tol=30.0)
    it = iters.cpu().numpy()
    assert np.array_equal(it, riters)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    P = ipiv.cpu().numpy()
    A_fwd = []
    for k, n in enumerate(ns):
        assert np.array_equal(P[offs[k]:offs[k] + n], rp[k]), k
        assert np.array_equal(X.view(k).cpu().numpy(), rX[k]), k
        A_fwd.append(A.view(k).cpu().numpy().copy())
    G = VBatch([g.shape for g in Gs], ns, torch.float64, cuda).load(Gs)
    GB, GA, it2 = mg.dxgesv_adjoint_vbatched(A, ipiv, offs, X, G, iters, info, work, tol=30.0)
    torch.cuda.synchronize()
    it2 = it2.cpu().numpy()
    for k, n in enumerate(ns):
        rGB, rGA, _, rit, _ = oracle.dsgesv_adjoint(A_fwd[k].copy(), P[offs[k]:offs[k] + n],
                                                    X.view(k).cpu().numpy(), Gs[k], it[k], tol=30.0)
        assert it2[k] == rit, k
        assert np.array_equal(GB.view(k).cpu().numpy(), rGB), k
        assert np.array_equal(GA.view(k).cpu().numpy(), rGA), k
