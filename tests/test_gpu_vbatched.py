"""GPU parity for the variable-size path (persistent one-CTA-per-matrix kernel)
through the C ABI, bit-identical to the CPU oracle matrix by matrix.

Cases follow testing/testing_zgetrf_vbatched.cpp: random sizes per matrix
(including 0 and 1), rectangular getrf, padded leading dimensions; plus the
solves MAGMA lacks (getrs N/T, gesv), singular matrices, CUDA-graph capture of
the no-sync entry point, and MAGMA's argument-error codes."""
import ctypes as C

import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, VBatch

pytestmark = pytest.mark.gpu


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _make(rng, ns, nrhss, ld_pad=0, dtype=np.float64):
    As = [rng.uniform(-1, 1, (n, n + ld_pad)).astype(dtype) for n in ns]   # (ncols, ld) storage
    Bs = [rng.uniform(-1, 1, (r, n + ld_pad)).astype(dtype) for n, r in zip(ns, nrhss)]
    return As, Bs


def _gpu_gesv(As, Bs, ns, cuda, dtype=torch.float64):
    A = VBatch([a.shape for a in As], ns, dtype, cuda).load(As)
    B = VBatch([b.shape for b in Bs], ns, dtype, cuda).load(Bs)
    ipiv, offs, info = mg.gesv_vbatched(A, B)
    torch.cuda.synchronize()
    Ao = [A.view(k).cpu().numpy() for k in range(len(ns))]
    Bo = [B.view(k).cpu().numpy() for k in range(len(ns))]
    P = ipiv.cpu().numpy()
    pivs = [P[offs[k]:offs[k] + ns[k]] for k in range(len(ns))]
    return Ao, Bo, pivs, info.cpu().numpy()


def _check_same(gpu, As, Bs, ns, nrhss):
    rA = [a.copy() for a in As]
    rB = [b.copy() for b in Bs]
    rp, rinfo = oracle.dgesv_vbatched(ns, nrhss, rA, rB)
    Ao, Bo, pivs, info = gpu
    assert np.array_equal(info, rinfo)
    for k in range(len(ns)):
        assert np.array_equal(pivs[k], rp[k]), k
        assert np.array_equal(Ao[k], rA[k], equal_nan=True), k
        assert np.array_equal(Bo[k], rB[k], equal_nan=True), k


@pytest.mark.parametrize("seed", [0, 1])
def test_gesv_vbatched_random_sizes(cuda, seed):
    rng = np.random.default_rng(seed)
    ns = list(rng.integers(1, 300, 60)) + [1, 2, 31, 32, 33, 64, 65, 256, 257]
    ns = [int(n) for n in ns]
    nrhss = [int(r) for r in rng.integers(1, 17, len(ns))]
    As, Bs = _make(rng, ns, nrhss, ld_pad=int(seed) * 3)
    _check_same(_gpu_gesv(As, Bs, ns, cuda), As, Bs, ns, nrhss)


def test_gesv_vbatched_singular_and_large(cuda):
    rng = np.random.default_rng(5)
    ns = [40, 700, 17, 129]
    nrhss = [3, 2, 16, 1]
    As, Bs = _make(rng, ns, nrhss)
    As[0][5, :] = 0.0          # column 6 of matrix 0 is zero (storage row = matrix column)
    As[2][:, :] = 0.0          # all-zero matrix
    _check_same(_gpu_gesv(As, Bs, ns, cuda), As, Bs, ns, nrhss)


def test_getrf_vbatched_rectangular(cuda):
    rng = np.random.default_rng(7)
    shapes = [(50, 30), (30, 50), (1, 9), (9, 1), (100, 100), (64, 70), (200, 33)]
    ms = [m for m, _ in shapes]
    ns = [n for _, n in shapes]
    mats = [rng.uniform(-1, 1, (n, m + 2)) for m, n in shapes]          # storage (ncols, ld)
    A = VBatch([a.shape for a in mats], ms, torch.float64, cuda).load(mats)
    tot = sum(max(min(m, n), 1) for m, n in shapes)
    ipiv = torch.zeros((tot,), dtype=torch.int32, device=cuda)
    offs = np.concatenate([[0], np.cumsum([max(min(m, n), 1) for m, n in shapes])[:-1]])
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=cuda) * 4
    info = torch.empty((len(shapes),), dtype=torch.int32, device=cuda)
    rc = L.load().magma_dgetrf_vbatched(_vp(A.rows), _vp(A.ncols), _vp(A.ptrs), _vp(A.ld), _vp(dP),
                                        _vp(info), len(shapes), Queue.current(cuda).handle)
    torch.cuda.synchronize()
    assert rc == 0
    P = ipiv.cpu().numpy()
    for k, (m, n) in enumerate(shapes):
        ref = mats[k].copy()
        rp, rinfo = oracle.dgetrf(ref, m)
        assert np.array_equal(A.view(k).cpu().numpy(), ref), k
        assert np.array_equal(P[offs[k]:offs[k] + min(m, n)], rp[:min(m, n)]), k


@pytest.mark.parametrize("trans", [False, True])
def test_getrs_vbatched(cuda, trans):
    rng = np.random.default_rng(11)
    ns = [5, 33, 100, 1, 64]
    nrhss = [2, 16, 7, 1, 20]
    LUs, Bs = _make(rng, ns, nrhss)
    pivs = []
    for k in range(len(ns)):
        p, _ = oracle.dgetrf(LUs[k])
        pivs.append(p)
    A = VBatch([a.shape for a in LUs], ns, torch.float64, cuda).load(LUs)
    B = VBatch([b.shape for b in Bs], ns, torch.float64, cuda).load(Bs)
    flat = np.concatenate(pivs).astype(np.int32)
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]])
    ipiv = torch.from_numpy(flat).to(cuda)
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=cuda) * 4
    rc = L.load().magma_dgetrs_vbatched(112 if trans else 111, _vp(A.ncols), _vp(B.ncols),
                                        _vp(A.ptrs), _vp(A.ld), _vp(dP), _vp(B.ptrs), _vp(B.ld),
                                        len(ns), Queue.current(cuda).handle)
    torch.cuda.synchronize()
    assert rc == 0
    for k in range(len(ns)):
        ref = Bs[k].copy()
        oracle.dgetrs(LUs[k], pivs[k], ref, trans=trans)
        assert np.array_equal(B.view(k).cpu().numpy(), ref), k


def test_gesv_vbatched_nocheck_work_in_cuda_graph(cuda):
    """The _max_nocheck_work entry enqueues without allocating or synchronising:
    captured once in a CUDA graph and replayed on fresh inputs."""
    rng = np.random.default_rng(3)
    ns = [int(n) for n in rng.integers(8, 257, 40)]
    nrhss = [int(r) for r in rng.integers(1, 17, 40)]
    As, Bs = _make(rng, ns, nrhss)
    A = VBatch([a.shape for a in As], ns, torch.float64, cuda)
    B = VBatch([b.shape for b in Bs], ns, torch.float64, cuda)
    tot = sum(ns)
    ipiv = torch.zeros((tot,), dtype=torch.int32, device=cuda)
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]])
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=cuda) * 4
    info = torch.empty((len(ns),), dtype=torch.int32, device=cuda)
    lib = L.load()
    lw = C.c_int(-1)
    lib.magma_dgesv_vbatched_max_nocheck_work(None, None, max(ns), max(nrhss), None, None, None,
                                              None, None, None, None, C.byref(lw), len(ns), None)
    work = torch.empty((lw.value,), dtype=torch.uint8, device=cuda)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        q = Queue(cuda.index, s.cuda_stream)
        # one eager call first (sets kernel attributes), then the capture
        rc = lib.magma_dgesv_vbatched_max_nocheck_work(
            _vp(A.ncols), _vp(B.ncols), max(ns), max(nrhss), _vp(A.ptrs), _vp(A.ld), _vp(dP),
            _vp(B.ptrs), _vp(B.ld), _vp(info), _vp(work), C.byref(lw), len(ns), q.handle)
        assert rc == 0
        s.synchronize()
        with torch.cuda.graph(g, stream=s):
            rc = lib.magma_dgesv_vbatched_max_nocheck_work(
                _vp(A.ncols), _vp(B.ncols), max(ns), max(nrhss), _vp(A.ptrs), _vp(A.ld), _vp(dP),
                _vp(B.ptrs), _vp(B.ld), _vp(info), _vp(work), C.byref(lw), len(ns), q.handle)
    assert rc == 0
    for rep in range(2):
        A.load(As)
        B.load(Bs)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        Ao = [A.view(k).cpu().numpy() for k in range(len(ns))]
        Bo = [B.view(k).cpu().numpy() for k in range(len(ns))]
        P = ipiv.cpu().numpy()
        pivs = [P[offs[k]:offs[k] + ns[k]] for k in range(len(ns))]
        _check_same((Ao, Bo, pivs, info.cpu().numpy()), As, Bs, ns, nrhss)


def test_vbatched_argument_errors(cuda):
    lib = L.load()
    q = Queue.current(cuda).handle
    n = torch.tensor([4, -1], dtype=torch.int32, device=cuda)
    r = torch.tensor([1, 1], dtype=torch.int32, device=cuda)
    ld = torch.tensor([4, 4], dtype=torch.int32, device=cuda)
    assert lib.magma_dgesv_vbatched(_vp(n), _vp(r), None, _vp(ld), None, None, _vp(ld), None, 2, q) == -1
    assert lib.magma_dgetrf_vbatched(_vp(ld), _vp(n), None, _vp(ld), None, None, 2, q) == -2
    n2 = torch.tensor([4, 8], dtype=torch.int32, device=cuda)
    assert lib.magma_dgesv_vbatched(_vp(n2), _vp(r), None, _vp(ld), None, None, _vp(n2), None, 2, q) == -4
    r2 = torch.tensor([1, -3], dtype=torch.int32, device=cuda)
    assert lib.magma_dgesv_vbatched(_vp(n2), _vp(r2), None, _vp(n2), None, None, _vp(n2), None, 2, q) == -2


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_every_tuning_choice_is_bit_exact(cuda, dtype):
    """Each (panel width, update tile) the tuner can choose, forced on every size bin, gives
    the oracle's factors, pivots and solutions bit for bit."""
    rng = np.random.default_rng(21)
    ns = [int(n) for n in rng.integers(1, 257, 24)] + [16, 17, 32, 33, 64, 65, 128, 129, 256]
    nrhss = [int(r) for r in rng.integers(1, 17, len(ns))]
    npdt = np.float64 if dtype == torch.float64 else np.float32
    As, Bs = _make(rng, ns, nrhss, ld_pad=1, dtype=npdt)
    saved = mg.vbatched_tuning(dtype)
    try:
        for nb in (8, 16, 32):
            for tile in range(3):
                mg.set_vbatched_tuning([nb] * 8, [tile] * 8, dtype)
                gpu = _gpu_gesv(As, Bs, ns, cuda, dtype)
                rA = [a.copy() for a in As]
                rB = [b.copy() for b in Bs]
                rp, rinfo = (oracle.dgesv_vbatched if dtype == torch.float64
                             else oracle.sgesv_vbatched)(ns, nrhss, rA, rB)
                Ao, Bo, pivs, info = gpu
                assert np.array_equal(info, rinfo), (nb, tile)
                for k in range(len(ns)):
                    assert np.array_equal(pivs[k], rp[k]), (nb, tile, k)
                    assert np.array_equal(Ao[k], rA[k], equal_nan=True), (nb, tile, k)
                    assert np.array_equal(Bo[k], rB[k], equal_nan=True), (nb, tile, k)
    finally:
        mg.set_vbatched_tuning([saved[b]["nb"] for b in mg.batched.TUNE_BINS],
                               [saved[b]["tile"] for b in mg.batched.TUNE_BINS], dtype)


def test_autotune_installs_a_valid_table(cuda):
    saved = mg.vbatched_tuning(torch.float64)
    try:
        t = mg.autotune_vbatched(96, torch.float64)
        assert t == mg.vbatched_tuning(torch.float64)
        for b in mg.batched.TUNE_BINS:
            assert t[b]["nb"] in (8, 16, 32) and t[b]["tile"] in mg.batched.TILES
        # bins above max_n keep their entries
        for b in ("<=256", "<=512", "<=1024", ">1024"):
            assert t[b] == saved[b]
        # results with the tuned table still match the oracle
        rng = np.random.default_rng(22)
        ns = [int(n) for n in rng.integers(1, 97, 20)]
        nrhss = [int(r) for r in rng.integers(1, 5, 20)]
        As, Bs = _make(rng, ns, nrhss)
        _check_same(_gpu_gesv(As, Bs, ns, cuda), As, Bs, ns, nrhss)
    finally:
        mg.set_vbatched_tuning([saved[b]["nb"] for b in mg.batched.TUNE_BINS],
                               [saved[b]["tile"] for b in mg.batched.TUNE_BINS], torch.float64)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_getrf_vbatched_large_blocked_path(cuda, dtype):
    """Batches with a matrix above 256 run the per-step kernels with per-matrix sizes:
    rectangular and square shapes from 1 to 1100, bit-exact with the oracle."""
    rng = np.random.default_rng(31)
    shapes = [(700, 300), (300, 700), (513, 513), (1, 900), (900, 1), (64, 64), (1100, 1000),
              (257, 256), (33, 40), (0, 5), (600, 600)]
    npdt = np.float64 if dtype == torch.float64 else np.float32
    ms = [m for m, _ in shapes]
    ns = [n for _, n in shapes]
    mats = [rng.uniform(-1, 1, (n, m + 3)).astype(npdt) for m, n in shapes]
    A = VBatch([a.shape for a in mats], ms, dtype, cuda).load(mats)
    mn = [max(min(m, n), 1) for m, n in shapes]
    ipiv = torch.zeros((sum(mn),), dtype=torch.int32, device=cuda)
    offs = np.concatenate([[0], np.cumsum(mn)[:-1]])
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=cuda) * 4
    info = torch.full((len(shapes),), -7, dtype=torch.int32, device=cuda)
    fn = L.load().magma_dgetrf_vbatched if dtype == torch.float64 else L.load().magma_sgetrf_vbatched
    rc = fn(_vp(A.rows), _vp(A.ncols), _vp(A.ptrs), _vp(A.ld), _vp(dP), _vp(info), len(shapes),
            Queue.current(cuda).handle)
    torch.cuda.synchronize()
    assert rc == 0
    P = ipiv.cpu().numpy()
    inf = info.cpu().numpy()
    for k, (m, n) in enumerate(shapes):
        ref = mats[k].copy()
        rp, rinfo = (oracle.dgetrf if dtype == torch.float64 else oracle.sgetrf)(ref, m)
        assert inf[k] == rinfo, k
        assert np.array_equal(A.view(k).cpu().numpy(), ref, equal_nan=True), k
        assert np.array_equal(P[offs[k]:offs[k] + min(m, n)], rp[:min(m, n)]), k
