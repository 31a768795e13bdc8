"""Seeded synthetic inputs for the batched LU workloads (numpy / torch).

The matrix families follow the reference tester's generators in kind
(testing/magma_generate.cpp): "rand" with entries uniform(-1,1) (larnv
idist=2 style), and the "svd" type A = U diag(s) V^T with U, V orthogonal
(here the Q factors of seeded Gaussian matrices) and s geometric from 1 down
to 1/kappa (magma_generate.cpp:133-135, 281-380).  Everything is generated
from an explicit seed so that runs are reproducible.
"""
from __future__ import annotations

import numpy as np


def uniform_batch(batch: int, m: int, n: int, seed: int, dtype=np.float64) -> np.ndarray:
    """(batch, m, n) entries i.i.d. uniform(-1, 1)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, size=(batch, m, n)).astype(dtype)


def colmajor_uniform(batch: int, n_cols: int, ld: int, m: int, seed: int,
                     dtype=np.float64) -> np.ndarray:
    """Column-major storage (batch, n_cols, ld) whose leading m rows are uniform(-1,1)
    and whose padding rows are zero."""
    rng = np.random.default_rng(seed)
    S = np.zeros((batch, n_cols, ld), dtype=dtype)
    S[:, :, :m] = rng.uniform(-1.0, 1.0, size=(batch, n_cols, m))
    return S


def svd_batch_torch(batch: int, n: int, kappas, seed: int, device="cuda"):
    """A = U diag(s) V^T (float64, math orientation, on `device`), s geometric
    from 1 to 1/kappa_k for matrix k; U, V = Q of seeded Gaussian matrices."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    kap = torch.as_tensor(np.asarray(kappas, dtype=np.float64))
    out = torch.empty((batch, n, n), dtype=torch.float64, device=device)
    chunk = 64
    # QR on the host (LAPACK through torch's CPU build): the same numbers on any
    # device, and no dependency on the GPU linear-algebra libraries
    for s in range(0, batch, chunk):
        e = min(batch, s + chunk)
        G1 = torch.randn((e - s, n, n), generator=g, dtype=torch.float64)
        G2 = torch.randn((e - s, n, n), generator=g, dtype=torch.float64)
        U, _ = torch.linalg.qr(G1)
        V, _ = torch.linalg.qr(G2)
        t = torch.linspace(0.0, 1.0, n, dtype=torch.float64)
        sig = torch.exp(-t[None, :] * torch.log(kap[s:e])[:, None])
        out[s:e] = ((U * sig[:, None, :]) @ V.transpose(1, 2)).to(device)
    return out
