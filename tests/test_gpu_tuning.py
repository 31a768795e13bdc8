"""The fixed-size tuning table on the GPU: every setting of every entry factors bit for
bit like the oracle (tuning changes only the time), and the autotuner installs a valid
table."""
import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from tests.util import to_storage

pytestmark = pytest.mark.gpu


@pytest.fixture
def keep_tables():
    saved = {dt: mg.getrf_batched_tuning(dt) for dt in (torch.float32, torch.float64)}
    yield
    for dt, t in saved.items():
        mg.set_getrf_batched_tuning([v["two_level"] for v in t.values()],
                                    [v["band_ctas"] for v in t.values()],
                                    [v["tile64"] for v in t.values()], dt)


@pytest.mark.parametrize("two_level", [0, 1])
@pytest.mark.parametrize("band", [1, 2, 4])
def test_every_fp32_setting_is_bit_exact(cuda, keep_tables, two_level, band):
    mg.set_getrf_batched_tuning([two_level] * 6, [band] * 6, [1] * 6, torch.float32)
    rng = np.random.default_rng(band * 10 + two_level)
    for m, n, b in ((300, 300, 320), (200, 520, 24)):
        S = to_storage(rng.uniform(-1, 1, (b, m, n)).astype(np.float32))
        rS = S.copy()
        ripiv, rinfo = oracle.sgetrf_batched(rS, m)
        dS = torch.from_numpy(S).to(cuda)
        ipiv, info = mg.getrf_batched(dS, m)
        torch.cuda.synchronize()
        assert np.array_equal(ipiv.cpu().numpy()[:, :min(m, n)], ripiv[:, :min(m, n)])
        assert np.array_equal(dS.cpu().numpy(), rS)


@pytest.mark.parametrize("tile64", [0, 1])
def test_every_fp64_setting_is_bit_exact(cuda, keep_tables, tile64):
    mg.set_getrf_batched_tuning([1] * 6, [2] * 6, [tile64] * 6, torch.float64)
    rng = np.random.default_rng(tile64)
    S = to_storage(rng.uniform(-1, 1, (6, 200, 200)))
    rS = S.copy()
    ripiv, _ = oracle.dgetrf_batched(rS)
    dS = torch.from_numpy(S).to(cuda)
    ipiv, _ = mg.getrf_batched(dS)
    torch.cuda.synchronize()
    assert np.array_equal(ipiv.cpu().numpy(), ripiv)
    assert np.array_equal(dS.cpu().numpy(), rS)


def test_autotuner_installs_a_valid_table(cuda, keep_tables):
    for dt in (torch.float32, torch.float64):
        t = mg.autotune_getrf_batched(300, 64, dt)
        for b in ("<=64", "<=128", "<=256", "<=512"):
            assert t[b]["two_level"] in (0, 1)
            assert t[b]["band_ctas"] in (1, 2, 4)
            assert t[b]["tile64"] in (0, 1)
