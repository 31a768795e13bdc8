"""The tuning tables and their JSON file, on the host (no GPU): set / get, save / load
round trip, a malformed file refused without changing anything, and the file named by
MAGMA_LU_TUNING_FILE loaded when a queue is created."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _mg():
    import magma_gb300 as mg
    mg.lib.load()
    return mg


def test_fixed_table_set_get_and_argument_errors():
    mg = _mg()
    import torch
    old = mg.getrf_batched_tuning(torch.float32)
    try:
        mg.set_getrf_batched_tuning([1, 0, 1, 0, 1, 0], [1, 2, 4, 1, 2, 4], [1] * 6, torch.float32)
        t = mg.getrf_batched_tuning(torch.float32)
        assert [v["two_level"] for v in t.values()] == [1, 0, 1, 0, 1, 0]
        assert [v["band_ctas"] for v in t.values()] == [1, 2, 4, 1, 2, 4]
        with pytest.raises(RuntimeError, match="-2"):
            mg.set_getrf_batched_tuning([1] * 6, [3] * 6, [1] * 6, torch.float32)
    finally:
        mg.set_getrf_batched_tuning([v["two_level"] for v in old.values()],
                                    [v["band_ctas"] for v in old.values()],
                                    [v["tile64"] for v in old.values()], torch.float32)


def test_save_load_round_trip(tmp_path):
    mg = _mg()
    import torch
    f32, f64 = mg.getrf_batched_tuning(torch.float32), mg.getrf_batched_tuning(torch.float64)
    v64 = mg.vbatched_tuning(torch.float64)
    try:
        mg.set_getrf_batched_tuning([0, 1, 0, 1, 0, 1], [4, 4, 2, 2, 1, 1], [1] * 6, torch.float32)
        mg.set_getrf_batched_tuning([1] * 6, [2] * 6, [0, 1, 0, 1, 0, 1], torch.float64)
        p = tmp_path / "tuning.json"
        mg.save_tuning(p)
        d = json.loads(p.read_text())                       # valid JSON
        assert d["format"] == "magma_lu tuning 1"
        assert d["getrf_batched"]["s"]["two_level"] == [0, 1, 0, 1, 0, 1]
        assert d["getrf_batched"]["d"]["tile64"] == [0, 1, 0, 1, 0, 1]
        assert len(d["getrf_vbatched"]["d"]["nb"]) == 8
        mg.set_getrf_batched_tuning([1] * 6, [2] * 6, [1] * 6, torch.float32)
        mg.load_tuning(p)
        assert [v["two_level"] for v in mg.getrf_batched_tuning(torch.float32).values()] == [0, 1, 0, 1, 0, 1]
        assert [v["tile64"] for v in mg.getrf_batched_tuning(torch.float64).values()] == [0, 1, 0, 1, 0, 1]
        # a malformed file is refused and changes nothing
        bad = dict(d)
        bad["getrf_batched"] = dict(d["getrf_batched"])
        bad["getrf_batched"]["s"] = dict(d["getrf_batched"]["s"], band_ctas=[3] * 6)
        q = tmp_path / "bad.json"
        q.write_text(json.dumps(bad))
        with pytest.raises(RuntimeError):
            mg.load_tuning(q)
        assert [v["two_level"] for v in mg.getrf_batched_tuning(torch.float32).values()] == [0, 1, 0, 1, 0, 1]
        with pytest.raises(RuntimeError):
            mg.load_tuning(tmp_path / "missing.json")
    finally:
        for dt, t in ((torch.float32, f32), (torch.float64, f64)):
            mg.set_getrf_batched_tuning([v["two_level"] for v in t.values()],
                                        [v["band_ctas"] for v in t.values()],
                                        [v["tile64"] for v in t.values()], dt)
        mg.set_vbatched_tuning([v["nb"] for v in v64.values()], [v["tile"] for v in v64.values()],
                               torch.float64)


def test_queue_creation_loads_the_environment_file(tmp_path):
    mg = _mg()
    import torch
    old = mg.getrf_batched_tuning(torch.float32)
    try:
        mg.set_getrf_batched_tuning([0] * 6, [4] * 6, [1] * 6, torch.float32)
        p = tmp_path / "env.json"
        mg.save_tuning(p)
    finally:
        mg.set_getrf_batched_tuning([v["two_level"] for v in old.values()],
                                    [v["band_ctas"] for v in old.values()],
                                    [v["tile64"] for v in old.values()], torch.float32)
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import torch, magma_gb300 as mg\n"
            "mg.lib.load()\n"
            "before = mg.getrf_batched_tuning(torch.float32)['<=512']['band_ctas']\n"
            "q = mg.Queue(0, 0)\n"
            "after = mg.getrf_batched_tuning(torch.float32)['<=512']\n"
            "print(before, after['band_ctas'], after['two_level'])\n") % str(ROOT)
    env = dict(os.environ, MAGMA_LU_TUNING_FILE=str(p))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.split() == ["2", "4", "0"]
