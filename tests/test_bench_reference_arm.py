"""The bench's reference arm (CPU): one JSON line in the bench's own format,
timing the reference's code (or, without the unpacked reference, the numpy
port) on the GPU arm's job; under a multi-rank launch only rank 0 works."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CMD = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "box32_tiny",
       "--steps", "1", "--warmup", "1"]


def _run(env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    env["CUDA_VISIBLE_DEVICES"] = ""
    return subprocess.run(CMD, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_line_of_the_bench_format():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "candidates/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 1 and d["ms_per_step"] > 0
    assert d["config"]["box"] == 32 and d["config"]["particles"] == 24
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("reference", "port")
    assert cb["cpu_model"] and cb["nproc"] >= cb["cores"]
    assert d["e2e"] == {"value": d["value"], "unit": "candidates/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    spc = d["seconds_per_candidate"]
    # every particle of the tiny job is in the sample: nothing is extrapolated
    assert abs(spc["value"] - (spc["density_s"] + spc["templates_s"]
                               + spc["particles_s_per_particle"] * spc["particles"])) < 1e-9


@pytest.mark.parametrize("rank", ["1"])
def test_reference_arm_other_ranks_exit_without_work(rank):
    r = _run({"RANK": rank, "WORLD_SIZE": "2", "LOCAL_RANK": rank})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_cpu_baseline_block_of_the_gpu_line():
    """The cpu_baseline block the GPU arm's line carries (run here on a tiny
    job: the reference's own CPU path when unpacked, else the port)."""
    import bench
    from gisapr_gb300 import synthetic as syn
    spec, data = bench.make_workload("box32_tiny", 1, "cpu", 0)
    pose = syn.candidate_poses(1, 7, spec.pose_rotation_deg, spec.pose_translation, exact=True)[0]
    cb = bench.run_cpu_baseline(spec, data, pose, 8)
    assert cb["value"] > 0 and cb["unit"] == "candidates/s" and cb["kind"] in ("reference", "port")
    assert cb["cpu_model"] and cb["nproc"] >= 1 and cb["cores"] >= 1 and cb["sample"]
