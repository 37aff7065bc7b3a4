"""Launch-shape autotuner for batched scoring.

Four launch choices decide a batch's speed for a given box, crop, psi count
and particle set, and the best values depend on the GPU:

* the thread-block cluster size of the plain FP32 correlation (CTAs that
  split one particle's packed columns; each holds its columns of every psi
  spectrum in shared memory), 1..8;
* the candidates per tensor-core launch: a 128-row MMA tile holds
  128 // ceil8(candidates) whole directions, so the chunk size sets how many
  directions share a tile (the tile shape) and how many tiles a particle
  needs;
* the tensor-core kernel's shared-memory ring depths (A: bulk-copied
  template rows, B: built particle rows): deeper rings hide more copy
  latency but leave less of the SM's shared memory to its L1 cache;
* the template lanes of a batch (streams, each with its own native
  context, over which the slots' density, volume transform and projector
  launches are spread): one slot's short launches fill the tail of
  another's projector.

``Autotuner.tune`` times the batched correlation stage (CUDA events, best of
a few runs on the job's own data) for every valid value, keeps the fastest,
and caches the result per (GPU, size, crop, psi count, particle count
bucket, batch size) in a JSON file. The reference has no autotuner (its
launch shapes are fixed in the torch code); these choices change launch
shapes only, not the algorithm.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import asdict, dataclass, field
from pathlib import Path
from typing import Dict, Optional, Sequence

from . import _native as nat

__all__ = ["Autotuner", "TuneResult", "default_cache_path"]

CLUSTER_CHOICES = (1, 2, 3, 4, 5, 6, 8)
CHUNK_CHOICES = (16, 32, 64, 128)
RING_CHOICES = ((4, 2), (3, 2), (6, 2), (4, 3))  # (A, B) ring depths; the first is the kernel's default
LANE_CHOICES = (1, 2, 3)
SMEM_LIMIT = 227 * 1024


def default_cache_path() -> Path:
    env = os.environ.get("GISAPR_TUNING_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "gisapr_gb300" / "tuning.json"


def plain_smem_bytes(n: int, n_psi: int, crop: int, cluster: int) -> int:
    """Shared memory of one CTA of the plain correlation (matches the kernel's carve-up)."""
    h = n // 2 + 1
    cw = -(-h // cluster)
    k_group, k_local = 4, 16
    return (n_psi * n * cw * 8 + k_group * n_psi * crop * cw * 8 + (n // 16) * crop * 8 + cw * crop * 8
            + k_local * n_psi * crop * crop * 4)


@dataclass
class TuneResult:
    key: str
    size: int
    corr_cluster: int
    tc_chunk: int
    times_ms: Dict[str, float] = field(default_factory=dict)
    tc_a_stages: int = 0  # 0: the kernel's default
    tc_b_stages: int = 0
    dirs_per_tile: int = 0
    template_lanes: int = 2

    def apply(self) -> None:
        """Make the cluster size and the ring depths the defaults of every
        native context at this size."""
        nat.set_default_tuning(nat.TUNE_CORR_CLUSTER, self.size, self.corr_cluster)
        nat.set_default_tuning(nat.TUNE_TC_A_STAGES, self.size, self.tc_a_stages)
        nat.set_default_tuning(nat.TUNE_TC_B_STAGES, self.size, self.tc_b_stages)


class Autotuner:
    def __init__(self, cache_path: Optional[os.PathLike] = None, trials: int = 2):
        self.cache_path = Path(cache_path) if cache_path else default_cache_path()
        self.trials = int(trials)

    @staticmethod
    def key(job, n_cand: int) -> str:
        import torch
        name = torch.cuda.get_device_name(job.device).replace("|", "/")
        bucket = 2 ** int(round(math.log2(max(1, len(job.records)))))
        return f"{name}|n={job.cfg.new_box}|crop={job.cfg.crop}|psi={job.n_psi}|particles~{bucket}|cand={n_cand}"

    def _load(self) -> dict:
        try:
            return json.loads(self.cache_path.read_text())
        except (OSError, ValueError):
            return {}

    def _save(self, key: str, entry: dict) -> None:
        """Add one entry to the cache file. Under an exclusive lock on a
        side file it re-reads the cache, so entries that other processes
        (replicas tuning at the same time) wrote are kept, and replaces it
        through a temporary file of this process."""
        import fcntl
        import tempfile
        try:
            self.cache_path.parent.mkdir(parents=True, exist_ok=True)
            with open(str(self.cache_path) + ".lock", "w") as lock:
                fcntl.flock(lock, fcntl.LOCK_EX)
                data = self._load()
                data[key] = entry
                fd, tmp = tempfile.mkstemp(dir=self.cache_path.parent, prefix=self.cache_path.name, suffix=".tmp")
                try:
                    with os.fdopen(fd, "w") as fh:
                        fh.write(json.dumps(data, indent=1, sort_keys=True))
                    os.replace(tmp, self.cache_path)
                except OSError:
                    os.unlink(tmp)
                    raise
        except OSError:
            pass  # a read-only home only loses the cache

    def _time_correlate(self, job, n_cand: int, precision: str, poses, tc_chunk: int = 128) -> float:
        from .engine import BatchScoringJob
        bj = BatchScoringJob(job, n_cand, use_graph=False, precision=precision, tc_chunk=tc_chunk)
        bj.stage_ms(poses)  # warm-up: plans, tables, launch attributes
        best = min(bj.stage_ms(poses)["correlate"] for _ in range(self.trials))
        bj.check_status()
        del bj
        return best

    def _time_templates(self, job, n_cand: int, poses, lanes: int) -> float:
        from .engine import BatchScoringJob
        bj = BatchScoringJob(job, n_cand, use_graph=False, lanes=lanes)
        bj.stage_ms(poses)  # warm-up: the lanes' contexts grow their scratch
        best = min(bj.stage_ms(poses)["templates"] for _ in range(self.trials))
        del bj
        return best

    def tune(self, job, n_cand: int = 64, precision: str = "fp16x3", force: bool = False,
             clusters: Sequence[int] = CLUSTER_CHOICES, chunks: Sequence[int] = CHUNK_CHOICES,
             rings: Sequence = RING_CHOICES, lanes: Sequence[int] = LANE_CHOICES) -> TuneResult:
        """Pick the cluster size (plain path) and, unless precision is
        "fp32", the tensor-core chunk size (hence directions per tile) and ring
        depths for batches of n_cand candidates."""
        from . import synthetic as syn
        key = self.key(job, n_cand) + f"|{precision}"
        cache = self._load()
        if not force and key in cache:
            r = TuneResult(**cache[key])
            r.apply()
            return r
        poses = list(syn.candidate_poses(n_cand, 1234, 5.0, 3.0))
        nb, crop, n_psi = job.cfg.new_box, job.cfg.crop, job.n_psi
        times: Dict[str, float] = {}
        best_k, best_t = 0, math.inf
        ctx = nat.Context.for_device(job.device)
        for k in clusters:
            if plain_smem_bytes(nb, n_psi, crop, k) > SMEM_LIMIT or k > nb // 2 + 1:
                continue
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_CORR_CLUSTER, nb, k)
            t = self._time_correlate(job, n_cand, "fp32", poses)
            times[f"plain_cluster_{k}"] = t
            if t < best_t:
                best_k, best_t = k, t
        nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_CORR_CLUSTER, nb, best_k)
        best_c = min(128, n_cand)
        if precision != "fp32":
            best_ct = math.inf
            for c in sorted({c for c in chunks if c < n_cand} | {min(n_cand, 128)}):
                t = self._time_correlate(job, n_cand, precision, poses, tc_chunk=c)
                times[f"tc_chunk_{c}"] = t
                if t < best_ct:
                    best_c, best_ct = c, t
        best_ring = (0, 0)
        if precision != "fp32":
            best_rt = math.inf
            for sa, sb in rings:
                nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_A_STAGES, nb, sa)
                nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_B_STAGES, nb, sb)
                t = self._time_correlate(job, n_cand, precision, poses, tc_chunk=best_c)
                times[f"tc_rings_{sa}_{sb}"] = t
                if t < best_rt:
                    best_ring, best_rt = (sa, sb), t
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_A_STAGES, nb, best_ring[0])
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_B_STAGES, nb, best_ring[1])
        dpt = 128 // ((min(best_c, 128) + 7) // 8 * 8)
        best_l, best_lt = 1, math.inf
        for n_l in lanes:
            if n_l > n_cand:
                continue
            t = self._time_templates(job, n_cand, poses, n_l)
            times[f"template_lanes_{n_l}"] = t
            if t < best_lt:
                best_l, best_lt = n_l, t
        r = TuneResult(key=key, size=nb, corr_cluster=best_k, tc_chunk=best_c, times_ms=times,
                       tc_a_stages=best_ring[0], tc_b_stages=best_ring[1], dirs_per_tile=dpt,
                       template_lanes=best_l)
        self._save(key, asdict(r))
        r.apply()
        return r
