"""Benchmark: candidate poses scored per second, box 128 / 5,000 particles.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (seeded synthetic data of the reference's published shapes): a
3,000-atom moving chain over a 20,000-atom fixed context, box 128 at
1.1 A/px, 5,000 particles (CTF, SNR 0.05), HEALPix order 3 directions
(768) searched +-10 deg, psi step 7.5 deg, translations +-5 px (crop 12),
logistic FSC. One step scores one candidate pose (a 3 deg / 1.5 A rigid
perturbation of the moving chain) end to end: splat, 3-D FFT, templates of
every needed direction, correlation of every particle, records, score.

The GB300 arm times K steps with CUDA events on the launching stream (job
tables and particle spectra resident in HBM, the 1.0 GB particle stack is
read every step, so inputs exceed L2), then the same K poses through the
public API with the pose copied host->device and the score plus the
per-particle peaks copied back each step (``e2e``). The reference arm
(``--impl reference``) runs GisAPR's own CPU torch path, installed
unmodified in baseline/_ref by baseline/install_reference.py, on the same job
and poses (each step one pose with a particle sample, the candidate rate
extrapolated over particles); without baseline/_ref it falls back to the
numpy restatement of that path and says so.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "candidates scored/s @box128·5k ptcl vs plain FP32 GPU; p50/p99 latency"
UNIT = "candidates/s"
L2_BYTES = 129e6  # GB300 L2 (126 MiB)


def l2_note(stack_bytes: float) -> str:
    """How the timed steps stand to L2: the particle stack is read in full
    every step."""
    if stack_bytes > L2_BYTES:
        return f"inputs larger than L2: the {stack_bytes / 1e9:.2f} GB particle stack is read every step"
    return f"inputs within L2: the {stack_bytes / 1e6:.0f} MB particle stack (reduced particle count)"


# FP32 CUDA-core rate of one GB300 at its maximum SM clock (152 SMs x 128
# lanes x 2 flop per FMA x 2.07 GHz), the ceiling of the plain correlation
FP32_CORE_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--workload", default="box128_5kp")
    ap.add_argument("--particles", type=int, default=0, help="override the particle count (tests only)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=400, help="particles and templates in the CPU sample")
    ap.add_argument("--batch", type=int, default=64, help="candidates per batched generation (0: skip)")
    ap.add_argument("--reference-cuda-sample", type=int, default=500,
                    help="particles of the reference's own torch CUDA path timed beside this one (0: skip)")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes (no tuning runs)")
    ap.add_argument("--precision-particles", type=int, default=4000,
                    help="particles of the box-256 precision comparison (0: skip it; 20000 is the full "
                         "configuration, about three minutes of synthetic-data generation)")
    ap.add_argument("--precision-fp64", type=int, default=100,
                    help="particles of the precision comparison also evaluated in FP64 (torch float64 on the GPU)")
    ap.add_argument("--serve-requests", type=int, default=40,
                    help="requests in the serving stream (0: skip the serving measurement)")
    ap.add_argument("--precisions", default="fp32,fp16x3,fp16",
                    help="batched correlation forms to time: fp32 (plain), fp16x3 (tensor-core split), fp16")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons every INTERVAL_MS
    while the run's timed regions execute. ``start`` returns once sampling
    is live; ``begin``/``end`` bracket each timed region (called after a
    device synchronize on both sides); ``stop`` keeps the samples whose
    timestamps fall inside a region. A region shorter than the interval may
    hold none: if no region holds any, the samples within two intervals
    after each region stand in for it."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
    INTERVAL_MS = 50

    def __init__(self, gpu_index: int, exe: str = "nvidia-smi"):
        self.gpu = gpu_index
        self.exe = exe
        self.proc = None
        self.path = None
        self.windows = []  # (t0, t1) host wall-clock seconds of each timed region
        self._t0 = None

    def start(self, wait_s: float = 5.0):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            with open(self.path, "w") as out:
                self.proc = subprocess.Popen([self.exe, "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                              "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                             stdout=out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        import atexit
        atexit.register(self._terminate)
        deadline = time.time() + wait_s
        while time.time() < deadline and self.proc.poll() is None and os.path.getsize(self.path) == 0:
            time.sleep(0.01)

    def begin(self):
        self._t0 = time.time()

    def end(self):
        if self._t0 is not None:
            self.windows.append((self._t0, time.time()))
        self._t0 = None

    def _terminate(self):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    @staticmethod
    def _when(stamp: str):
        import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.datetime.strptime(stamp, fmt).timestamp()
            except ValueError:
                pass
        return None

    def _samples(self):
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm, smax = float(parts[2]), float(parts[3])
            except ValueError:
                continue
            active = {nm for nm, v in zip(self.REASONS, parts[6:10]) if v.lower() == "active"}
            rows.append((self._when(parts[0]), sm, smax, active))
        return rows

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self._terminate()
        rows = self._samples()
        os.unlink(self.path)
        dt = self.INTERVAL_MS / 1e3
        if rows and all(r[0] is not None for r in rows) and self.windows:
            inside = [r for r in rows if any(t0 <= r[0] <= t1 for t0, t1 in self.windows)]
            span = "samples inside the timed regions"
            if not inside:
                inside = [r for r in rows if any(t1 < r[0] <= t1 + 2 * dt for _, t1 in self.windows)]
                span = "no sample inside the timed regions: the samples within two intervals after each"
        else:
            inside, span = rows, "timestamps unavailable: every sample of the run"
        sm = [r[1] for r in inside]
        reasons = set().union(*(r[3] for r in inside)) if inside else set()
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(r[2] for r in inside) if inside else None,
                "reasons": sorted(reasons), "samples": len(sm), "interval_ms": self.INTERVAL_MS,
                "regions": len(self.windows), "span": span}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

BATCH_CHAINS = (1500, 3000, 6000)  # moving-chain sizes mixed in a batched generation


def make_workload(name: str, seed: int, device: str, particles: int = 0, with_models: bool = False):
    """Seeded job data; with_models also returns moving-chain variants of
    1,500 / 3,000 / 6,000 atoms sharing the job's fixed context (the job's
    particles come from the 3,000-atom model)."""
    from gisapr_gb300 import synthetic as syn
    spec = syn.WORKLOADS[name]
    if not with_models:
        job = syn.make_job(spec, seed=seed, device=device, n_particles=particles or None)
        return spec, job
    models = syn.make_models_shared_fixed(BATCH_CHAINS, spec.n_fixed_atoms, seed)
    job = syn.make_job(spec, seed=seed, device=device, n_particles=particles or None, model=models[1])
    return spec, job, models


def job_records(job):
    from gisapr_gb300.tables import ParticleRecord
    r = job.records
    return [ParticleRecord(int(r.line_index[i]), f"{i + 1}@particles.mrcs", float(r.rot[i]), float(r.tilt[i]),
                           float(r.psi[i]), float(r.defocus_u[i]), float(r.defocus_v[i]),
                           float(r.defocus_angle[i])) for i in range(len(r.rot))]


def run_batched(job, dens, gen, precision, n_batch, K, W, device, barrier, tc_chunk=128, lanes=2, clocks=None):
    """Time K graph-replayed generations of n_batch candidates (device events on
    the batch stream), then K end-to-end generations (poses from the host,
    scores and per-particle peaks back). ``clocks`` (a running ClockSampler)
    gets both timed regions."""
    import torch
    from gisapr_gb300.engine import BatchScoringJob
    model_of = [i % len(dens) for i in range(n_batch)]
    bj = BatchScoringJob(job, n_batch, models=dens, model_of=model_of, precision=precision,
                         tc_chunk=min(tc_chunk, 128), lanes=lanes)
    for k in range(W):
        bj.score_batch(gen[k])
    barrier()
    torch.cuda.synchronize(device)
    if clocks is not None:
        clocks.begin()
    b0 = torch.cuda.Event(enable_timing=True)
    b1 = torch.cuda.Event(enable_timing=True)
    b_steps = []
    with torch.cuda.stream(bj.stream):
        b0.record()
        for k in range(K):
            bj.set_poses(gen[W + k])
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            b_steps.append(ev)
            bj.run()
        b1.record()
    torch.cuda.synchronize(device)
    if clocks is not None:
        clocks.end()
    barrier()
    bj.check_status()
    b_elapsed = b0.elapsed_time(b1) / 1e3
    b_steps.append(b1)
    b_lat = sorted(b_steps[i].elapsed_time(b_steps[i + 1]) for i in range(K))
    bpeaks_host = torch.empty(tuple(bj.peak.shape), dtype=torch.float32).pin_memory()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    if clocks is not None:
        clocks.begin()
    e2.record()
    for k in range(K):
        bj.score_batch(gen[W + k])
        bpeaks_host.copy_(bj.peak, non_blocking=True)
    e3.record()
    torch.cuda.synchronize(device)
    if clocks is not None:
        clocks.end()
    b_e2e = e2.elapsed_time(e3) / 1e3
    stages = bj.stage_ms(gen[W])
    extra = {}
    if precision != "fp32":
        # tensor pipe: MMA flops the generation issues over the correlation
        # stage's device time (the stage also holds the operand copy of the banks)
        _, bf16_peak, peak_kind = load_peaks()
        flops = bj.tc_mma_flops()
        ach = flops / (stages["correlate"] / 1e3) / 1e12
        extra["roofline"] = {
            "kernel": "correlate_tc", "bound": "tensor", "achieved": ach, "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": ach / bf16_peak, "traffic": None,
            "peak_source": f"{peak_kind} bf16 dense (MEASURED_PEAKS.json)" if peak_kind == "measured" else "fallback",
            "algorithmic": f"{flops:.4g} MMA flop issued per generation (M=128, K=16 MMAs of every work item, "
                           f"padding rows included) over the correlation stage",
            "stage_ms": stages["correlate"]}
    return {"candidates_per_step": n_batch, "precision": precision, **extra,
            "moving_chain_atoms": [m.n_moving for m in dens],
            "graph": bj.graph is not None, "ms_per_step": b_elapsed / K * 1e3,
            "latency_ms": {"p50": b_lat[len(b_lat) // 2],
                           "p99": b_lat[min(len(b_lat) - 1, int(math.ceil(0.99 * len(b_lat))) - 1)]},
            "stage_ms": stages,
            "elapsed_s": b_elapsed, "e2e_elapsed_s": b_e2e, "e2e_h2d_bytes_per_step": 12 * 8 * n_batch,
            "e2e_d2h_bytes_per_step": 8 * n_batch + 4 * n_batch * len(job.records),
            "gpu_launches": bj.launches_per_batch() * K}


def cpu_baseline(spec, job, pose, sample: int):
    from oracle.cpu_baseline import time_candidate
    r = job.records
    out = time_candidate(job.model.pdb_text, pose, spec.box, spec.apix, spec.res, job.model_rot, job.model_tilt,
                         job.images, r, job.fsc, spec.mask_radius, spec.mask_edge, spec.psi_step,
                         spec.local_range, spec.crop, kk=spec.kk, n_template_sample=sample,
                         n_particle_sample=sample)
    return out


def correlation_flops(n: int, maps: int) -> float:
    """Algorithmic flops of the plain correlation: M * (6K + 2.5 n^2 log2 n^2)."""
    K = n * (n // 2 + 1)
    return maps * (6.0 * K + 2.5 * n * n * math.log2(n * n))


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of ``kernel`` from the committed ncu summary, at
    the workload's own particle count (a run with another count has none)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return d.get(workload, {}).get(kernel)
    except (ValueError, OSError):
        return None


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

REF_PARTICLE_SAMPLE = 200  # particles the reference arm runs per step, evenly spaced over the job


def gb300_config(spec) -> dict:
    """The workload both arms run (the reference's published shapes)."""
    return {"workload": f"{spec.name}: box {spec.box} at {spec.apix} A/px, {spec.n_particles} particles, "
                        f"{spec.n_moving_atoms} moving + {spec.n_fixed_atoms} fixed atoms, HEALPix order "
                        f"{spec.healpix_order} within +-{spec.local_range} deg, psi step {spec.psi_step} deg, "
                        f"crop {spec.crop}; one candidate pose per step",
            "box": spec.box, "apix": spec.apix, "particles": spec.n_particles, "moving_atoms": spec.n_moving_atoms,
            "fixed_atoms": spec.n_fixed_atoms, "healpix_order": spec.healpix_order,
            "local_range_deg": spec.local_range, "psi_step_deg": spec.psi_step, "crop": spec.crop,
            "candidates_per_step": 1}


def reference_job(args):
    """The GPU arm's own rank-0 job (same seeds, same model, same particles)
    and its poses, generated on the GPU when there is one (data generation
    is not timed)."""
    import torch
    from gisapr_gb300 import synthetic as syn
    from gisapr_gb300.replicas import replica_seed
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    spec, data, _ = make_workload(args.workload, replica_seed(args.seed, 0), dev, args.particles, with_models=True)
    poses = syn.candidate_poses(args.steps + args.warmup, args.seed + 100, spec.pose_rotation_deg,
                                spec.pose_translation, exact=True)
    return spec, data, poses


def run_reference(args):
    """GisAPR's own CPU path (baseline/reference_runner.py, from baseline/_ref) on
    the GPU arm's job and poses. Each step scores one candidate pose:
    density of every atom, every template of the angle table, and the
    reference's per-particle loop over an evenly spaced sample of the
    job's particles. ms_per_step is that measured work; the candidate rate
    extrapolates the per-particle time to every particle of the job (the
    loop is linear in particles). Without baseline/_ref the numpy port of
    the same path (the oracle) stands in and the line says so."""
    import numpy as np
    from baseline import reference_runner as ref_runner
    spec, data, poses = reference_job(args)
    n_p = len(data.records.rot)
    sample = np.unique(np.linspace(0, n_p - 1, min(REF_PARTICLE_SAMPLE, n_p)).astype(int)).tolist()
    if ref_runner.available():
        runner = ref_runner.RefRunner(data)
        kind, dtype = "reference", "f32"
        step = lambda pose: runner.step(pose, sample)  # noqa: E731
        threads = runner.threads
        what = ("GisAPR's own CPU torch path (optimized-3 tree: pdb2mrc v3 generate_volume, v606 "
                "IntegratedProjector.build_templates over all directions, PackedCTFTorch, per-particle "
                "prepare / correlate_templates_and_particle / make_result_records)")
    else:
        kind, dtype = "port", "f64"
        threads = os.cpu_count() or 1

        def step(pose):
            info = cpu_baseline(spec, data, pose, len(sample))
            return {"density_s": info["density_s"] + info["volume_fft_s"],
                    "templates_s": info["template_s"] * info["n_templates"],
                    "particles_s": info["particle_s"] * len(sample), "n_templates": info["n_templates"]}
        what = "numpy restatement of the reference's CPU path (oracle), baseline/_ref not installed"
    per, meas = [], []
    info = None
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        info = step(poses[k])
        dt = time.perf_counter() - t0
        full = info["density_s"] + info["templates_s"] + info["particles_s"] * n_p / len(sample)
        if k >= args.warmup:
            per.append(full)
            meas.append(dt)
    sec = statistics.mean(per)
    value = 1.0 / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(meas) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": gb300_config(spec),
        "seconds_per_candidate": {"value": sec, "density_s": info["density_s"],
                                  "templates_s": info["templates_s"],
                                  "particles_s_per_particle": info["particles_s"] / len(sample),
                                  "templates": int(info["n_templates"]), "particles": n_p,
                                  "note": f"each step runs {len(sample)} of the {n_p} particles; the candidate "
                                          f"rate extrapolates the per-particle time to all {n_p}"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": int(threads), "kind": kind, **host_cpu(),
                         "sample": f"{what}; per step one pose: density, {int(info['n_templates'])} templates "
                                   f"and {len(sample)} of {n_p} particles, particle time scaled to all {n_p}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def fp64_maxima(bank, stack, ptr, idx, n_part, crop):
    """FP64 maxima of the crop-window maps of the first ``n_part`` particles
    (torch float64 on the GPU): raw(y, x) = sum_{r,c} w_c Re[T P e^{2 pi i
    (r y + c x)/n}] on the stored (pre-shifted) arrays, w_c = 1 for c in
    {0, n/2} else 2 (the closed form of the reference's crop-window irfft2,
    v606:1437-1449), score = 1024 max raw, first maximum in row-major crop
    order. Returns per particle (scores [d, n_psi], y, x) or None."""
    import torch
    n, h = stack.shape[-2], stack.shape[-1]
    dev = stack.device
    off = torch.arange(crop, device=dev, dtype=torch.float64) - crop // 2
    ey = torch.exp(2j * math.pi * torch.outer(torch.arange(n, device=dev, dtype=torch.float64), off) / n)
    w = torch.full((h,), 2.0, dtype=torch.float64, device=dev)
    w[0] = 1.0
    w[n // 2] = 1.0
    ex = w[:, None] * torch.exp(2j * math.pi * torch.outer(torch.arange(h, device=dev, dtype=torch.float64), off) / n)
    out = []
    for i in range(n_part):
        a, b = int(ptr[i]), int(ptr[i + 1])
        if b <= a:
            out.append(None)
            continue
        t = bank[idx[a:b]].to(torch.complex128)                     # [d, n, h]
        pp = stack[i].to(torch.complex128)                           # [n_psi, n, h]
        q = t[:, None] * pp[None]                                    # [d, n_psi, n, h]
        z = torch.einsum("ry,abrc->abyc", ey, q)
        raw = torch.einsum("abyc,cx->abyx", z, ex).real.reshape(b - a, pp.shape[0], -1)
        k = torch.argmax(raw, dim=-1)
        best = torch.gather(raw, -1, k[..., None])[..., 0] * 1024.0
        out.append((best.cpu().numpy(), (k // crop).cpu().numpy(), (k % crop).cpu().numpy()))
    return out


def run_precision(args, device):
    """Box-256 precision configuration (crop 14, psi step 3.75, local 6 deg)
    on a particle set: every tensor-core form against the plain FP32 batched
    path (all particles) and against an FP64 evaluation of the same
    contraction on the same templates and particle spectra (the first
    ``args.precision_fp64`` particles): per candidate score and per particle
    argmax (direction, psi, shift), identical or tied within 1e-5 of the
    FP64 maxima."""
    import numpy as np
    from gisapr_gb300 import synthetic as syn
    from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob
    from gisapr_gb300.tables import model_angles_from_lists
    spec = syn.WORKLOADS["box256_20kp"]
    n_part = args.precision_particles
    data = syn.make_job(spec, seed=args.seed + 77, device=str(device), n_particles=n_part)
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                    local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                     job_records(data), data.images, fsc_values=data.fsc, device=device)
    poses = list(syn.candidate_poses(8, args.seed + 78, 5.0, 3.0))
    n64 = min(n_part, args.precision_fp64)
    ptr = job.local_ptr.cpu().numpy()
    idx = job.local_idx.cpu().numpy()
    n_psi = job.n_psi
    forms = ("fp32", "fp16x3", "bf16x3", "fp16", "bf16")
    runs, ref64 = {}, None
    for prec in forms:
        bj = BatchScoringJob(job, len(poses), use_graph=False, precision=prec)
        scores = bj.score_active(poses)
        runs[prec] = (scores, bj.score_buf.cpu().numpy(),
                      np.stack([t.cpu().numpy() for t in (bj.best_entry, bj.best_psi, bj.peak_y, bj.peak_x)], -1),
                      bj.stage_ms(poses)["correlate"], bj.peak.cpu().numpy())
        if prec == "fp32" and n64 > 0:
            # the same float32 templates and spectra feed every form
            ref64 = [fp64_maxima(bj.banks[c], job.stack, ptr, idx, n64, cfg.crop) for c in range(len(poses))]
        del bj
    ref_scores, ref_maps, ref_arg, _, _ = runs["fp32"]
    out = {"workload": f"box256_20kp shapes, {n_part} particles, {len(poses)} candidates",
           "box": spec.box, "crop": spec.crop, "directions": len(data.model_rot),
           "maps_per_candidate": job.nnz * job.n_psi,
           "fp64": f"torch float64 on the GPU, first {n64} particles, same templates and particle spectra"}
    for prec in forms:
        sc, maps, arg, ms, peak = runs[prec]
        entry = {"correlate_ms": ms, "plain_correlate_ms": runs["fp32"][3]}
        if prec != "fp32":
            valid = ref_arg[..., 0] >= 0
            agree = np.all(arg == ref_arg, axis=-1)[valid]
            entry.update({"score_max_rel_err_vs_fp32": float(np.max(np.abs(sc / ref_scores - 1.0))),
                          "map_max_err_rel_to_scale": float(np.max(np.abs(maps - ref_maps)) / np.max(np.abs(ref_maps))),
                          "argmax_agreement_vs_fp32": float(np.mean(agree))})
        if ref64 is not None:
            worst, hits, total = 0.0, 0, 0
            for c in range(len(poses)):
                want = got = 0.0
                for i in range(n64):
                    r = ref64[c][i]
                    if r is None:
                        continue
                    s64, y64, x64 = r
                    k = int(np.argmax(s64.reshape(-1)))
                    want += math.exp(float(s64.reshape(-1)[k]) / 1024.0)
                    got += math.exp(float(peak[c][i]) / 1024.0)
                    mine = int(arg[c, i, 0] - ptr[i]) * n_psi + int(arg[c, i, 1])
                    hit = mine == k and int(arg[c, i, 2]) == int(y64.reshape(-1)[k]) and \
                        int(arg[c, i, 3]) == int(x64.reshape(-1)[k])
                    if not hit:  # a tie within 1e-5 of the FP64 maxima
                        hit = abs(float(s64.reshape(-1)[mine]) - float(s64.reshape(-1)[k])) <= \
                            1e-5 * abs(float(s64.reshape(-1)[k]))
                    hits += int(hit)
                    total += 1
                worst = max(worst, abs(got / want - 1.0))
            entry.update({"score_max_rel_err_vs_fp64": worst,
                          "argmax_agreement_vs_fp64": hits / max(1, total)})
        out[prec] = entry
    return out


SERVE_BOXES = ("box96_serve", "box128_5kp", "box192_serve")  # boxes 96 / 128 / 192, 1k / 3k / 6k moving atoms
SERVE_POOL = 600        # unique particle images per box; jobs draw their particles from these
SERVE_JOBS = 5          # resident jobs, particles log-uniform over 1,000-20,000
SERVE_MAX_BATCH = 64
SERVE_WORKERS = 3


def _serve_stream(srv, jids, req_job, req_poses, arrive):
    """Submit the requests at their arrival times (seconds after t0) from
    four driver threads; wait for all; (wall seconds, results)."""
    import threading
    t0 = time.perf_counter()
    futs = [None] * len(req_job)

    def driver(d):
        for i in range(d, len(req_job), 4):
            wait = t0 + arrive[i] - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            futs[i] = srv.submit(req_job[i], req_poses[i])

    ts = [threading.Thread(target=driver, args=(d,)) for d in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    srv.drain()
    return time.perf_counter() - t0, [f.result() for f in futs]


def run_serving(args, device):
    """Candidate-evaluation requests from concurrent drivers over resident
    jobs at the serving configuration's shapes: jobs of box 96, 128 or 192
    with 1,000-20,000 particles (log-uniform), requests of 1-64 candidates,
    tensor-core split form, continuous batching. Three streams:
    capacity (every request offered at once, load above capacity),
    latency (Poisson arrivals at half the measured capacity, p50/p99 from
    arrival to scores on the host, against serial plain FP32 evaluation of
    the same stream) and admission (the HBM cap lowered to the largest
    and smallest jobs' footprints, jobs retired once served, so admission
    defers jobs)."""
    import numpy as np
    import torch
    from gisapr_gb300 import synthetic as syn
    from gisapr_gb300.engine import JobConfig, ScoringJob
    from gisapr_gb300.serving import ScoringServer, job_footprint_bytes
    from gisapr_gb300.tables import model_angles_from_lists

    rng = np.random.default_rng(args.seed + 4242)
    t_gen = time.perf_counter()
    pools = {name: syn.make_job(syn.WORKLOADS[name], seed=args.seed + 50 + k, device=str(device),
                                n_particles=SERVE_POOL) for k, name in enumerate(SERVE_BOXES)}
    jobs = {}
    for k in range(SERVE_JOBS):
        name = SERVE_BOXES[int(rng.integers(0, len(SERVE_BOXES)))]
        npart = int(round(math.exp(rng.uniform(math.log(1000.0), math.log(20000.0)))))
        data = syn.job_from_pool(pools[name], npart, args.seed + 60 + k)
        spec = data.spec
        cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                        local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
        fp = job_footprint_bytes(cfg.box, cfg.new_box, npart, 3, len(data.model_rot), SERVE_MAX_BATCH, "fp16x3",
                                 contexts=SERVE_WORKERS + 1)  # workers' contexts + a batch's second template lane
        jobs[f"job{k}"] = (cfg, data, spec, fp)
    t_gen = time.perf_counter() - t_gen
    jids = sorted(jobs)

    def factory(jid):
        cfg, data, _, _ = jobs[jid]
        return lambda: ScoringJob(cfg, data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                                  job_records(data), data.images, fsc_values=data.fsc, device=device)

    def requests(n_req, seed):
        r = np.random.default_rng(seed)
        rj = [jids[int(i)] for i in r.integers(0, len(jids), size=n_req)]
        rn = [int(x) for x in r.integers(1, 65, size=n_req)]
        rp = [syn.candidate_poses(k, seed + 9000 + i, 5.0, 3.0) for i, k in enumerate(rn)]
        return rj, rn, rp

    n_req = args.serve_requests
    out = {"jobs": [f"{jid}: box {jobs[jid][0].box}, {len(jobs[jid][1].records.rot)} particles, "
                    f"{jobs[jid][3] / 1e9:.1f} GB footprint" for jid in jids],
           "precision": "fp16x3", "max_batch": SERVE_MAX_BATCH, "workers": SERVE_WORKERS, "drivers": 4,
           "synthetic_data_s": t_gen}
    with ScoringServer(device, hbm_cap_bytes=150e9, max_batch=SERVE_MAX_BATCH, n_workers=SERVE_WORKERS,
                       precision="fp16x3") as srv:
        for jid in jids:
            srv.register(jid, factory(jid), jobs[jid][3])
        t_build = time.perf_counter()
        for jid in jids:  # build every job and its batch buffers
            srv.submit(jid, syn.candidate_poses(1, 7, 5.0, 3.0)).result()
        out["job_build_s"] = time.perf_counter() - t_build
        # (A) capacity: every request offered at once
        rj, rn, rp = requests(n_req, args.seed + 11)
        srv.reset_stats()
        torch.cuda.synchronize(device)
        wall, _ = _serve_stream(srv, jids, rj, rp, np.zeros(n_req))
        st = srv.stats()
        capacity = sum(rn) / wall
        out["capacity"] = {"value": capacity, "unit": UNIT, "requests": n_req, "candidates": int(sum(rn)),
                           "offered": "all requests at t = 0", "wall_s": wall, "batches": st.batches,
                           "mean_batch": st.mean_batch}
        # (B) latency at half the measured capacity
        rj, rn, rp = requests(n_req, args.seed + 12)
        mean_req = float(np.mean(rn))
        rate = 0.5 * capacity / mean_req  # requests per second
        arrive = np.cumsum(np.random.default_rng(args.seed + 13).exponential(1.0 / rate, size=n_req))
        srv.reset_stats()
        torch.cuda.synchronize(device)
        wall, served = _serve_stream(srv, jids, rj, rp, arrive)
        st = srv.stats()
        out["latency"] = {"value": sum(rn) / wall, "unit": UNIT, "offered": f"Poisson, {rate:.2f} requests/s "
                          f"(half the capacity, mean {mean_req:.1f} candidates per request)",
                          "latency_ms": {"p50": st.latency_ms_p50, "p99": st.latency_ms_p99},
                          "batches": st.batches, "mean_batch": st.mean_batch}
    # serial plain FP32 of stream B, one candidate at a time, in arrival order
    sjobs = {jid: factory(jid)() for jid in jids}
    for jid in jids:
        sjobs[jid].score(rp[0][0])
    torch.cuda.synchronize(device)
    lat, serial_scores = [], []
    t_free = t_busy = 0.0
    for i in range(n_req):
        t1 = time.perf_counter()
        serial_scores.append(np.asarray([sjobs[rj[i]].score(p) for p in rp[i]]))
        dt = time.perf_counter() - t1
        t_busy += dt
        start = max(arrive[i], t_free)
        t_free = start + dt
        lat.append(t_free - arrive[i])
    del sjobs
    lat_ms = np.asarray(lat) * 1e3
    out["latency"]["serial_plain_fp32"] = {"value": sum(rn) / t_busy, "unit": UNIT,
                                           "latency_ms": {"p50": float(np.percentile(lat_ms, 50)),
                                                          "p99": float(np.percentile(lat_ms, 99))}}
    out["latency"]["max_score_rel_diff_vs_serial_fp32"] = max(
        float(np.max(np.abs(a / b - 1.0))) for a, b in zip(served, serial_scores))
    torch.cuda.empty_cache()
    # (C) admission under a lowered cap: the largest plus the smallest
    # footprint, so every job fits alone but not all at once
    fps = sorted((jobs[j][3] for j in jids), reverse=True)
    cap = fps[0] + fps[-1]
    with ScoringServer(device, hbm_cap_bytes=cap, max_batch=SERVE_MAX_BATCH, n_workers=SERVE_WORKERS,
                       precision="fp16x3") as srv:
        t0 = time.perf_counter()
        futs = []
        for k, jid in enumerate(jids):
            srv.register(jid, factory(jid), jobs[jid][3])
        for k, jid in enumerate(jids):
            futs.append((jid, [srv.submit(jid, syn.candidate_poses(16, args.seed + 300 + 8 * k + i, 5.0, 3.0))
                               for i in range(4)]))
        for jid, fl in futs:  # serve each job's requests, then retire it
            for f in fl:
                f.result()
            srv.retire(jid)
        srv.drain()
        st = srv.stats()
        out["admission"] = {"hbm_cap_gb": cap / 1e9, "jobs": len(jids), "deferred_admissions": st.deferred_admissions,
                            "peak_admitted_gb": st.peak_in_use / 1e9, "candidates": st.candidates,
                            "wall_s": time.perf_counter() - t0, "out_of_memory": st.out_of_memory}
    torch.cuda.empty_cache()
    return out


def run_gb300(args, rank: int, world: int, local_rank: int):
    import numpy as np
    import torch
    import __graft_entry__ as g
    from gisapr_gb300 import synthetic as syn
    from gisapr_gb300.engine import JobConfig, ScoringJob
    from gisapr_gb300.tables import model_angles_from_lists

    g.build()
    device = torch.device("cuda", local_rank)
    torch.cuda.set_device(device)
    t_setup = time.perf_counter()
    from gisapr_gb300.replicas import replica_seed
    spec, data, models = make_workload(args.workload, replica_seed(args.seed, rank), str(device), args.particles,
                                       with_models=True)
    t_data = time.perf_counter() - t_setup
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                    local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                     job_records(data), data.images, fsc_values=data.fsc, device=device)
    K, W = args.steps, args.warmup
    poses = syn.candidate_poses(K + W, args.seed + 100 + rank, spec.pose_rotation_deg, spec.pose_translation,
                                exact=True)
    pose_dev = torch.stack([job.density.pose_tensor(p) for p in poses]).to(device)
    for k in range(W):
        job.enqueue(pose_dev[k])
    torch.cuda.synchronize(device)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-timed region: poses resident in HBM
    stage_events = {}
    step_ev = []
    clocks = ClockSampler(local_rank)
    barrier()
    torch.cuda.synchronize(device)
    clocks.start()
    clocks.begin()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record()
    for k in range(K):
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        step_ev.append(e)
        job.enqueue(pose_dev[W + k], stage_events=stage_events)
    end.record()
    torch.cuda.synchronize(device)
    clocks.end()
    barrier()
    elapsed = start.elapsed_time(end) / 1e3
    step_ev.append(end)
    lat = sorted(step_ev[i].elapsed_time(step_ev[i + 1]) for i in range(K))
    stage_ms = {s: statistics.mean(a.elapsed_time(b) for a, b in v) for s, v in stage_events.items()}

    # ---- end to end through the public API, host buffers each step (two
    # untimed calls first: the second captures the call's launch sequence)
    peaks_host = torch.empty(len(job.records), dtype=torch.float32).pin_memory()
    for _ in range(2):
        job.score(poses[0])
    barrier()
    torch.cuda.synchronize(device)
    clocks.begin()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    scores = []
    for k in range(K):
        scores.append(job.score(poses[W + k]))
        peaks_host.copy_(job.peak, non_blocking=True)
    e1.record()
    torch.cuda.synchronize(device)
    clocks.end()
    barrier()
    e2e_elapsed = e0.elapsed_time(e1) / 1e3

    # ---- batched generations: args.batch candidates per step, one CUDA graph
    batched = {}
    if args.batch > 0:
        from gisapr_gb300.pdb2mrc import MovedChainDensity
        dens = [MovedChainDensity(m.pdb_text, "A", spec.box, spec.apix, spec.res, device, from_text=True)
                for m in models]
        gen = [syn.candidate_poses(args.batch, args.seed + 1000 + 31 * k + rank, 5.0, 3.0) for k in range(K + W)]
        # launch shapes from the autotuner (cluster size of the plain correlation,
        # candidates per tensor-core launch), timed on this job
        from gisapr_gb300.autotune import Autotuner
        t_tune = time.perf_counter()
        if args.no_autotune:
            tuned = None
            autotune = {"corr_cluster": "default", "tc_chunk": min(args.batch, 128)}
        else:
            tuned = Autotuner(trials=1).tune(job, n_cand=args.batch, precision="fp16x3")
            autotune = {"corr_cluster": tuned.corr_cluster, "tc_chunk": tuned.tc_chunk,
                        "tc_dirs_per_tile": tuned.dirs_per_tile,
                        "tc_rings": [tuned.tc_a_stages, tuned.tc_b_stages],
                        "template_lanes": tuned.template_lanes,
                        "correlate_ms": tuned.times_ms, "tune_s": time.perf_counter() - t_tune}
        for precision in args.precisions.split(","):
            batched[precision] = run_batched(job, dens, gen, precision, args.batch, K, W, device, barrier,
                                             tc_chunk=tuned.tc_chunk if tuned else 128,
                                             lanes=tuned.template_lanes if tuned else 2, clocks=clocks)
            batched[precision]["autotune"] = autotune
    clk = clocks.stop()  # samples inside the timed regions above (plain, end to end, batched)
    tl = [elapsed, e2e_elapsed]
    for b in batched.values():
        tl += [b["elapsed_s"], b["e2e_elapsed_s"]]
    from gisapr_gb300.replicas import job_rate, max_over_ranks
    times = max_over_ranks(tl, device=device)  # the slowest replica's times
    elapsed, e2e_elapsed = times[0], times[1]
    for i, b in enumerate(batched.values()):
        b["value"] = job_rate(world, K * args.batch, times[2 + 2 * i])
        b["unit"] = UNIT
        b["e2e"] = {"value": job_rate(world, K * args.batch, times[3 + 2 * i]), "unit": UNIT,
                    "h2d_bytes_per_step": b.pop("e2e_h2d_bytes_per_step"),
                    "d2h_bytes_per_step": b.pop("e2e_d2h_bytes_per_step")}
        b.pop("elapsed_s")
        b.pop("e2e_elapsed_s")
        b["vs_plain_single"] = b["value"] / job_rate(world, K, elapsed)
    if "fp32" in batched:
        for b in batched.values():
            b["vs_plain_batched"] = b["value"] / batched["fp32"]["value"]
    if rank != 0:
        return
    value = job_rate(world, K, elapsed)
    e2e_value = job_rate(world, K, e2e_elapsed)
    hbm_peak, bf16_peak, peak_kind = load_peaks()
    maps = job.nnz * job.n_psi
    flops = correlation_flops(cfg.new_box, maps)
    corr_s = stage_ms["correlate"] / 1e3
    dominant = max(stage_ms, key=stage_ms.get)
    achieved = flops / corr_s / 1e12
    traffic = profiled_traffic("correlate_plain", args.workload) if not args.particles else None
    roofline = {
        "kernel": "correlate_plain", "bound": "tensor", "achieved": achieved, "peak": bf16_peak,
        "unit": "TFLOP/s", "frac": achieved / bf16_peak, "traffic": traffic,
        "peak_source": f"{peak_kind} bf16 dense (MEASURED_PEAKS.json)" if peak_kind == "measured" else "fallback",
        "algorithmic": f"{flops:.4g} flop per launch = {maps} maps x (6K + 2.5 n^2 log2 n^2), n={cfg.new_box}",
        "note": "plain FP32 correlation runs on CUDA cores; its fraction is against the bf16 tensor peak",
        "fp32_cuda_core": {"peak": FP32_CORE_PEAK_TFLOPS, "unit": "TFLOP/s",
                           "frac": achieved / FP32_CORE_PEAK_TFLOPS,
                           "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 flop (FMA) x 2070 MHz"},
        "dominant_stage": dominant, "stage_ms": stage_ms,
    }
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": elapsed / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": dict(gb300_config(spec), form="plain FP32", parallelism=f"replicas x{world}",
                       l2=l2_note(job.stack.numel() * job.stack.element_size())),
        "job": {"particles": len(job.records), "moving_atoms": job.density.n_moving,
                "fixed_atoms": job.density.fixed_atom_count, "directions": len(data.model_rot),
                "needed_directions": len(job.needed), "maps_per_candidate": maps},
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)]},
        "roofline": roofline,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 12 * 8,
                "d2h_bytes_per_step": 8 + 4 * len(job.records)},
        "gpu_launches": job.launches_per_candidate() * K,
        "clocks": clk,
        "setup_s": {"synthetic_data": t_data, "job": job.setup_s},
        "score_sample": scores[0],
    }
    if batched:
        line["batched"] = batched
    if world == 1 and args.serve_requests > 0:
        line["serving"] = run_serving(args, device)
    if world == 1 and args.precision_particles > 0:
        line["precision"] = run_precision(args, device)
    if world == 1:
        line["deposit_vs_reference"] = run_deposit_comparison(job, data, spec, poses[W], device)
    if world == 1 and args.reference_cuda_sample > 0:
        rc = run_reference_cuda(data, poses[W], device, args.reference_cuda_sample)
        if "value" in rc:
            # the reference's partial score over its particle sample against the
            # same particles' peaks from this path (one candidate, same pose)
            import numpy as np
            job.score(poses[W])
            pk = job.peak.cpu().numpy().astype(np.float64)
            has = (job.local_ptr[1:] > job.local_ptr[:-1]).cpu().numpy()
            sel = [i for i in rc.pop("particles") if has[i]]
            ours = float(np.sum(np.exp(pk[sel] / 1024.0)))
            rc["partial_score_rel_diff"] = abs(ours / rc.pop("partial_score") - 1.0)
            rc["gb300_plain_vs_reference_cuda"] = value / rc["value"]
            for name, b in batched.items():
                rc[f"gb300_batched_{name}_vs_reference_cuda"] = b["value"] / rc["value"]
        line["reference_torch_cuda"] = rc
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = run_cpu_baseline(spec, data, poses[W], args.cpu_sample)
    print(json.dumps(line), flush=True)


def host_cpu() -> dict:
    """The host's CPU model (lscpu, else /proc/cpuinfo, else the machine
    type) and its logical core count, stated beside every CPU timing."""
    import platform
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        model = next((ln.split(":", 1)[1].strip() for ln in out.splitlines()
                      if ln.lower().startswith("model name:")), None)
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as fh:
                model = next((ln.split(":", 1)[1].strip() for ln in fh
                              if ln.lower().startswith(("model name", "hardware"))), None)
        except OSError:
            pass
    return {"cpu_model": model or platform.machine(), "nproc": os.cpu_count()}


def run_cpu_baseline(spec, data, pose, sample: int) -> dict:
    """The reference's own CPU path on this job (one pose, 100 particles;
    about 10 s of CPU work), or the numpy port when baseline/_ref is absent."""
    import numpy as np
    from baseline import reference_runner as ref_runner
    n_p = len(data.records.rot)
    if ref_runner.available():
        idx = np.unique(np.linspace(0, n_p - 1, min(100, n_p)).astype(int)).tolist()
        runner = ref_runner.RefRunner(data)
        t0 = time.perf_counter()
        r = runner.step(pose, idx)
        wall = time.perf_counter() - t0
        sec = r["density_s"] + r["templates_s"] + r["particles_s"] * n_p / len(idx)
        return {"value": 1.0 / sec, "unit": UNIT, "cores": runner.threads, "kind": "reference",
                "sample": f"GisAPR's own CPU torch path from baseline/_ref, one pose: density, "
                          f"{int(r['n_templates'])} templates, {len(idx)} of {n_p} particles "
                          f"(particle time scaled to all {n_p}; {wall:.1f} s of CPU work)", **host_cpu()}
    cb = cpu_baseline(spec, data, pose, sample)
    return {"value": 1.0 / cb["seconds_per_candidate"], "unit": UNIT, "cores": int(cb["threads"]), "kind": "port",
            **host_cpu(),
            "sample": f"numpy port of the reference's CPU path (baseline/_ref absent), one pose: full "
                      f"moving-chain splat and 3-D FFT, {int(cb['sample_templates'])} templates timed "
                      f"(extrapolated to the {int(cb['n_templates'])} needed), {int(cb['sample_particles'])} of "
                      f"{n_p} particles (prepare + correlate), extrapolated ({cb['sample_wall_s']:.1f} s of CPU work)"}


def run_reference_cuda(data, pose, device, sample: int = 500) -> dict:
    """GisAPR's own torch path on this GPU (the same functions the CPU
    baseline runs, device cuda): one pose, density, every template, and an
    evenly spaced sample of the job's particles, the particle time scaled to
    the whole job; the score of the sample is checked against the GB300
    path's per-particle peaks by the caller."""
    import numpy as np
    from baseline import reference_runner as ref_runner
    if not ref_runner.available():
        return {"unavailable": "baseline/_ref (the reference's optimized-3 tree) is not installed"}
    n_p = len(data.records.rot)
    idx = np.unique(np.linspace(0, n_p - 1, min(sample, n_p)).astype(int)).tolist()
    try:
        runner = ref_runner.RefRunner(data, device=str(device))
        runner.step(pose, idx[:4])  # warm-up: cuFFT plans, kernel loads, caching allocator
        t0 = time.perf_counter()
        r = runner.step(pose, idx)
        wall = time.perf_counter() - t0
    except Exception as exc:  # noqa: BLE001 - reported, not hidden
        return {"unavailable": f"reference torch CUDA path failed: {type(exc).__name__}: {exc}"[:300]}
    sec = r["density_s"] + r["templates_s"] + r["particles_s"] * n_p / len(idx)
    return {"value": 1.0 / sec, "unit": UNIT,
            "stage_s": {"density": r["density_s"], "templates": r["templates_s"],
                        "particles_scaled": r["particles_s"] * n_p / len(idx)},
            "sample": f"GisAPR's own torch path from baseline/_ref on {device}, one pose: density, "
                      f"{int(r['n_templates'])} templates, {len(idx)} of {n_p} particles (particle time "
                      f"scaled to all {n_p}; {wall:.1f} s wall)",
            "partial_score": r["partial_score"], "particles": idx}


def run_deposit_comparison(job, data, spec, pose, device, reps: int = 20) -> dict:
    """The moving chain onto the cached fixed context, as one candidate's
    density step: the reference's GPU splat (pdb2mrc v4 with the NVRTC
    deposit kernel: a clone of the fixed volume, one block per atom, global
    float atomics) against gisapr_deposit_moved (pose, 8.3 round trip and
    binned splat fused), device time per call with CUDA events. The
    reference gets the moved coordinates the way its Lite path does (pose
    and PDB 8.3 round trip on the host, not timed)."""
    import numpy as np
    import torch
    from baseline import reference_runner as ref_runner
    if not ref_runner.RefDeposit.available():
        return {"unavailable": "baseline/_ref (the reference's Lite tree) is not installed"}
    from gisapr_gb300.pdb_text import quantize_coordinates, transform_coordinates
    dens = job.density
    mv = dens.moving_xyz.cpu().numpy()
    moved = quantize_coordinates(transform_coordinates(mv.astype(np.float64), pose,
                                                        pivot=dens.pivot.cpu().numpy().astype(np.float64)))
    xyz = torch.from_numpy(np.ascontiguousarray(moved, np.float32)).to(device)
    z = dens.moving_z.to(device)
    fixed = dens.fixed.to(device)
    ref = ref_runner.RefDeposit()
    try:
        ref.deposit(xyz, z, spec.box, spec.apix, spec.res, fixed)  # compiles the kernel (NVRTC)
    except Exception as exc:  # noqa: BLE001 - reported, not hidden
        return {"unavailable": f"reference deposit failed: {type(exc).__name__}: {exc}"[:300]}
    out = torch.empty_like(fixed)
    pose_dev = dens.pose_tensor(pose).to(device)

    def timed(fn):
        torch.cuda.synchronize(device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize(device)
        return a.elapsed_time(b) / reps

    ref_ms = timed(lambda: ref.deposit(xyz, z, spec.box, spec.apix, spec.res, fixed))
    ours_ms = timed(lambda: dens.generate(None, out=out, pose_device=pose_dev))
    got = ref.deposit(xyz, z, spec.box, spec.apix, spec.res, fixed).cpu().numpy().astype(np.float64)
    dens.generate(None, out=out, pose_device=pose_dev)
    mine = out.cpu().numpy().astype(np.float64)
    rrms = float(np.sqrt(np.sum((mine - got) ** 2) / np.sum(got ** 2)))
    return {"moving_atoms": int(dens.n_moving), "box": spec.box,
            "reference_nvrtc_deposit_ms": ref_ms, "gb300_deposit_moved_ms": ours_ms, "speedup": ref_ms / ours_ms,
            "density_rrms_vs_reference": rrms,
            "note": "device time per call (CUDA events, mean of 20); the reference clones the fixed volume and "
                    "adds the moved atoms with global atomics, gisapr_deposit_moved also applies the pose"}


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    try:
        run_gb300(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
