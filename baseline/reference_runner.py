"""GisAPR's own code, timed -- BENCH INFRASTRUCTURE ONLY.

The reference arm of bench.py runs the reference's code itself, unmodified,
from baseline/_ref (unpacked there by baseline/install_reference.py;
nothing reads the original source tree at run time): the optimized-3
tree's pdb2mrc v3 ``generate_volume`` (every atom re-splatted per
candidate), v606's ``IntegratedProjector.build_templates`` over every
direction of the angle table, ``PackedCTFTorch.batch``, and per particle
``ParticleFourierPreparer.prepare``, ``correlate_templates_and_particle``
and ``make_result_records``, in the order of its ``run_search`` loop
(v606:1594-1825). On the CPU torch uses every host thread; with a CUDA
device the same functions run on the GPU (the reference's own torch CUDA
path), with a synchronize at each stage boundary.

``RefRunner(job, device=...).step(pose, particle_index)`` scores one
candidate pose on the given particles of the job and returns the seconds of
each stage. ``RefDeposit`` is the Lite tree's NVRTC splat. The package never
imports this module; bench.py's reference arm, its CPU baseline and its
comparisons with the reference's GPU code are its only users.
"""
from __future__ import annotations

import os
import sys
import tempfile
import time
import types
from pathlib import Path
from typing import Dict, Optional, Sequence

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
REF_TREE = ROOT / "baseline" / "_ref" / "GisAPR-210-optimized"
LITE_TREE = ROOT / "baseline" / "_ref" / "GisAPR-210-DE-v1.3.2"
V606 = "test1_with_isspa_weight_varingKK_search_translation_also_v606_torch_optimized_standalone"


def available() -> bool:
    return (REF_TREE / f"{V606}.py").exists() and (REF_TREE / "pdb2mrc_gpu_ver_fp32_v3.py").exists()


def _stub_mrcfile():
    if "mrcfile" not in sys.modules:
        stub = types.ModuleType("mrcfile")

        def _no_io(*a, **k):
            raise RuntimeError("file IO is bypassed: volumes and images are passed as tensors")

        stub.mmap = stub.new = stub.open = _no_io
        stub.mrcfile = types.SimpleNamespace(MrcFile=object)
        sys.modules["mrcfile"] = stub


def import_reference():
    """(v606, pdb2mrc, pdb_text) modules of the reference's optimized-3 tree."""
    import importlib
    _stub_mrcfile()
    if str(REF_TREE) not in sys.path:
        sys.path.insert(0, str(REF_TREE))
    return (importlib.import_module(V606), importlib.import_module("pdb2mrc_gpu_ver_fp32_v3"),
            importlib.import_module("pdb_text"))


def _write_angle_star(path, rot, tilt):
    with open(path, "w") as f:
        f.write("\ndata_\n\nloop_\n_rlnAngleRot #1\n_rlnAngleTilt #2\n_rlnAnglePsi #3\n")
        for r, t in zip(rot, tilt):
            f.write(f"{float(r)!r}\t{float(t)!r}\t0.0\n")


def _write_particle_star(path, rec):
    with open(path, "w") as f:
        head = ("\ndata_\n\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAngleTilt #3\n"
                "_rlnAnglePsi #4\n_rlnDefocusU #5\n_rlnDefocusV #6\n_rlnDefocusAngle #7\n")
        f.write(head)
        lines = head.count("\n")
        for i in range(len(rec.rot)):
            while lines < int(rec.line_index[i]):
                f.write("\n")
                lines += 1
            vals = [float(v[i]) for v in (rec.rot, rec.tilt, rec.psi, rec.defocus_u, rec.defocus_v,
                                          rec.defocus_angle)]
            f.write(f"{i + 1}@stack.mrcs\t" + "\t".join(repr(v) for v in vals) + "\n")
            lines += 1


class RefRunner:
    """One job's tables built once (as the reference's worker caches them),
    then candidate evaluations through the reference's functions."""

    def __init__(self, job, threads: int = 0, device: str = "cpu"):
        import torch
        self.threads = threads or (os.cpu_count() or 1)
        torch.set_num_threads(self.threads)
        self.device = torch.device(device)
        self.v606, self.pdb2mrc, self.pdb_text = import_reference()
        v = self.v606
        spec = job.spec
        self.job, self.spec = job, spec
        self.tmp = Path(tempfile.mkdtemp(prefix="gisapr_ref_"))
        self.pdb_path = self.tmp / "model.pdb"
        self.pdb_path.write_text(job.model.pdb_text)
        _write_angle_star(self.tmp / "angles.star", job.model_rot, job.model_tilt)
        _write_particle_star(self.tmp / "particles.star", job.records)
        self.angles = v.read_model_angles(str(self.tmp / "angles.star"))
        table = v.read_particle_table(str(self.tmp / "particles.star"))
        self.table = table
        self.records = table.records
        dev = self.device
        n, nb = spec.box, spec.new_box
        self.layout = v.PackedFourierLayout(nb, spec.crop, dev)
        self.new_apix = n / nb * spec.apix
        self.trans_scale = spec.apix / self.new_apix
        self.local = {e[0]: e[1:] for e in v.build_local_orientation_entries(
            self.records, self.angles.rot, self.angles.tilt, spec.local_range)}
        mask = torch.from_numpy(v.generate_soft_mask((n, n), spec.mask_radius, spec.mask_edge)).to(dev)
        fsc_path = ""
        if spec.fsc_half_res is not None:
            fsc_path = str(self.tmp / "fsc.txt")
            with open(fsc_path, "w") as f:
                for k, val in enumerate(job.fsc):
                    f.write(f"{k} {float(val)!r}\n")
        packed_fsc = self.layout.centered_full_to_packed(
            torch.from_numpy(v.read_fsc_map(fsc_path, n, nb, False)).to(dev))
        self.projector = v.IntegratedProjector(dev, n, nb, self.layout, mask, packed_fsc, 8)
        self.psi_meta = {}
        uniq = {}
        for rec in self.records:
            fake, eff = v.psi_sampling_for_record(rec.psi, spec.psi_step, True, spec.local_range)
            self.psi_meta[rec.line_index] = (fake, eff)
            for a in eff:
                uniq[float(np.round(a, 6))] = None
        bank = v.PsiGridBank(n, dev, list(uniq.keys()), 8)
        self.prep = v.ParticleFourierPreparer(n, nb, dev, self.layout, mask, bank)
        self.ctfgen = v.PackedCTFTorch(nb, self.new_apix, spec.cs, spec.voltage, spec.kk, dev)
        self.ws = v.CorrelationWorkspace(dev)
        self.images = job.images

    def step(self, pose, particle_index: Sequence[int]) -> Dict[str, float]:
        """One candidate on the given particles: stage seconds, the number of
        templates built and the partial score sum_i exp(rawCC_i / 1024)."""
        import torch
        v, spec, dev = self.v606, self.spec, self.device
        out: Dict[str, float] = {}

        def now():
            if dev.type == "cuda":
                torch.cuda.synchronize(dev)
            return time.perf_counter()

        with torch.no_grad():
            t0 = now()
            density = self.pdb2mrc.generate_volume(str(self.pdb_path), spec.box, spec.apix, spec.res,
                                                   device=str(dev), source_pdb=str(self.pdb_path), chain_id="A",
                                                   pose=list(map(float, pose)))
            t1 = now()
            templates = self.projector.build_templates(density, self.angles)
            t2 = now()
            recs = [self.records[i] for i in particle_index]
            ctf = self.ctfgen.batch(recs, self.table.has_ctf)
            if isinstance(ctf, np.ndarray):
                ctf = torch.from_numpy(ctf)
            ctf = ctf.to(dev)
            raw = []
            for k, (i, rec) in enumerate(zip(particle_index, recs)):
                idx = self.local.get(rec.line_index, [])
                if not idx:
                    continue
                fake, eff = self.psi_meta[rec.line_index]
                p = self.prep.prepare(torch.from_numpy(self.images[i]).to(dev), eff, ctf[k])
                lt = templates.index_select(0, torch.tensor(idx, dtype=torch.long, device=dev))
                s, y, x = v.correlate_templates_and_particle(lt, p, self.layout, self.ws)
                rr = v.make_result_records(rec, fake, self.angles.rot, self.angles.tilt, idx, s, y, x,
                                           self.layout.crop_size, self.trans_scale)
                raw.append(rr[2][2])
            t3 = now()
        out["density_s"] = t1 - t0
        out["templates_s"] = t2 - t1
        out["particles_s"] = t3 - t2
        out["n_templates"] = float(templates.shape[0])
        out["n_particles"] = float(len(particle_index))
        out["partial_score"] = float(np.sum(np.exp(np.asarray(raw, dtype=np.float64) / 1024.0)))
        return out


class RefDeposit:
    """The reference's GPU splat: pdb2mrc v4 ``density_from_coords`` with
    ``backend='cuda'`` (a clone of the cached fixed-context volume plus the
    NVRTC ``deposit`` kernel, one block per atom with global atomics) from
    the Lite tree in baseline/_ref."""

    def __init__(self):
        import importlib
        _stub_mrcfile()
        if str(LITE_TREE) not in sys.path:
            sys.path.insert(0, str(LITE_TREE))
        self.pdb2mrc = importlib.import_module("pdb2mrc_gpu_ver_fp32_v4")

    @staticmethod
    def available() -> bool:
        return (LITE_TREE / "gisapr_cuda_density.py").exists() and (LITE_TREE / "pdb2mrc_gpu_ver_fp32_v4.py").exists()

    def deposit(self, xyz, numbers, box, apix, res, fixed):
        return self.pdb2mrc.density_from_coords(xyz, numbers, box, apix, res, device=fixed.device,
                                                _initial_volume=fixed, backend="cuda")
