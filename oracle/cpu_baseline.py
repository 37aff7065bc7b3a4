"""CPU baseline of the candidate-scoring path -- TEST/BENCH INFRASTRUCTURE.

Times the oracle (the numpy restatement of the reference in
gisapr_oracle.py) on the host cores for one candidate pose of a job, on a
bounded sample, and extrapolates to the whole candidate:

    t = t_density(moving atoms onto the cached fixed context)
      + t_volume_fft
      + t_template * n_needed_directions      (sampled)
      + t_particle * n_particles              (sampled: prepare + correlate)

Particle spectra are candidate-independent, but the reference's run_search
prepares every particle for every candidate (v606:1749-1810), so the
per-particle cost includes the preparation as the reference pays it.
Template and particle work runs on a thread pool (numpy and pocketfft
release the GIL) and the FFTs use all ``threads`` workers.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import time
from typing import Dict, Sequence

import numpy as np
import scipy.fft as sfft

from . import gisapr_oracle as O


def time_candidate(pdb_text: str, pose, box: int, apix: float, res: float, model_rot: Sequence[float],
                   model_tilt: Sequence[float], images: np.ndarray, rec, fsc_values, mask_radius: int,
                   mask_edge: int, psi_step: float, local_range: float, crop: int, kk: float = 3.0,
                   n_template_sample: int = 64, n_particle_sample: int = 64,
                   threads: int = 0, chain_id: str = "A") -> Dict[str, float]:
    """Seconds per candidate (extrapolated) and the measured sample times."""
    threads = threads or (os.cpu_count() or 1)
    n = int(box)
    rot_t = O.rotation_matrices_t(model_rot, model_tilt)
    mask = O.soft_mask(n, mask_radius, mask_edge)
    packed_fsc = O.centered_to_packed(O.radial_map(fsc_values, n))
    n_particles = len(rec.rot)
    sample_p = np.linspace(0, n_particles - 1, min(n_particle_sample, n_particles)).astype(int)
    local = O.local_orientations(rec.rot[sample_p], rec.tilt[sample_p], model_rot, model_tilt, local_range)
    needed_all = None
    ctfgen = O.PackedCTF(n, apix, 2.7, 300.0, kk)
    out: Dict[str, float] = {"threads": float(threads)}
    with sfft.set_workers(threads):
        # fixed context once (cached by the reference's Lite path), moving chain per candidate
        coords, z, chains = O.moved_density_atoms(pdb_text, chain_id, pose)
        fixed = O.splat_density(coords[chains != chain_id], z[chains != chain_id], n, apix, res)
        t0 = time.perf_counter()
        moved, zm, ch = O.moved_density_atoms(pdb_text, chain_id, pose)
        sel = ch == chain_id
        density = O.splat_density(moved[sel], zm[sel], n, apix, res, initial=fixed)
        t1 = time.perf_counter()
        dft = O.volume_spectrum(density)
        t2 = time.perf_counter()
        out["density_s"] = t1 - t0
        out["volume_fft_s"] = t2 - t1
        needed = sorted({k for l in local for k in l})
        tdirs = np.linspace(0, len(model_rot) - 1, min(n_template_sample, len(model_rot))).astype(int)
        tdirs = sorted(set(tdirs.tolist()) | set(needed))

        def one_template(k):
            return k, O.template_from_slice(O.central_slice(dft, rot_t[k], n), n, n, mask, packed_fsc)

        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            t3 = time.perf_counter()
            templates = dict(ex.map(one_template, tdirs))
            t4 = time.perf_counter()

            def one_particle(j):
                i = int(sample_p[j])
                fake, eff = O.psi_sampling(float(rec.psi[i]), psi_step, True, local_range)
                ctf = ctfgen.one(rec.defocus_u[i], rec.defocus_v[i], rec.defocus_angle[i])
                spec = O.prepare_particle(images[i], eff, ctf, mask, n)
                if local[j]:
                    O.correlate(np.stack([templates[k] for k in local[j]]), spec, crop)
                return i

            t5 = time.perf_counter()
            list(ex.map(one_particle, range(len(sample_p))))
            t6 = time.perf_counter()
        per_template = (t4 - t3) / len(tdirs)
        per_particle = (t6 - t5) / len(sample_p)
        if needed_all is None:
            full_local = O.local_orientations(rec.rot[::max(1, n_particles // 500)],
                                              rec.tilt[::max(1, n_particles // 500)], model_rot, model_tilt,
                                              local_range)
            frac = len({k for l in full_local for k in l}) / max(1, len(model_rot))
            needed_all = max(len(needed), int(round(frac * len(model_rot))))
    out["template_s"] = per_template
    out["particle_s"] = per_particle
    out["n_templates"] = float(needed_all)
    out["n_particles"] = float(n_particles)
    out["sample_templates"] = float(len(tdirs))
    out["sample_particles"] = float(len(sample_p))
    out["seconds_per_candidate"] = (out["density_s"] + out["volume_fft_s"] + per_template * needed_all
                                    + per_particle * n_particles)
    out["sample_wall_s"] = (t2 - t0) + (t4 - t3) + (t6 - t5)
    return out
