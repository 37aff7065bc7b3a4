"""Generate the box-128 fixture by running GisAPR's reference code itself.

    python tests/golden/make_golden_box128.py --reference <GisAPR source root>

This is the benchmarked configuration (box 128 at 1.1 A/px, moving chain of
3,000 atoms over a 20,000-atom fixed context, HEALPix order 3 within +-10
degrees, psi step 7.5 degrees, translations +-5 px so crop 12, logistic FSC
crossing 0.5 at 4 A, SNR 0.05, the moving chain perturbed by 3 degrees and
1.5 A), on the first 160 particles of its seeded generator. The reference's
optimized-3 tree (v606 with in-memory volumes, pdb2mrc v3) runs on the CPU
through the same ``run_reference`` as tests/golden/make_golden.py: density,
every template of the 768 directions, CTF, particle spectra, correlation,
result records and the candidate score.

The particle images are regenerated from the seed by the tests, so the file
holds input checksums and the reference's outputs: a density slab and
checksum, 16 templates (every needed direction's map maxima are stored, so
all of them are covered indirectly), the spectra of two particles, every
per-map maximum with its position, per-particle records and the score.
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(HERE))

from gisapr_gb300 import synthetic as syn  # noqa: E402
from make_golden import _flat, _import_reference, run_reference  # noqa: E402

SEED = 31
POSE_SEED = 32
N_PARTICLES = 160


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE))
    args = ap.parse_args()
    import torch
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        v606, pdb2mrc, pdb_text = _import_reference(Path(args.reference), td / "ref")
        spec = syn.WORKLOADS["box128_5kp"]
        job = syn.make_job(spec, seed=SEED, n_particles=N_PARTICLES)
        pose = syn.candidate_poses(1, POSE_SEED, 3.0, 1.5, exact=True)[0]
        r = run_reference(v606, pdb2mrc, pdb_text, job, pose, td)
        needed = sorted(set(int(k) for k in r["local_idx"]))
        sel_t = np.asarray(needed, np.int64)[np.linspace(0, len(needed) - 1, 16).astype(np.int64)]
        sel_p = np.asarray([0, 7], np.int64)
        dens = r["density"].astype(np.float64)
        np.savez_compressed(
            Path(args.out) / "golden_box128.npz",
            spec_name=np.asarray(spec.name), seed=np.asarray(SEED), n_particles=np.asarray(N_PARTICLES),
            pose=pose,
            image_checksum=np.asarray([job.images.astype(np.float64).sum(),
                                       (job.images.astype(np.float64) ** 2).sum()]),
            image_probe=job.images[:, 64, 64].copy(),
            density_slab=r["density"][62:66].copy(),
            density_checksum=np.asarray([dens.sum(), (dens ** 2).sum()]),
            template_index=sel_t, templates=r["templates"][sel_t],
            particle_index=sel_p, spectra=np.stack(r["spectra"])[sel_p],
            local_ptr=np.asarray(r["local_ptr"], np.int64),
            local_idx=np.asarray(r["local_idx"], np.int64),
            scores=_flat(r["scores"], np.float32), ys=_flat(r["ys"], np.int64),
            xs=_flat(r["xs"], np.int64),
            z=np.asarray(r["z"]), peak=np.asarray(r["peak"]), best_dir=np.asarray(r["best_dir"]),
            best_psi=np.asarray(r["best_psi"]), shift_x=np.asarray(r["shift_x"]),
            shift_y=np.asarray(r["shift_y"]), score=np.asarray(r["score"]))
        print("box128 score", r["score"], "needed directions", len(needed), "maps", len(_flat(r["scores"], np.float32)))


if __name__ == "__main__":
    main()
