"""Generate golden_restraint.npz by running the reference's geometric restraint.

    python tests/golden/make_golden_restraint.py --reference <GisAPR source root>

The reference's func_check_boundary_for_testing_v8.py with the modules it
imports (pdb2mrc_gpu_ver_fp32_v3.py, pdb_text.py) is copied to a temporary
directory (the sources are read, never modified) and its GeometryRestraint
runs on the CPU for a seeded two-chain model at box 96 / 1.5 A. The fixture
stores the model's PDB text, the poses, the reference's (overlap, distance)
per pose, the main-body mask voxel count and the reference's moved chain
coordinates of two poses.
"""
from __future__ import annotations

import argparse
import shutil
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from gisapr_gb300 import synthetic as syn  # noqa: E402

FILES = ("func_check_boundary_for_testing_v8.py", "pdb2mrc_gpu_ver_fp32_v3.py", "pdb_text.py")

BOX, APIX, THRESHOLD = 96, 1.5, 1.0
# rotation vector in degrees, then translation in Angstrom
POSES = np.asarray([
    [0.0, 0.0, 0.0, 0.0, 0.0, 0.0],          # fully overlapping
    [5.0, 3.0, -2.0, 4.0, -3.0, 2.0],
    [10.0, -5.0, 20.0, 25.0, 0.0, 0.0],
    [0.0, 30.0, 0.0, 40.0, 10.0, -5.0],
    [40.0, 10.0, -30.0, 0.0, 48.0, 10.0],
    [-20.0, 15.0, 5.0, -38.0, -38.0, 20.0],
    [60.0, -40.0, 10.0, 52.0, 40.0, 0.0],    # partly outside the box
    [0.0, 0.0, 0.0, 0.0, 0.0, 58.0],
    [0.0, 0.0, 0.0, 150.0, 0.0, 0.0],        # chain wholly outside the box
], dtype=np.float64)
PIVOT = np.asarray([3.0, -2.0, 1.5], dtype=np.float64)
PIVOT_POSES = np.asarray([[0.0, 25.0, 10.0, 30.0, 20.0, 0.0], [15.0, 0.0, -35.0, -20.0, 30.0, 12.0]])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE / "golden_restraint.npz"))
    args = ap.parse_args()
    model = syn.make_model(syn.residues_for_atoms(760), syn.residues_for_atoms(3030), seed=41)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for f in FILES:
            shutil.copy(Path(args.reference) / f, td / f)
        sys.path.insert(0, str(td))
        sys.dont_write_bytecode = True
        import func_check_boundary_for_testing_v8 as v8
        pdb_path = td / "model.pdb"
        pdb_path.write_text(model.pdb_text)
        r = v8.GeometryRestraint(str(pdb_path), "A", device="cpu", boxsize=BOX, apix=APIX, threshold=THRESHOLD)
        results = np.asarray([r.evaluate(p) for p in POSES], dtype=np.float64)
        pivot_results = np.asarray([r.evaluate(p, pivot=PIVOT) for p in PIVOT_POSES], dtype=np.float64)
        moved = np.stack([v8.rotate_coords_rotvec(r.chain_coords, *POSES[3]),
                          v8.rotate_coords_rotvec(r.chain_coords, *PIVOT_POSES[0], pivot=PIVOT)])
        mask_voxels = int(r.mainbody_mask.sum().item())
    np.savez_compressed(args.out, pdb_text=np.asarray(model.pdb_text), box=BOX, apix=APIX, threshold=THRESHOLD,
                        poses=POSES, results=results, pivot=PIVOT, pivot_poses=PIVOT_POSES,
                        pivot_results=pivot_results, moved=moved.astype(np.float32), mask_voxels=mask_voxels)
    for p, (o, d) in zip(POSES, results):
        print(p, int(o), d)
    print("pivot", pivot_results.tolist(), "mask voxels", mask_voxels)


if __name__ == "__main__":
    main()
