"""Golden templates at boxes 96, 192 and 256, made by GisAPR's own projector.

Run in a checkout that has the reference sources (read, never modified):

    python tests/golden/make_golden_templates.py --reference <GisAPR source root>

The reference is imported as make_golden.py does (the optimized-3 tree with a
stub ``mrcfile``). For each box a seeded density (synthetic.blob_density) goes
through IntegratedProjector.build_templates (v606:1054-1147) for a few random
directions, with the reference's soft mask (generate_soft_mask) and a
logistic FSC read back through read_fsc_map. The fixture stores the seeds,
the directions, the mask and FSC parameters and the reference's float32
templates; the test regenerates the density from its seed.
"""
from __future__ import annotations

import argparse
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(HERE))

from gisapr_gb300 import synthetic as syn  # noqa: E402
from make_golden import _import_reference, _write_angle_star  # noqa: E402

# box -> (directions, FSC half-resolution in A at 1.1 A/pixel)
CASES = {96: (2, 4.0), 192: (1, 4.0), 256: (1, 4.0)}
APIX = 1.1
MASK_EDGE = 6


def reference_templates(v606, n: int, n_dir: int, half_res: float, tmp: Path) -> dict:
    import torch
    rng = np.random.default_rng(1000 + n)
    rot = rng.uniform(-180.0, 180.0, n_dir)
    tilt = np.rad2deg(np.arccos(rng.uniform(-1.0, 1.0, n_dir)))
    vol = syn.blob_density(n, n)
    ang_path = tmp / f"angles{n}.star"
    _write_angle_star(ang_path, rot, tilt)
    angles = v606.read_model_angles(str(ang_path))
    dev = torch.device("cpu")
    layout = v606.PackedFourierLayout(n, 8, dev)
    radius = int(round(0.43 * n))
    mask = torch.from_numpy(v606.generate_soft_mask((n, n), radius, MASK_EDGE))
    fsc = syn.logistic_fsc(n, APIX, half_res)
    fsc_path = tmp / f"fsc{n}.txt"
    with open(fsc_path, "w") as f:
        for k, v in enumerate(fsc):
            f.write(f"{k} {float(v)!r}\n")
    fsc_centered = v606.read_fsc_map(str(fsc_path), n, n, False)
    packed_fsc = layout.centered_full_to_packed(torch.from_numpy(fsc_centered))
    projector = v606.IntegratedProjector(dev, n, n, layout, mask, packed_fsc, 8)
    templates = projector.build_templates(torch.from_numpy(vol), angles)
    return {f"b{n}_seed": np.int64(n), f"b{n}_rot": rot, f"b{n}_tilt": tilt,
            f"b{n}_mask_radius": np.int64(radius), f"b{n}_half_res": np.float64(half_res),
            f"b{n}_templates": templates.numpy().astype(np.complex64)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE / "golden_templates.npz"))
    a = ap.parse_args()
    out = {"apix": np.float64(APIX), "mask_edge": np.int64(MASK_EDGE)}
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        v606, _, _ = _import_reference(Path(a.reference), tmp)
        for n, (n_dir, half_res) in CASES.items():
            out.update(reference_templates(v606, n, n_dir, half_res, tmp))
            print(n, out[f"b{n}_templates"].shape, flush=True)
    np.savez_compressed(a.out, **out)
    print(a.out)


if __name__ == "__main__":
    main()
