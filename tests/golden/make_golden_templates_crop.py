"""Golden templates with a Fourier crop (new box below the box), made by
GisAPR's own projector.

    python tests/golden/make_golden_templates_crop.py --reference <GisAPR source root>

As make_golden_templates.py (the optimized-3 tree's
IntegratedProjector.build_templates, v606:1054-1147, on a seeded blob
density with the reference's soft mask and a logistic FSC read back through
read_fsc_map), but with the templates cropped in Fourier space to a smaller
new box: 128 -> 64, 192 -> 96 and 256 -> 128 (v606:1115-1147 keeps the
central new-box square of each slice spectrum).
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

# (box, new box, directions, FSC half-resolution A, seed)
CASES = ((128, 64, 2, 4.0, 71), (192, 96, 1, 4.0, 72), (256, 128, 1, 4.0, 73))
APIX = 1.1
MASK_EDGE = 6


def case_directions(n_dir: int, seed: int):
    rng = np.random.default_rng(seed)
    return rng.uniform(-180.0, 180.0, n_dir), np.rad2deg(np.arccos(rng.uniform(-1.0, 1.0, n_dir)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="GisAPR source root (read only)")
    ap.add_argument("--out", type=Path, default=HERE / "golden_templates_crop.npz")
    args = ap.parse_args()
    import torch
    torch.set_num_threads(4)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        v606, _, _ = _import_reference(args.reference, tmp)
        dev = torch.device("cpu")
        for k, (n, nb, n_dir, half_res, seed) in enumerate(CASES):
            rot, tilt = case_directions(n_dir, seed)
            ang_path = tmp / f"angles{k}.star"
            _write_angle_star(ang_path, rot, tilt)
            angles = v606.read_model_angles(str(ang_path))
            layout = v606.PackedFourierLayout(nb, 8, dev)
            radius = int(round(0.43 * n))
            mask = torch.from_numpy(v606.generate_soft_mask((n, n), radius, MASK_EDGE))
            fsc = syn.logistic_fsc(n, APIX, half_res)
            fsc_path = tmp / f"fsc{k}.txt"
            with open(fsc_path, "w") as f:
                for i, v in enumerate(fsc):
                    f.write(f"{i} {float(v)!r}\n")
            packed_fsc = layout.centered_full_to_packed(torch.from_numpy(v606.read_fsc_map(str(fsc_path), n, nb,
                                                                                           False)))
            projector = v606.IntegratedProjector(dev, n, nb, layout, mask, packed_fsc, 8)
            vol = syn.blob_density(n, seed)
            t = projector.build_templates(torch.from_numpy(vol), angles)
            out[f"case{k}"] = np.asarray([n, nb, n_dir, half_res, seed, radius], np.float64)
            out[f"templates{k}"] = t.numpy().astype(np.complex64)
            print(n, nb, t.shape, flush=True)
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
