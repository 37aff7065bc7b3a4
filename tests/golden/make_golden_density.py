"""Generate golden_density.npz by running the reference's own splat.

    python tests/golden/make_golden_density.py --reference <GisAPR source root>

pdb2mrc v3's ``density_from_coords`` (R/pdb2mrc_gpu_ver_fp32_v3.py:41-98, the
optimized-3 tree, imported as make_golden.py does) on seeded atoms at the
box sizes and pixel sizes the stage fixtures do not cover: box 256 at
0.85 A (the precision configuration) and box 96 at 1.4 A. The atoms are
spread over the whole box, some within a kernel width of its faces (where
the reference clips the voxel range), with element numbers drawn from H, C,
N, O, P and S. Coordinates are regenerated from the seeds; the file stores
the density's float64 sum and sum of squares and three planes (the central
z plane and planes near both z faces).
"""
from __future__ import annotations

import argparse
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_golden import _import_reference  # noqa: E402

# (box, pixel size A, resolution A, atoms, seed)
CASES = ((256, 0.85, 3.0, 2000, 41), (96, 1.4, 4.0, 1500, 42))
ELEMENTS = np.asarray([1, 6, 7, 8, 15, 16], np.float32)


def case_atoms(n: int, apix: float, n_atoms: int, seed: int):
    """Seeded coordinates (Angstrom, origin at the box centre, float32 after an
    8.3 PDB round trip) and atomic numbers."""
    rng = np.random.default_rng(seed)
    half = n / 2 * apix
    xyz = rng.uniform(-half * 0.99, half * 0.99, size=(n_atoms, 3))
    xyz = np.round(xyz, 3).astype(np.float32)
    z = ELEMENTS[rng.integers(0, len(ELEMENTS), n_atoms)]
    return xyz, z


def planes(n: int) -> np.ndarray:
    return np.asarray([1, n // 2, n - 2])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="GisAPR source root (read only)")
    ap.add_argument("--out", type=Path, default=HERE / "golden_density.npz")
    args = ap.parse_args()
    import torch
    torch.set_num_threads(4)
    with tempfile.TemporaryDirectory() as td:
        _, pdb2mrc, _ = _import_reference(args.reference, Path(td))
        out = {}
        for k, (n, apix, res, n_atoms, seed) in enumerate(CASES):
            xyz, z = case_atoms(n, apix, n_atoms, seed)
            d = pdb2mrc.density_from_coords(xyz, z, n, apix, res, device="cpu")
            d = d.numpy() if hasattr(d, "numpy") else np.asarray(d)
            d64 = d.astype(np.float64)
            out[f"case{k}"] = np.asarray([n, apix, res, n_atoms, seed], np.float64)
            out[f"sums{k}"] = np.asarray([d64.sum(), (d64 * d64).sum()])
            out[f"planes{k}"] = d[planes(n)].astype(np.float32)
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
