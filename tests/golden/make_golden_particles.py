"""Generate golden_particles.npz by running the reference's own particle
preparation.

    python tests/golden/make_golden_particles.py --reference <GisAPR source root>

v606's ``ParticleFourierPreparer.prepare`` (v606:1321-1374: psi rotation by
grid_sample, soft mask, 2-D FFT, Fourier crop to the new box, CTF * ISSPA
weight, conjugate, normalise, pre-shift; the optimized-3 tree, imported as
make_golden.py does) on seeded random images, packed weights and in-plane
angles at boxes the stage fixtures do not cover: 96, 192 cropped to 96 in
Fourier space, and 256 (the precision configuration's box). Inputs are
regenerated from the seeds; the file stores the reference's spectra (at box
256 the first 32 packed rows of each psi angle, and every angle's norm).
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

# (box, new box, mask radius, mask edge, seed)
CASES = ((96, 96, 41, 6, 21), (192, 96, 82, 6, 22), (256, 256, 110, 6, 23))
ROWS_KEPT = 32  # packed rows stored per psi angle at box 256


def case_inputs(n: int, nb: int, seed: int):
    """Seeded image [n][n] float32, packed weights [nb][nb/2+1] float32 in
    [0.05, 1) and three in-plane angles (degrees, 6 decimals)."""
    rng = np.random.default_rng(seed)
    image = rng.standard_normal((n, n)).astype(np.float32)
    weights = (0.05 + 0.95 * rng.random((nb, nb // 2 + 1))).astype(np.float32)
    angles = [float(np.round(a, 6)) for a in rng.uniform(-180.0, 180.0, size=3)]
    return image, weights, angles


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="GisAPR source root (read only)")
    ap.add_argument("--out", type=Path, default=HERE / "golden_particles.npz")
    args = ap.parse_args()
    import torch
    torch.set_num_threads(4)
    with tempfile.TemporaryDirectory() as td:
        v606, _, _ = _import_reference(args.reference, Path(td))
        dev = torch.device("cpu")
        out = {}
        for k, (n, nb, radius, edge, seed) in enumerate(CASES):
            image, weights, angles = case_inputs(n, nb, seed)
            layout = v606.PackedFourierLayout(nb, 8, dev)
            mask = torch.from_numpy(v606.generate_soft_mask((n, n), radius, edge))
            bank = v606.PsiGridBank(n, dev, angles, 8)
            prep = v606.ParticleFourierPreparer(n, nb, dev, layout, mask, bank)
            spec = prep.prepare(torch.from_numpy(image), angles, torch.from_numpy(weights)).numpy()
            out[f"case{k}"] = np.asarray([n, nb, radius, edge, seed], np.int64)
            out[f"norms{k}"] = np.sqrt((np.abs(spec.astype(np.complex128)) ** 2).sum(axis=(1, 2)))
            out[f"spectra{k}"] = spec[:, :ROWS_KEPT] if n == 256 else spec
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
