"""Generate golden_ctf.npz by running the reference's own CTF * ISSPA tables.

    python tests/golden/make_golden_ctf.py --reference <GisAPR source root>

v606's ``PackedCTFTorch.batch`` and ``PackedCTFNumPy.batch`` (v606:695-829;
the optimized-3 tree, imported as make_golden.py does) for seeded defocus
values (U and V in 0.8-3.0 um, any astigmatism angle) at the boxes, pixel
sizes and ISSPA constants of the other configurations: box 96 at 1.4 A,
box 128 at 1.1 A, box 256 at 0.85 A with kk 0 and 10. Each table stores the
rows of the lowest and of the highest packed frequencies (ROWS), where the
phase is smallest and largest.
"""
from __future__ import annotations

import argparse
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_golden import _import_reference  # noqa: E402

# (box, pixel size A, kk, seed)
CASES = ((96, 1.4, 3.0, 31), (128, 1.1, 3.0, 32), (256, 0.85, 0.0, 33), (256, 0.85, 10.0, 34))
N_PARTICLES = 4
CS, VOLTAGE = 2.7, 300.0


def rows(n: int) -> np.ndarray:
    """Packed rows kept: the first 8 (lowest frequencies) and the 8 around n/2 (highest)."""
    return np.concatenate([np.arange(8), np.arange(n // 2 - 4, n // 2 + 4)])


def case_defocus(seed: int):
    """Seeded (dfu, dfv, angle) per particle, Angstrom and degrees."""
    rng = np.random.default_rng(seed)
    dfu = rng.uniform(8000.0, 30000.0, N_PARTICLES)
    dfv = rng.uniform(8000.0, 30000.0, N_PARTICLES)
    ang = rng.uniform(0.0, 180.0, N_PARTICLES)
    return [(float(u), float(v), float(a)) for u, v, a in zip(dfu, dfv, ang)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="GisAPR source root (read only)")
    ap.add_argument("--out", type=Path, default=HERE / "golden_ctf.npz")
    args = ap.parse_args()
    import torch
    with tempfile.TemporaryDirectory() as td:
        v606, _, _ = _import_reference(args.reference, Path(td))
        out = {}
        for k, (n, apix, kk, seed) in enumerate(CASES):
            recs = [types.SimpleNamespace(defocus_u=u, defocus_v=v, defocus_angle=a) for u, v, a in case_defocus(seed)]
            t = v606.PackedCTFTorch(n, apix, CS, VOLTAGE, kk, torch.device("cpu")).batch(recs, True).numpy()
            m = np.asarray(v606.PackedCTFNumPy(n, apix, CS, VOLTAGE, kk).batch(recs, True))
            out[f"case{k}"] = np.asarray([n, apix, kk, seed], np.float64)
            out[f"torch{k}"] = t[:, rows(n)].astype(np.float32)
            out[f"numpy{k}"] = m[:, rows(n)].astype(np.float32)
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
