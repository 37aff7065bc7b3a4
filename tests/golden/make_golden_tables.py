"""Generate golden_tables.npz by running the reference's own search tables.

    python tests/golden/make_golden_tables.py --reference <GisAPR source root>

v606's ``build_local_orientation_entries`` (v606:331-378) and
``psi_sampling_for_record`` (v606:1163-1190; the optimized-3 tree, imported
as make_golden.py does) for seeded particle orientations against the HEALPix
direction sets of the larger configurations: order 3 within +-10 degrees with
psi step 7.5 (box 128) and order 4 within +-6 degrees with psi step 3.75
(box 256). The model directions come from the synthetic generator's HEALPix
list (itself checked against the reference's); particle angles are
regenerated from the seeds. The file stores each particle's direction list
(CSR) and its psi sampling.
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
sys.path.insert(0, str(HERE.parent.parent))

from make_golden import _import_reference  # noqa: E402

# (HEALPix order, local range deg, psi step deg, particles, seed)
CASES = ((3, 10.0, 7.5, 300, 51), (4, 6.0, 3.75, 300, 52))


def case_particles(n: int, seed: int):
    """Seeded particle (rot, tilt, psi) in degrees, RELION ranges, rounded
    to 6 decimals as a STAR file holds them."""
    rng = np.random.default_rng(seed)
    rot = np.round(rng.uniform(-180.0, 180.0, n), 6)
    tilt = np.round(np.degrees(np.arccos(rng.uniform(-1.0, 1.0, n))), 6)
    psi = np.round(rng.uniform(-180.0, 180.0, n), 6)
    return rot, tilt, psi


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="GisAPR source root (read only)")
    ap.add_argument("--out", type=Path, default=HERE / "golden_tables.npz")
    args = ap.parse_args()
    from gisapr_gb300 import synthetic as syn
    with tempfile.TemporaryDirectory() as td:
        v606, _, _ = _import_reference(args.reference, Path(td))
        out = {}
        for k, (order, local, step, n, seed) in enumerate(CASES):
            m_rot, m_tilt = syn.healpix_directions(order)
            rot, tilt, psi = case_particles(n, seed)
            recs = [types.SimpleNamespace(line_index=i + 10, rot=float(r), tilt=float(t), psi=float(p))
                    for i, (r, t, p) in enumerate(zip(rot, tilt, psi))]
            entries = v606.build_local_orientation_entries(recs, m_rot, m_tilt, local)
            ptr = np.cumsum([0] + [len(e) - 1 for e in entries])
            idx = np.asarray([d for e in entries for d in e[1:]], np.int64)
            fake, eff = zip(*(v606.psi_sampling_for_record(r.psi, step, True, local) for r in recs))
            out[f"case{k}"] = np.asarray([order, local, step, n, seed], np.float64)
            out[f"ptr{k}"] = ptr.astype(np.int64)
            out[f"idx{k}"] = idx
            out[f"fake{k}"] = np.asarray(fake, np.float64)
            out[f"eff{k}"] = np.asarray(eff, np.float64)
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
