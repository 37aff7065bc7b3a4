"""Generate golden_records.json by running the reference's own record
formatter.

    python tests/golden/make_golden_records.py --reference <GisAPR source root>

v606's ``make_result_records`` (v606:1452-1516; the optimized-3 tree,
imported as make_golden.py does) on seeded per-particle maxima (float32
scores per direction and psi angle, peak rows and columns inside the crop,
some maxima tied) at crops and translation scales the stage fixtures do not
cover: crop 14 with scale 0.5, crop 12 with scale 2/3 (half-integer shifts,
which Python's round sends to the even neighbour), crop 10 with scale 1.
Inputs are regenerated from the seeds; the file stores the reference's
three records per particle.
"""
from __future__ import annotations

import argparse
import json
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

from make_golden import _import_reference  # noqa: E402

# (crop, translation scale, psi step, local range, particles, seed); every
# case samples three psi angles per particle
CASES = ((14, 0.5, 3.75, 6.0, 40, 61), (12, 2.0 / 3.0, 7.5, 10.0, 40, 62), (10, 1.0, 15.0, 15.0, 40, 63))
HEALPIX_ORDER = 2


def case_inputs(crop: int, n: int, seed: int, n_dirs_total: int):
    """Per particle: a record (line_index, rot, tilt, psi), its direction
    list, float32 scores [dirs][3], peak rows and columns [dirs][3]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        d = int(rng.integers(1, 13))
        dirs = np.sort(rng.choice(n_dirs_total, size=d, replace=False)).tolist()
        scores = rng.normal(5000.0, 300.0, size=(d, 3)).astype(np.float32)
        if i % 4 == 0 and scores.size > 1:  # a tied maximum later in row-major order
            flat = scores.reshape(-1)
            j = int(np.argmax(flat))
            flat[(j + 1 + int(rng.integers(0, flat.size - 1))) % flat.size] = flat[j]
        ys = rng.integers(0, crop, size=(d, 3))
        xs = rng.integers(0, crop, size=(d, 3))
        rec = dict(line_index=100 + i, rot=float(np.round(rng.uniform(-180, 180), 6)),
                   tilt=float(np.round(rng.uniform(0, 180), 6)), psi=float(np.round(rng.uniform(-180, 180), 6)))
        out.append((rec, dirs, scores, ys, xs))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="GisAPR source root (read only)")
    ap.add_argument("--out", type=Path, default=HERE / "golden_records.json")
    args = ap.parse_args()
    import torch
    from gisapr_gb300 import synthetic as syn
    m_rot, m_tilt = syn.healpix_directions(HEALPIX_ORDER)
    with tempfile.TemporaryDirectory() as td:
        v606, _, _ = _import_reference(args.reference, Path(td))
        out = []
        for crop, scale, step, local, n, seed in CASES:
            rows = []
            for rec, dirs, scores, ys, xs in case_inputs(crop, n, seed, len(m_rot)):
                fake, _ = v606.psi_sampling_for_record(rec["psi"], step, True, local)
                assert len(fake) == scores.shape[1]
                r = v606.make_result_records(types.SimpleNamespace(**rec), fake, m_rot, m_tilt, dirs,
                                             torch.from_numpy(scores), torch.from_numpy(ys), torch.from_numpy(xs),
                                             crop, scale)
                rows.append(r)
            out.append({"case": [crop, scale, step, local, n, seed], "records": rows})
    args.out.write_text(json.dumps(out))
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
