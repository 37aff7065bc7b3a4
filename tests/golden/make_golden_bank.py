"""Generate the orientation-bank fixture by running GisAPR's reference code.

    python tests/golden/make_golden_bank.py --reference <GisAPR source root>

The Lite tree (GisAPR-Lite-v1.3.2.zip) is extracted to a temporary
directory and its orientation_bank_v1 module writes a bank exactly as its
search does with --orientations-out: settings of a particle STAR and an
angle STAR (by content hash), rows ranked by ranked_row from seeded per-map
peaks (with a repeated (rot, tilt) pair and ties), packed with its digest.
The fixture stores both STAR texts, the per-particle inputs of ranked_row,
the bank JSON, and restricted_indices outcomes (index list, or "error") for
valid and corrupted rows.
"""
from __future__ import annotations

import argparse
import json
import sys
import tempfile
import zipfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

ANGLES = [(0.0, 0.0), (10.0, 5.0), (20.0, 7.5), (10.0, 5.0), (-30.0, 90.0), (45.5, 120.25), (60.0, 12.0)]
PARTICLES = [  # (line image rot tilt psi), line indices follow the text below
    ("000001@stack.mrcs", 1.0, 2.0, 3.0),
    ("000002@stack.mrcs", 15.0, 6.0, 40.0),
    ("000003@stack.mrcs", -20.0, 88.0, 100.0),
    ("000004@stack.mrcs", 50.0, 20.0, 200.0),
]


def angle_star() -> str:
    rows = "".join(f"{r!r}\t{t!r}\t0.0\n" for r, t in ANGLES)
    return "\ndata_\n\nloop_\n_rlnAngleRot #1\n_rlnAngleTilt #2\n_rlnAnglePsi #3\n" + rows


def particle_star() -> str:
    head = "\ndata_\n\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAngleTilt #3\n_rlnAnglePsi #4\n"
    return head + "".join(f"{n}\t{r!r}\t{t!r}\t{p!r}\n" for n, r, t, p in PARTICLES)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE))
    args = ap.parse_args()
    import torch
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        with zipfile.ZipFile(Path(args.reference) / "GisAPR-Lite-v1.3.2.zip") as z:
            z.extractall(td / "ref")
        sys.path.insert(0, str(td / "ref" / "GisAPR-210-DE-v1.3.2"))
        import orientation_bank_v1 as ob
        from types import SimpleNamespace
        (td / "p.star").write_text(particle_star())
        (td / "a.star").write_text(angle_star())
        keep = 3
        ctx = ob.settings(str(td / "p.star"), str(td / "a.star"), keep, True, 20.0, 7.5)
        angles = SimpleNamespace(rot=[a[0] for a in ANGLES], tilt=[a[1] for a in ANGLES])
        lines = particle_star().splitlines()
        first = next(i for i, ln in enumerate(lines) if ln.startswith("000001"))
        rng = np.random.default_rng(5)
        rows, inputs = {}, []
        for k, (name, _, _, _) in enumerate(PARTICLES):
            rec = SimpleNamespace(line_index=first + k, image_name=name)
            indices = [[0, 1, 2, 3, 6], [1, 2, 3], [4, 5], [0, 6]][k]
            scores = rng.normal(size=(len(indices), 3)).astype(np.float32)
            if k == 0:
                scores[1] = scores[3] = 9.0  # the repeated (rot, tilt) pair with a tie
            if k == 1:
                scores[:, 0] = 2.0           # ties in the psi maximum
            rows[str(rec.line_index)] = ob.ranked_row(rec, indices, angles, torch.from_numpy(scores), keep)
            inputs.append(dict(line=rec.line_index, image=name, indices=indices, scores=scores.tolist()))
        bank = ob.pack_bank(ctx, rows, mrc="/data/model.mrc")
        cases = []
        for key, row in rows.items():
            k = int(key) - first
            rec = SimpleNamespace(line_index=int(key), image_name=PARTICLES[k][0])
            allowed = inputs[k]["indices"]
            variants = [row, None, dict(row, image="x@y"), dict(row, directions=[]),
                        dict(row, directions=row["directions"] + row["directions"]),
                        dict(row, directions=[[d[0], d[1] + 1.0, d[2], d[3]] for d in row["directions"]]),
                        dict(row, directions=[[float(d[0]), d[1], d[2], d[3]] for d in row["directions"]])]
            for v in variants:
                try:
                    out = ob.restricted_indices(v, rec, allowed, angles, keep)
                except ValueError:
                    out = "error"
                cases.append(dict(line=int(key), row=v, allowed=allowed, result=out))
        fixture = dict(particle_star=particle_star(), angle_star=angle_star(), keep=keep, local=True,
                       local_range=20.0, psi_step=7.5, inputs=inputs, bank=bank, restricted=cases)
        (Path(args.out) / "golden_bank.json").write_text(json.dumps(fixture, indent=1) + "\n")
        print("bank digest", bank["sha256"])


if __name__ == "__main__":
    main()
