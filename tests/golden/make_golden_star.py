"""Generate the STAR-reader fixture by running GisAPR's reference reader.

    python tests/golden/make_golden_star.py --reference <GisAPR source root>

The reference search's read_model_angles and read_particle_table (v606, in
the optimized-3 tree) read STAR texts that exercise the loop rules: comment
and blank lines, labels with and without "#k" columns, repeated labels, an
optics loop before the particle loop, a loop without the required labels,
rows interrupted by another block, and a loop without rows. The fixture
stores the parsed rows (line index, image, angles, defocus) or "error".
"""
from __future__ import annotations

import argparse
import json
import sys
import tempfile
import types
import zipfile
from pathlib import Path

HERE = Path(__file__).resolve().parent

P = "000001@s.mrcs 10.0 20.0 30.0 10000 11000 45\n000002@s.mrcs 11.5 21.5 31.5 12000 13000 50\n"
TEXTS = dict(
    relion31=("# version 30001\n\ndata_optics\n\nloop_\n_rlnOpticsGroup #1\n_rlnImagePixelSize #2\n1 1.1\n\n"
              "data_particles\n\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAngleTilt #3\n_rlnAnglePsi #4\n"
              "_rlnDefocusU #5\n_rlnDefocusV #6\n_rlnDefocusAngle #7\n" + P),
    no_columns=("data_\nloop_\n_rlnImageName\n# a comment between labels\n_rlnAngleRot\n_rlnAngleTilt\n"
                "_rlnAnglePsi\n\n" + P.replace(" 10000 11000 45", "").replace(" 12000 13000 50", "")),
    shuffled=("data_\nloop_\n_rlnAngleTilt #3\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAnglePsi #4\n"
              "000003@s.mrcs 1.0 2.0 3.0\n# mid comment\n\n000004@s.mrcs 4.0 5.0 6.0\n"),
    repeated=("data_\nloop_\n_rlnImageName\n_rlnAngleRot\n_rlnImageName\n_rlnAngleTilt\n_rlnAnglePsi\n"
              "a@s.mrcs 1.0 b@s.mrcs 2.0 3.0\n"),
    interrupted=("data_\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAngleTilt #3\n"
                 "x@s.mrcs 1 2\n_rlnStray\ny@s.mrcs 3 4\n"),
    short_rows=("data_\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAngleTilt #3\n_rlnAnglePsi #4\n"
                "x@s.mrcs 1 2\ny@s.mrcs 3\nz@s.mrcs 5 6 7\n"),
    no_rows="data_\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAngleTilt #3\n\ndata_next\n",
    missing="data_\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\nx@s.mrcs 1\n",
    angles=("data_\nloop_\n_rlnAngleRot #1\n_rlnAngleTilt #2\n_rlnAnglePsi #3\n0 0 0\n-180 90.5 0\n"
            "12.25 170 5\n"),
    angles_no_psi="loop_\n_rlnAngleTilt #2\n_rlnAngleRot #1\n1 2\n3 4\n5\n",
)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE))
    args = ap.parse_args()
    stub = types.ModuleType("mrcfile")
    sys.modules["mrcfile"] = stub
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        with zipfile.ZipFile(Path(args.reference) / "GisAPR-210-optimized-3.zip") as z:
            z.extractall(td / "ref")
        sys.path.insert(0, str(td / "ref" / "GisAPR-210-optimized"))
        import importlib
        v606 = importlib.import_module(
            "test1_with_isspa_weight_varingKK_search_translation_also_v606_torch_optimized_standalone")
        cases = []
        for name, text in TEXTS.items():
            path = td / f"{name}.star"
            path.write_text(text)
            try:
                t = v606.read_particle_table(str(path))
                parts = dict(has_ctf=bool(t.has_ctf), data_start=int(t.loop.data_start),
                             rows=[[r.line_index, r.image_name, r.rot, r.tilt, r.psi, r.defocus_u, r.defocus_v,
                                    r.defocus_angle] for r in t.records])
            except ValueError:
                parts = "error"
            try:
                a = v606.read_model_angles(str(path))
                angles = dict(rot=list(a.rot), tilt=list(a.tilt), psi=list(a.psi))
            except ValueError:
                angles = "error"
            cases.append(dict(name=name, particles=parts, angles=angles))
    (Path(args.out) / "golden_star.json").write_text(json.dumps(dict(texts=TEXTS, cases=cases), indent=1) + "\n")
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
