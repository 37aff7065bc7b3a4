"""Generate golden_scorer.npz by running the reference's search-text scorer.

    python tests/golden/make_golden_scorer.py --reference <GisAPR source root>

new_method_to_fit_the_2nd_Gaussian_PEAK_v4.py (read, never modified) is
copied to a temporary directory and its run_this scores seeded synthetic
search texts in all four modes (rawCC or z-score, fitted or simple sum),
plus a text whose fit fails (every rawCC outside the histogram range) and an
empty text. The fixture stores the texts and the reference's outputs.
"""
from __future__ import annotations

import argparse
import contextlib
import io
import shutil
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
MODULE = "new_method_to_fit_the_2nd_Gaussian_PEAK_v4"
MODES = [(1.0, 1.0), (1.0, 0.0), (0.0, 0.0), (0.0, 1.0)]


def search_text(raw_over_1024, zscores, first_line=20) -> str:
    """Three records per particle in the search text layout."""
    out = []
    for i, (r, z) in enumerate(zip(raw_over_1024, zscores)):
        line = first_line + i
        out.append(str(["cc: ", line, float(z), int(z > 3.0), 1, 12.5, 80.0, 4.2, 1, -2, 0, 0]) + "\n")
        out.append(str(["psi: ", line, 45.0, 47.5]) + "\n")
        out.append(str(["rawCC: ", line, float(r * 1024.0)]) + "\n")
    return "".join(out)


def make_texts(seed=7):
    rng = np.random.default_rng(seed)
    n = 3000
    sig = rng.random(n) < 0.3
    raw = np.where(sig, rng.normal(0.42, 0.05, n), rng.normal(0.30, 0.02, n))
    z = np.where(sig, rng.normal(4.5, 1.5, n), rng.normal(2.0, 0.3, n))
    texts = {"mixture": search_text(raw, z)}
    raw2 = np.where(rng.random(800) < 0.5, rng.normal(0.25, 0.03, 800), rng.normal(0.33, 0.04, 800))
    texts["small"] = search_text(raw2, rng.normal(2.5, 0.8, 800))
    texts["fit_fails"] = search_text(np.full(50, 1.5), np.full(50, 2.0))
    texts["empty"] = ""
    return texts


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE / "golden_scorer.npz"))
    args = ap.parse_args()
    texts = make_texts()
    names, outs = [], []
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        shutil.copy(Path(args.reference) / (MODULE + ".py"), td / (MODULE + ".py"))
        sys.path.insert(0, str(td))
        sys.dont_write_bytecode = True
        ref = __import__(MODULE)
        for name, text in texts.items():
            path = td / (name + ".txt")
            path.write_text(text)
            for cc, ss in MODES:
                with contextlib.redirect_stdout(io.StringIO()):
                    res = ref.run_this(str(path), cc, ss)
                names.append(f"{name}|{cc}|{ss}")
                outs.append([float(v) for v in res])
                print(name, cc, ss, res)
    np.savez_compressed(args.out, text_names=np.asarray(list(texts)), texts=np.asarray(list(texts.values())),
                        cases=np.asarray(names), outputs=np.asarray(outs, dtype=np.float64))


if __name__ == "__main__":
    main()
