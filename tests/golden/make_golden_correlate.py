"""Generate golden_correlate.npz by running the reference's own correlation.

    python tests/golden/make_golden_correlate.py --reference <GisAPR source root>

v606's ``correlate_templates_and_particle`` (v606:1418-1449; the optimized-3
tree, imported as make_golden.py does) is run on seeded random complex
templates and particle spectra in the packed layout at the sizes and crops of
the configurations the other fixtures do not cover: box 256 with crop 14 (the
precision configuration), 192, 96 and 64. The inputs are regenerated from the
seeds (numpy's default_rng), so the file stores only the reference's scores
and peak positions.
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

# (n, crop, n_psi, templates, seed)
CASES = ((256, 14, 3, 5, 11), (192, 10, 4, 3, 12), (96, 12, 3, 4, 13), (64, 14, 2, 3, 14))


def case_inputs(n: int, n_psi: int, n_t: int, seed: int):
    """Seeded templates [n_t][n][n/2+1] and particle spectra [n_psi][n][n/2+1], complex64."""
    rng = np.random.default_rng(seed)
    h = n // 2 + 1

    def c(shape):
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    return c((n_t, n, h)), c((n_psi, n, h))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="GisAPR source root (read only)")
    ap.add_argument("--out", type=Path, default=HERE / "golden_correlate.npz")
    args = ap.parse_args()
    import torch
    torch.set_num_threads(4)
    with tempfile.TemporaryDirectory() as td:
        v606, _, _ = _import_reference(args.reference, Path(td))
        dev = torch.device("cpu")
        out = {}
        for k, (n, crop, n_psi, n_t, seed) in enumerate(CASES):
            t, p = case_inputs(n, n_psi, n_t, seed)
            layout = v606.PackedFourierLayout(n, crop, dev)
            ws = v606.CorrelationWorkspace(dev)
            s, y, x = v606.correlate_templates_and_particle(torch.from_numpy(t), torch.from_numpy(p), layout, ws)
            out[f"case{k}"] = np.asarray([n, crop, n_psi, n_t, seed], np.int64)
            out[f"scores{k}"] = s.numpy().astype(np.float32)
            out[f"ys{k}"] = y.numpy().astype(np.int64)
            out[f"xs{k}"] = x.numpy().astype(np.int64)
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
