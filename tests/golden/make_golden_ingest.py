"""Generate golden_ingest.npz by running the reference's particle preparation.

    python tests/golden/make_golden_ingest.py --reference <GisAPR source root>

read_star_shift_crop_and_generate_new_star_v5.py (read, never modified) is
copied to a temporary directory and imported with stub ``starfile`` and
``mrcfile`` modules (only its image functions are called). Seeded particle
images go through the per-particle body of its loop (v5:202-235): shift by
the origin in pixels, centred crop, whitening (getSpectrum_divideBySpectrum
then normalize) and the high-pass filter, in the combinations stored below,
plus the two whitening functions alone on an odd-sized image.
"""
from __future__ import annotations

import argparse
import shutil
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
MODULE = "read_star_shift_crop_and_generate_new_star_v5"
CROP, PIXEL, HIGHPASS = 48, 1.5, 20.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE / "golden_ingest.npz"))
    args = ap.parse_args()
    for name in ("starfile", "mrcfile"):
        sys.modules[name] = types.ModuleType(name)
    rng = np.random.default_rng(5)
    n = 5
    yy, xx = np.mgrid[0:64, 0:64]
    images = (rng.normal(0.0, 1.0, (n, 64, 64)) + 0.02 * xx - 0.01 * yy
              + 3.0 * np.exp(-((xx - 30) ** 2 + (yy - 34) ** 2) / 60.0)).astype(np.float32)
    shifts = rng.uniform(-6.0, 6.0, (n, 2))
    shifts[0] = (2.5, -3.5)  # half-pixel values round up
    odd = rng.normal(0.0, 1.0, (2, 45, 45)).astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        shutil.copy(Path(args.reference) / (MODULE + ".py"), Path(td) / (MODULE + ".py"))
        sys.path.insert(0, td)
        sys.dont_write_bytecode = True
        v5 = __import__(MODULE)

        def crop(img):
            h, w = img.shape
            return img[h // 2 - CROP // 2:h // 2 + CROP // 2, w // 2 - CROP // 2:w // 2 + CROP // 2]

        def body(img, sx, sy, whiten, highpass):
            out = crop(v5.translation_twoD_image(img, sx, sy))
            if whiten:
                out = v5.normalize(v5.getSpectrum_divideBySpectrum(out))
            if highpass:
                out = v5.highpassfilter(out, HIGHPASS, PIXEL)
            return np.asarray(out, dtype=np.float32)

        res = {}
        for key, (wh, hp) in {"cropped": (False, False), "whiten": (True, False), "highpassed": (False, True),
                              "both": (True, True)}.items():
            res[key] = np.stack([body(images[i], shifts[i, 0], shifts[i, 1], wh, hp) for i in range(n)])
        res["odd_spectrum"] = np.stack([np.asarray(v5.getSpectrum_divideBySpectrum(o), np.float32) for o in odd])
        res["odd_normalize"] = np.stack([np.asarray(v5.normalize(o.astype(np.float64)), np.float32) for o in odd])
        res["odd_highpass"] = np.stack([np.asarray(v5.highpassfilter(o, 9.0, 1.0), np.float32) for o in odd])
    np.savez_compressed(args.out, images=images, shifts=shifts, odd=odd, crop=CROP, pixel=PIXEL,
                        highpass=HIGHPASS, **res)
    for k, v in res.items():
        print(k, v.shape, float(np.abs(v).max()))


if __name__ == "__main__":
    main()
