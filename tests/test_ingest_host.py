"""Host side of the particle preparation (no GPU): shift + crop and the
bin and mask tables, against the reference's outputs."""
from pathlib import Path

import numpy as np

from gisapr_gb300 import ingest

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_ingest.npz"


def test_translation_and_crop_match_reference():
    g = np.load(GOLDEN)
    c = int(g["crop"])
    for i, img in enumerate(g["images"]):
        t = ingest.translation_twoD_image(img, *g["shifts"][i])
        np.testing.assert_array_equal(t[32 - c // 2:32 + c // 2, 32 - c // 2:32 + c // 2], g["cropped"][i])


def test_radial_bins_cover_every_pixel_once():
    for h, w in [(48, 48), (45, 45), (16, 24)]:
        ptr, pix, cnt = ingest.radial_bins(h, w)
        assert ptr[-1] == h * w and sorted(pix.tolist()) == list(range(h * w))
        assert np.array_equal(np.diff(ptr), cnt.astype(np.int64))
        assert pix[0] == 0  # bin 0 is the zero frequency alone
        assert cnt[0] == 1


def test_highpass_mask_shape_and_dc():
    m = ingest.highpass_mask(48, 48, 20.0, 1.5)
    assert m.shape == (48, 48) and m[0, 0] == 0.0 and m.max() == 1.0 and m.min() == 0.0


def test_only_make_star_needs_no_device(tmp_path):
    star = tmp_path / "in.star"
    rows = "".join(f"{i + 1}@stack.mrcs\t1.0\t-2.0\n" for i in range(7))
    star.write_text("data_optics\nloop_\n_rlnOpticsGroup #1\n_rlnImagePixelSize #2\n_rlnImageSize #3\n1\t1.0\t64\n"
                    "\ndata_particles\nloop_\n_rlnImageName #1\n_rlnOriginXAngst #2\n_rlnOriginYAngst #3\n" + rows)
    args = ingest.create_gridsearch_parser().parse_args(
        ["--star_name", str(star), "--output_root_name", str(tmp_path / "o"), "--batchsize", "3",
         "--doOnlyMakeStar", "--newboxsize", "32"])
    res = ingest.run_preprocess(args)
    assert res["particles"] == 7
    text = (tmp_path / "o.star").read_text()
    assert "3@" + str(tmp_path / "o") + "_0002.mrcs\t0.0\t0.0" in text
    assert "1@" + str(tmp_path / "o") + "_0003.mrcs" in text
    assert "1\t1.0\t32" in text
