"""Host side of the geometric restraint (no GPU): the reference's float32
pose transform, the output formatting and the command's arguments."""
from pathlib import Path

import numpy as np
import pytest

from gisapr_gb300 import restraint as rs

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_restraint.npz"


def test_rotate_coords_matches_reference(tmp_path):
    g = np.load(GOLDEN)
    pdb = tmp_path / "m.pdb"
    pdb.write_text(str(g["pdb_text"]))
    chain, _, rest, _ = rs.read_pdb_split_chain_and_rest(str(pdb), "A")
    assert chain.dtype == np.float32 and len(rest) > len(chain)
    np.testing.assert_array_equal(rs.rotate_coords_rotvec(chain, *g["poses"][3]), g["moved"][0])
    np.testing.assert_array_equal(rs.rotate_coords_rotvec(chain, *g["pivot_poses"][0], pivot=g["pivot"]),
                                  g["moved"][1])
    with pytest.raises(ValueError):
        rs.rotate_coords_rotvec(chain, 0, 0, 0, 0, 0, 0, pivot=[1.0, 2.0])
    with pytest.raises(ValueError):
        rs.read_pdb_split_chain_and_rest(str(pdb), "Z")


def test_format_and_parser():
    f = rs.convert_float_into_my_format
    assert [f(12.34), f(-0.5), f(3.0), f(-7.25)] == ["12p3", "N0p5", "3p0", "N7p2"]
    a = rs.create_BOUNDARY_CHECK_parser().parse_args(["--i", "m.pdb", "--chainID", "A", "--rot", "1", "--tilt", "2",
                                                      "--psi", "3", "--outputRoot", "o", "--outputFile", "f.txt"])
    assert (a.maskBoxsize, a.apix, a.thresholdForMask, a.thresholdChainIsTooFar, a.thresholdPixelHits) == \
        (256, 1.5, 1.0, 50.0, 5)
    assert a.pivot is None and not a.skip_geometric_restraint


def test_skip_writes_the_reference_line(tmp_path):
    out = tmp_path / "r.txt"
    rs.main(["--i", "m.pdb", "--chainID", "B", "--rot", "-1.25", "--tilt", "2", "--psi", "0", "--centerX", "10.5",
             "--outputRoot", "o", "--outputFile", str(out), "--skip-geometric-restraint"])
    assert out.read_text() == "B\tN1p2\t2p0\t0p0\t10p5\t0p0\t0p0\t0\t0.0\n"


def test_cpu_device_is_rejected(tmp_path):
    with pytest.raises(ValueError):
        rs.GeometryRestraint(str(tmp_path / "none.pdb"), "A", device="cpu")
