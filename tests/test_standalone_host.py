"""Host side of the file-based entry points (no GPU): argument names and
defaults, particle stack reading, the local-direction cache, particle
chunking, and the direction-bank rows of the round evaluation."""
import pickle

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gisapr_gb300 import batch_search as bs  # noqa: E402
from gisapr_gb300 import standalone as sa  # noqa: E402
from gisapr_gb300.mrc import write_mrc  # noqa: E402
from gisapr_gb300.tables import (ParticleRecord, model_angles_from_lists, read_model_angles,  # noqa: E402
                                 read_particle_table)
from tests.helpers import write_search_inputs  # noqa: E402

# Defaults of the standalone command's arguments (v606:1525-1567).
REFERENCE_DEFAULTS = dict(FSC="", kk=0.0, gpuid=0, oriboxsize=256, newboxsize=256, apix=1.42, transRange=0,
                          voltage=300.0, cs=2.7, maskRadius=110, maskEdge=6, ignoreFSC=False, discardMask=False,
                          psiStep=15.0, start=-1, end=-1, doLocalSearch=False, localRange=20.0, doContinue=False,
                          ctfBackend="torch", ctfBatchSize=256, projectionBatchSize=8, psiGridBuildBatch=8,
                          ccgCropSize=32, chunkSizeA=16, chunkSizeB=32, outputBufferParticles=96, torchThreads=4,
                          profileStages=False)


def test_parser_names_and_defaults():
    a = sa.create_search_parser().parse_args(["--i", "x", "--p", "p.star", "--o", "o.txt", "--ang", "a.star",
                                              "--mrc", "m.mrc"])
    for k, v in REFERENCE_DEFAULTS.items():
        assert getattr(a, k) == v, k
    with pytest.raises(SystemExit):  # --mrc and --ang are required, as in the reference
        sa.create_search_parser().parse_args(["--i", "x", "--p", "p", "--o", "o"])


def test_input_files_round_trip(golden32, tmp_path):
    g = golden32
    args = write_search_inputs(tmp_path, g)
    table = read_particle_table(args.p)
    assert [r.line_index for r in table.records] == [int(v) for v in g["rec_line"]]
    assert table.has_ctf
    angles = read_model_angles(args.ang)
    assert angles.rot == [float(v) for v in g["model_rot"]]
    reader = sa.ParticleMRCReader(32, "cpu")
    out = torch.empty((len(table.records), 32, 32), dtype=torch.float32)
    stack = reader.read_stack(table.records, out)
    np.testing.assert_array_equal(stack.numpy(), g["images"])
    np.testing.assert_array_equal(reader.read(table.records[3].image_name).numpy(), g["images"][3])
    reader.close()


def test_reader_single_image_and_shape_check(tmp_path):
    img = np.arange(64, dtype=np.float32).reshape(8, 8)
    write_mrc(tmp_path / "one.mrc", img)
    reader = sa.ParticleMRCReader(8, "cpu")
    np.testing.assert_array_equal(reader.read(f"1@{tmp_path / 'one.mrc'}").numpy(), img)
    bad = sa.ParticleMRCReader(16, "cpu")
    with pytest.raises(ValueError):
        bad.read(f"1@{tmp_path / 'one.mrc'}")


def test_local_cache_written_reused_and_rebuilt(golden32, tmp_path, monkeypatch):
    g = golden32
    args = write_search_inputs(tmp_path, g)
    table = read_particle_table(args.p)
    angles = read_model_angles(args.ang)
    first = sa.load_or_build_local_orientation_map(args.p, table.records, angles, args.localRange)
    cache = tmp_path / "particles.star_LocalSearch_Angle_30_data.pkl"
    assert cache.exists()
    # a valid cache is read, not rebuilt
    monkeypatch.setattr(sa, "build_local_orientation_entries",
                        lambda *a, **k: (_ for _ in ()).throw(AssertionError("rebuilt")))
    assert sa.load_or_build_local_orientation_map(args.p, table.records, angles, args.localRange) == first
    monkeypatch.undo()
    # a cache of another particle set is replaced
    with open(cache, "wb") as fh:
        pickle.dump([[999, 0]], fh)
    again = sa.load_or_build_local_orientation_map(args.p, table.records, angles, args.localRange)
    assert again == first
    with open(cache, "rb") as fh:
        assert len(pickle.load(fh)) == len(table.records)
    # lists follow the fixture's CSR arrays
    ptr, idx = g["local_ptr"], g["local_idx"]
    for k, line in enumerate(g["rec_line"]):
        assert first[int(line)] == [int(v) for v in idx[ptr[k]:ptr[k + 1]]]


def test_particle_chunks():
    recs = [ParticleRecord(i, f"{i}@s", 0.0, 0.0, 0.0) for i in range(10)]
    chunks = sa.particle_chunks(recs, per_particle_bytes=2 ** 20, budget_mb=3)
    assert [len(c) for c in chunks] == [3, 3, 3, 1]
    assert [r.line_index for c in chunks for r in c] == list(range(10))
    assert [len(c) for c in sa.particle_chunks(recs, 2 ** 30, 1)] == [1] * 10


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")
def test_run_search_needs_a_cuda_device(golden32, tmp_path):
    args = write_search_inputs(tmp_path, golden32)
    with pytest.raises(RuntimeError):
        sa.run_search(args, verbose=False)
    with pytest.raises(ValueError):
        bs.BatchSearchEngine(None, "cpu", {})


def _rec(line=20, image="1@s.mrcs"):
    return ParticleRecord(line, image, 0.0, 0.0, 0.0)


def test_ranked_row_order_dedup_and_invalid():
    angles = model_angles_from_lists([0.0, 10.0, 0.0, 20.0], [0.0, 5.0, 0.0, 7.0])
    rec = _rec()
    row = bs.ranked_row(rec, [0, 1, 2, 3], angles, np.asarray([5.0, 7.0, 9.0, 7.0], np.float32), keep=3)
    # 2 first (9), then the 7.0 tie in grid order (1 before 3); direction 0
    # repeats the (rot, tilt) of 2 and is dropped
    assert [d[0] for d in row["directions"]] == [2, 1, 3]
    assert row["directions"][0][1:3] == [0.0, 0.0]
    assert bs.ranked_row(rec, [0, 1], angles, [1.0, float("nan")], 2)["invalid_rawcc"] is True
    with pytest.raises(ValueError):
        bs.ranked_row(rec, [0, 1], angles, [1.0, float("inf")], 2)
    one = bs.ranked_row(rec, [1, 3], angles, torch.tensor([3.0, 4.0]), keep=1)
    assert [d[0] for d in one["directions"]] == [3]


def test_restricted_indices_validation():
    angles = model_angles_from_lists([0.0, 10.0, 20.0], [0.0, 5.0, 7.0])
    rec = _rec()
    good = dict(image=rec.image_name, directions=[[2, 20.0, 7.0, 1.5], [0, 0.0, 0.0, 1.0]])
    assert bs.restricted_indices(good, rec, [0, 1, 2], angles, keep=2) == [0, 2]
    bad_cases = [
        None,
        dict(image="2@s.mrcs", directions=good["directions"]),
        dict(image=rec.image_name, directions=[]),                                  # empty with allowed dirs
        dict(image=rec.image_name, directions=good["directions"] * 2),              # more than keep
        dict(image=rec.image_name, directions=[[1, 10.0, 5.0, 1.0]]),               # not allowed
        dict(image=rec.image_name, directions=[[2, 20.0, 8.0, 1.0]]),               # wrong grid coordinates
        dict(image=rec.image_name, directions=[[2, 20.0, 7.0, float("nan")]]),      # non-finite score
        dict(image=rec.image_name, directions=[[2.0, 20.0, 7.0, 1.0]]),             # index not an int
    ]
    for row in bad_cases:
        with pytest.raises(ValueError):
            bs.restricted_indices(row, rec, [0, 2], angles, keep=2)
