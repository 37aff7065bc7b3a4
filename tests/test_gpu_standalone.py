"""File-based entry points on the GPU: run_search (v606 standalone command)
and BatchSearchEngine (Lite round evaluation), against the reference's own
records of the box-32 fixture and against the in-memory engine."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.batch_search import BatchSearchEngine  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.standalone import run_search  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from tests.helpers import (PEAK_REL, SCORE_REL, parse_search_text, records_from_golden,  # noqa: E402
                           write_search_inputs)

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


def _check_against_golden(rows, g, check_z=True):
    """Search text records against the reference's values of the fixture
    (the z-score only with ``check_z``: it runs over the searched maps)."""
    assert len(rows) == len(g["z"])
    rot, tilt = np.asarray(g["model_rot"]), np.asarray(g["model_tilt"])
    for k, (cc, psi, raw) in enumerate(rows):
        assert cc[1] == int(g["rec_line"][k]) == psi[1] == raw[1]
        d = int(g["best_dir"][k])
        assert (cc[5], cc[6]) == (float(rot[d]), float(tilt[d])), k
        assert psi[2] == float(g["best_psi"][k]), k
        assert (cc[8], cc[9]) == (int(g["shift_x"][k]), int(g["shift_y"][k])), k
        assert (cc[3], cc[4]) == (int(g["l3"][k]), int(g["accu"][k])), k
        assert abs(cc[7] - float(g["angdist"][k])) <= 1e-9 * max(1.0, abs(float(g["angdist"][k])))
        assert abs(raw[2] / float(g["peak"][k]) - 1.0) < PEAK_REL, k
        if check_z:
            assert abs(cc[2] - float(g["z"][k])) < 1e-3 * max(1.0, abs(float(g["z"][k]))), k


def test_run_search_matches_reference_records_golden32(golden32, tmp_path):
    g = golden32
    args = write_search_inputs(tmp_path, g)
    times = run_search(args, verbose=False)
    rows = parse_search_text(args.o)
    _check_against_golden(rows, g)
    assert abs(times["score"] / float(g["score"]) - 1.0) < SCORE_REL
    # the local-direction cache is written under the reference's name and reused
    cache = tmp_path / ("particles.star_LocalSearch_Angle_" + str(int(args.localRange)) + "_data.pkl")
    assert cache.exists()
    again = run_search(args, verbose=False)
    assert again["score"] == times["score"]


def test_run_search_chunks_selection_and_continue(golden32, tmp_path):
    g = golden32
    args = write_search_inputs(tmp_path, g)
    run_search(args, verbose=False)
    whole = open(args.o).read()
    # chunks of a few particles give the same text as one chunk
    per_particle = 5 * 32 * 17 * 8 + 32 * 32 * 4
    args.particleChunkMB = 5 * per_particle / 2 ** 20
    args.o = str(tmp_path / "chunked.txt")
    t = run_search(args, verbose=False)
    assert t["chunks"] == 5.0
    assert open(args.o).read() == whole
    # [start, end) by STAR line, then --doContinue appends the rest
    lines = [int(v) for v in g["rec_line"]]
    cut = lines[10]
    args.o = str(tmp_path / "parts.txt")
    args.particleChunkMB = 16384.0
    args.start, args.end = -1, cut
    run_search(args, verbose=False)
    args.start, args.end, args.doContinue = cut, -1, True
    run_search(args, verbose=False)
    assert open(args.o).read() == whole


def test_run_search_global_search_matches_engine(golden32, tmp_path):
    """Without --doLocalSearch every particle searches every direction over
    the full psi circle; the written score equals the in-memory engine's."""
    g = golden32
    args = write_search_inputs(tmp_path, g)
    args.doLocalSearch = False
    args.psiStep = 30.0
    t = run_search(args, verbose=False)
    spec = syn.WORKLOADS["box32_tiny"]
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=30.0, local_range=spec.local_range,
                    do_local_search=False, mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, None, model_angles_from_lists(g["model_rot"], g["model_tilt"]), records_from_golden(g),
                     g["images"], fsc_values=g["fsc"], device=DEV)
    assert job.n_psi == 12 and job.nnz == len(g["rec_line"]) * len(g["model_rot"])
    want = job.score_volume(np.asarray(g["density"]))
    assert t["score"] == pytest.approx(want, rel=1e-12)
    assert open(args.o).read() == job.search_text()


def _models(g, tmp_path, poses):
    spec = syn.WORKLOADS["box32_tiny"]
    pdb = str(tmp_path / "model.pdb")
    return [dict(pdb_path=pdb, source_pdb=pdb, chain_id="A", pose=list(map(float, p)), boxsize=spec.box,
                 apix=spec.apix, res=spec.res, device=DEV) for p in poses]


@pytest.mark.parametrize("precision", ["fp32", "fp16x3"])
def test_batch_search_engine_scores_and_texts(golden32, tmp_path, precision):
    g = golden32
    args = write_search_inputs(tmp_path, g)
    poses = [g["pose"]] + list(syn.candidate_poses(4, 51, 5.0, 3.0))
    eng = BatchSearchEngine(None, torch.device(DEV), dict(batch_candidates=3, precision=precision))
    out = eng.run(args, _models(g, tmp_path, poses))
    assert len(out) == len(poses)
    # the fixture pose against the reference's records and score
    assert abs(out[0]["score"] / float(g["score"]) - 1.0) < SCORE_REL
    _check_against_golden(parse_search_text(out[0]["search_text"]), g)
    # every slot against the in-memory engine's single-candidate path
    spec = syn.WORKLOADS["box32_tiny"]
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                    local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, str(g["pdb_text"]), model_angles_from_lists(g["model_rot"], g["model_tilt"]),
                     records_from_golden(g), g["images"], fsc_values=g["fsc"], device=DEV)
    want = job.score_many(poses)
    got = np.asarray([o["score"] for o in out])
    np.testing.assert_allclose(got, want, rtol=1e-6 if precision == "fp16x3" else 1e-12)
    if precision == "fp32":
        job.score(poses[2])
        assert out[2]["search_text"] == job.search_text()
    # the particle set is prepared once and reused by the next round
    first = eng.context
    eng.run(args, _models(g, tmp_path, poses[:2]))
    assert eng.context is first


def test_batch_search_engine_calibrate_then_restricted(golden32, tmp_path):
    g = golden32
    args = write_search_inputs(tmp_path, g)
    args.keep_orientations = 2
    poses = [g["pose"]] + list(syn.candidate_poses(2, 61, 5.0, 3.0))
    eng = BatchSearchEngine(None, torch.device(DEV), dict(batch_candidates=4))
    cal = eng.run(args, _models(g, tmp_path, poses), calibrate=True)
    rows = cal[0]["orientation_rows"]
    assert set(rows) == {str(int(v)) for v in g["rec_line"]}
    for k, line in enumerate(g["rec_line"]):
        row = rows[str(int(line))]
        assert 1 <= len(row["directions"]) <= 2
        assert row["directions"][0][0] == int(g["best_dir"][k])
        peaks = [d[3] for d in row["directions"]]
        assert peaks == sorted(peaks, reverse=True)
    # restricting to the bank keeps every particle's best direction, so the
    # score (sum over particles of exp(peak / 1024)) is unchanged bit for bit
    res = eng.run(args, _models(g, tmp_path, poses[:1]), orientation_rows=rows)
    assert res[0]["score"] == cal[0]["score"]
    assert eng.context.job.nnz <= 2 * len(g["rec_line"])


def test_batch_search_engine_volume_models(golden32, tmp_path):
    """A model without a moving chain (the whole PDB) is scored through its
    generated density, equal to the engine's volume path."""
    g = golden32
    args = write_search_inputs(tmp_path, g)
    spec = syn.WORKLOADS["box32_tiny"]
    pdb = str(tmp_path / "model.pdb")
    model = dict(pdb_path=pdb, boxsize=spec.box, apix=spec.apix, res=spec.res, device=DEV)
    eng = BatchSearchEngine(None, torch.device(DEV), {})
    out = eng.run(args, [model])
    from gisapr_gb300.pdb2mrc import generate_volume
    vol = generate_volume(pdb, spec.box, spec.apix, spec.res, device=DEV)
    assert out[0]["score"] == eng.context.job.score_volume(vol)


def test_run_search_bank_files_calibrate_then_restricted(golden32, tmp_path):
    """--orientations-out writes a bank in the reference's format (settings
    by input hashes, digest) whose best direction per particle is the
    reference's; --orientations-in then searches only the bank's directions
    and writes the reference's records again, with the same score."""
    import json
    from gisapr_gb300 import orientation_bank as ob
    g = golden32
    bank_path = tmp_path / "bank.json"
    args = write_search_inputs(tmp_path, g, extra=("--keep-orientations", "2", "--orientations-out",
                                                   str(bank_path)))
    cal = run_search(args, verbose=False)
    settings = ob.bank_settings(args.p, args.ang, 2, True, args.localRange, args.psiStep)
    bank = json.loads(bank_path.read_text())
    ob.check_bank(bank, settings)
    assert bank["mrc"] == str((tmp_path / "model.mrc").resolve())
    for k, line in enumerate(g["rec_line"]):
        row = bank["rows"][str(int(line))]
        assert 1 <= len(row["directions"]) <= 2
        assert row["directions"][0][0] == int(g["best_dir"][k])
    args = write_search_inputs(tmp_path, g, extra=("--keep-orientations", "2", "--orientations-in",
                                                   str(bank_path)))
    res = run_search(args, verbose=False)
    assert res["score"] == cal["score"]
    # the records keep the reference's direction, psi and shifts (the z-score
    # now runs over the bank's directions only)
    _check_against_golden(parse_search_text(tmp_path / "search.txt"), g, check_z=False)
    # a bank for other settings is refused
    args = write_search_inputs(tmp_path, g, extra=("--keep-orientations", "3", "--orientations-in",
                                                   str(bank_path)))
    with pytest.raises(ValueError):
        run_search(args, verbose=False)
