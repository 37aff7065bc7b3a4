"""Per-slot particle subsets in a batch (BatchScoringJob.set_subsets): each
slot's score and records equal those of a job that holds only its particles
(scored alone on the single-candidate path), for the plain FP32 and the
split tensor-core forms, eagerly and through graph replays whose subsets
change between replays."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from tests.helpers import records_from_job  # noqa: E402

DEV = "cuda:0"
N_PARTICLES = 60


@pytest.fixture(scope="module")
def case():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    spec = syn.WORKLOADS["box64_200p"]
    data = syn.make_job(spec, seed=11, device=DEV, n_particles=N_PARTICLES)
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                    local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
    records = records_from_job(data)
    angles = model_angles_from_lists(data.model_rot, data.model_tilt)

    def job_of(idx):
        idx = np.asarray(idx, dtype=np.int64)
        return ScoringJob(cfg, data.model.pdb_text, angles, [records[i] for i in idx], data.images[idx],
                          fsc_values=data.fsc, device=DEV)

    full = job_of(np.arange(N_PARTICLES))
    rng = np.random.default_rng(3)
    subsets = [None,                                                   # every particle
               np.arange(0, N_PARTICLES, 2),                           # every other particle
               np.sort(rng.choice(N_PARTICLES, 17, replace=False)),    # a ragged draw
               np.array([N_PARTICLES - 1]),                            # one particle
               rng.random(N_PARTICLES) < 0.5]                          # a boolean mask
    poses = list(syn.candidate_poses(len(subsets), 29, 4.0, 2.0))
    return full, job_of, subsets, poses


def _indices(sub, n):
    if sub is None:
        return np.arange(n)
    a = np.asarray(sub)
    return np.flatnonzero(a) if a.dtype == np.bool_ else a


def _alone(job_of, sub, pose, n):
    """Score and per-particle records of a job holding only the subset."""
    idx = _indices(sub, n)
    j = job_of(idx)
    score = j.score(pose)
    r = j.particle_results()
    ptr, lidx = j.local_ptr.cpu().numpy(), j.local_idx.cpu().numpy()
    dirs = np.where(r["best_entry"] >= 0, np.asarray(j.needed)[lidx[np.maximum(r["best_entry"], 0)]], -1)
    return idx, score, r, dirs, j.search_text()


def _check_slot(batch, c, full, job_of, sub, pose, rel):
    n = len(full.records)
    idx, want, r_alone, dirs_alone, text_alone = _alone(job_of, sub, pose, n)
    got = float(batch.totals[c].item())
    assert abs(got / want - 1.0) < rel, (c, got, want)
    r = batch.slot_results(c + 1)[c]
    left_out = np.setdiff1d(np.arange(n), idx)
    assert np.all(r["best_entry"][left_out] == -1), c
    lidx = full.local_idx.cpu().numpy()
    be = r["best_entry"][idx]
    dirs = np.where(be >= 0, np.asarray(full.needed)[lidx[np.maximum(be, 0)]], -1)
    np.testing.assert_allclose(r["peak"][idx], r_alone["peak"], rtol=rel)
    if rel <= 1e-6:
        np.testing.assert_array_equal(dirs, dirs_alone)
        np.testing.assert_array_equal(r["best_psi"][idx], r_alone["best_psi"])
        np.testing.assert_array_equal(r["peak_y"][idx], r_alone["peak_y"])
        np.testing.assert_array_equal(r["peak_x"][idx], r_alone["peak_x"])
    else:
        assert np.mean(dirs == dirs_alone) >= 0.95, c
    # the slot's search text is the alone job's (same records, same lines)
    if rel <= 1e-6:
        got_lines = batch.search_texts(c + 1)[c].splitlines()
        want_lines = text_alone.splitlines()
        assert len(got_lines) == len(want_lines), c
        assert [ln.split(",")[:2] for ln in got_lines] == [ln.split(",")[:2] for ln in want_lines], c


@pytest.mark.parametrize("precision, rel", [("fp32", 1e-6), ("fp16x3", 1e-5)])
def test_subsets_eager_equal_alone(case, precision, rel):
    full, job_of, subsets, poses = case
    b = BatchScoringJob(full, len(poses), use_graph=False, precision=precision)
    b.score_active(poses, subsets=subsets)
    for c, sub in enumerate(subsets):
        _check_slot(b, c, full, job_of, sub, poses[c], rel)


def test_subsets_change_between_graph_replays(case):
    full, job_of, subsets, poses = case
    b = BatchScoringJob(full, len(poses), use_graph=True)
    all_scores = b.score_batch(poses)                      # captured with every slot scoring everything
    np.testing.assert_allclose(all_scores[0], full.score(poses[0]), rtol=1e-6)
    b.score_batch(poses, subsets=subsets)                  # same graph, new mask
    assert b.graph is not None
    for c, sub in enumerate(subsets):
        _check_slot(b, c, full, job_of, sub, poses[c], 1e-6)
    again = b.score_batch(poses, subsets=[None] * len(poses))
    np.testing.assert_array_equal(again, all_scores)


def test_empty_subset_scores_zero(case):
    full, _, _, poses = case
    b = BatchScoringJob(full, 2, use_graph=False)
    s = b.score_active(poses[:2], subsets=[[], None])
    assert s[0] == 0.0
    assert np.all(b.slot_results(1)[0]["best_entry"] == -1)
    np.testing.assert_allclose(s[1], full.score(poses[1]), rtol=1e-6)
