"""Tensor-core batched correlation (tcgen05 MMA, fp16 hi/lo split) against
the plain FP32 batch path and the FP64 oracle.

Precision bars: the split form (three fp16 products, ~22 bits) must sit
within the plain path's own parity bar of the FP64 oracle (peaks and score
1e-4 relative) and agree with the plain FP32 maps to 1e-5 of the map scale;
the single fp16 product (hi*hi, ~11 bits) is the fast form and is held to
2e-3 of the map scale.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from oracle import gisapr_oracle as O  # noqa: E402
from tests.helpers import PEAK_REL, SCORE_REL, TIE_REL, records_from_golden, records_from_job  # noqa: E402

DEV = "cuda:0"
SPLIT_MAP_REL = 1e-5   # |tc - plain| / max |plain| over every (candidate, entry, psi) map peak
FAST_MAP_REL = 2e-3


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


def _cfg(spec, box=None, apix=None):
    return JobConfig(box=box or spec.box, apix=apix or spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                     local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)


def _golden32_job(g):
    spec = syn.WORKLOADS["box32_tiny"]
    return ScoringJob(_cfg(spec), str(g["pdb_text"]), model_angles_from_lists(g["model_rot"], g["model_tilt"]),
                      records_from_golden(g), g["images"], fsc_values=g["fsc"], device=DEV)


def _maps(batch):
    return batch.score_buf.cpu().numpy(), batch.y_buf.cpu().numpy(), batch.x_buf.cpu().numpy()


def _compare_to_plain(job, poses, precision, map_rel):
    plain = BatchScoringJob(job, len(poses), use_graph=False)
    tc = BatchScoringJob(job, len(poses), use_graph=False, precision=precision)
    want = plain.score_batch(poses)
    got = tc.score_batch(poses)
    ps, py, px = _maps(plain)
    ts, ty, tx = _maps(tc)
    scale = float(np.max(np.abs(ps)))
    err = float(np.max(np.abs(ts - ps))) / scale
    assert err <= map_rel, (precision, err)
    # a map's argmax may move only between values the plain map holds as ties
    # within the stated error
    moved = (ty != py) | (tx != px)
    assert np.mean(moved) <= 0.01 if precision == "fp16" else np.mean(moved) <= 0.001, np.mean(moved)
    return plain, tc, want, got, err


def test_split_matches_plain_batch_golden32(golden32):
    g = golden32
    job = _golden32_job(g)
    poses = [g["pose"]] + list(syn.candidate_poses(4, 3, 5.0, 3.0))
    plain, tc, want, got, err = _compare_to_plain(job, poses, "fp16x3", SPLIT_MAP_REL)
    np.testing.assert_allclose(got, want, rtol=1e-6)
    pp, tp = plain.peak.cpu().numpy(), tc.peak.cpu().numpy()
    np.testing.assert_allclose(tp, pp, rtol=1e-5, atol=1e-5 * np.max(np.abs(pp)))
    same = (plain.best_entry.cpu().numpy() == tc.best_entry.cpu().numpy()) & \
           (plain.best_psi.cpu().numpy() == tc.best_psi.cpu().numpy())
    ps = plain.score_buf.cpu().numpy()
    n_psi = job.n_psi
    be_p, bp_p = plain.best_entry.cpu().numpy(), plain.best_psi.cpu().numpy()
    be_t, bp_t = tc.best_entry.cpu().numpy(), tc.best_psi.cpu().numpy()
    for c, i in zip(*np.where(~same)):
        a = ps[c, be_p[c, i] * n_psi + bp_p[c, i]]
        b = ps[c, be_t[c, i] * n_psi + bp_t[c, i]]
        assert abs(a - b) <= TIE_REL * abs(a), (c, i, a, b)
    assert int(tc.tc_status.item()) == 0


def test_split_vs_fp64_oracle_golden32(golden32):
    g = golden32
    job = _golden32_job(g)
    poses = [g["pose"], syn.candidate_poses(1, 5, 5.0, 3.0)[0]]
    tc = BatchScoringJob(job, len(poses), use_graph=False, precision="fp16x3")
    got = tc.score_batch(poses)
    assert abs(got[0] / float(g["score"]) - 1.0) < SCORE_REL
    peak = tc.peak.cpu().numpy()[0]
    valid = tc.best_entry.cpu().numpy()[0] >= 0
    np.testing.assert_allclose(peak[valid], g["peak"], rtol=PEAK_REL)
    best_dir = np.asarray([job.needed[int(job.local_idx[e])] for e in tc.best_entry.cpu().numpy()[0][valid]])
    assert np.mean(best_dir == g["best_dir"]) >= 0.999


def test_split_vs_fp64_oracle_box64(golden64):
    g = golden64
    spec = syn.WORKLOADS["box64_200p"]
    data = syn.make_job(spec, seed=int(g["seed"]))
    job = ScoringJob(_cfg(spec), data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                     records_from_job(data), data.images, fsc_values=data.fsc, device=DEV)
    rd = data.records
    ora = O.evaluate_candidate(data.model.pdb_text, g["pose"], 64, 1.5, 3.0, data.model_rot, data.model_tilt,
                               data.images, rd.line_index, rd.rot, rd.tilt, rd.psi, rd.defocus_u, rd.defocus_v,
                               rd.defocus_angle, data.fsc, spec.mask_radius, spec.mask_edge, spec.psi_step,
                               spec.local_range, spec.crop, kk=spec.kk, keep_templates=False)
    poses = [g["pose"]] + list(syn.candidate_poses(2, 17, 5.0, 3.0))
    tc = BatchScoringJob(job, len(poses), use_graph=True, precision="fp16x3")
    got = tc.score_batch(poses)
    assert abs(got[0] / ora["score"] - 1.0) < SCORE_REL
    be = tc.best_entry.cpu().numpy()[0]
    valid = be >= 0
    peak = tc.peak.cpu().numpy()[0][valid]
    np.testing.assert_allclose(peak, ora["raw"], rtol=PEAK_REL)
    # per-particle argmax (direction, psi, shift) against the oracle's first maxima
    bpsi = tc.best_psi.cpu().numpy()[0][valid]
    py, px = tc.peak_y.cpu().numpy()[0][valid], tc.peak_x.cpu().numpy()[0][valid]
    parts = [p for p in ora["particles"] if p["local"]]
    agree = 0
    for k, p in enumerate(parts):
        s = p["scores"]
        flat = int(np.argmax(s))
        a, psi = divmod(flat, s.shape[1])
        e = int(be[valid][k]) - int(job.local_ptr[np.where(valid)[0][k]])
        hit = (e == a and int(bpsi[k]) == psi and int(py[k]) == int(p["ys"][a, psi])
               and int(px[k]) == int(p["xs"][a, psi]))
        if not hit:
            hit = abs(float(s[e, int(bpsi[k])]) - float(s[a, psi])) <= TIE_REL * abs(float(s[a, psi]))
        agree += int(hit)
    assert agree / len(parts) >= 0.999, agree / len(parts)
    assert int(tc.tc_status.item()) == 0


def test_single_fp16_product_golden32(golden32):
    g = golden32
    job = _golden32_job(g)
    poses = [g["pose"]] + list(syn.candidate_poses(3, 7, 5.0, 3.0))
    plain, tc, want, got, err = _compare_to_plain(job, poses, "fp16", FAST_MAP_REL)
    np.testing.assert_allclose(got, want, rtol=1e-3)


def test_split_graph_replay_equals_eager(golden32):
    g = golden32
    job = _golden32_job(g)
    poses = list(syn.candidate_poses(6, 21, 5.0, 3.0))
    eager = BatchScoringJob(job, len(poses), use_graph=False, precision="fp16x3").score_batch(poses)
    graph = BatchScoringJob(job, len(poses), use_graph=True, precision="fp16x3")
    np.testing.assert_array_equal(graph.score_batch(poses), eager)
    poses2 = list(syn.candidate_poses(6, 22, 5.0, 3.0))
    np.testing.assert_array_equal(graph.score_batch(poses2),
                                  BatchScoringJob(job, 6, use_graph=False, precision="fp16x3").score_batch(poses2))


def test_split_more_than_128_candidates_in_chunks(golden32):
    """A batch above 128 candidates runs as equal chunks; each slot's scores
    equal those of a batch holding only that slot's pose."""
    g = golden32
    job = _golden32_job(g)
    poses = list(syn.candidate_poses(130, 31, 5.0, 3.0))
    big = BatchScoringJob(job, len(poses), use_graph=False, precision="fp16x3")
    assert [cc for _, cc in big.tc_chunks] == [65, 65]
    got = big.score_batch(poses)
    small = BatchScoringJob(job, 65, use_graph=False, precision="fp16x3")
    np.testing.assert_array_equal(got[65:], small.score_batch(poses[65:]))
    np.testing.assert_array_equal(got[:65], small.score_batch(poses[:65]))


def test_tensor_path_rejects_unsupported_sizes(golden32):
    import ctypes as C
    from gisapr_gb300 import _native as nat
    ctx = nat.Context.for_device(DEV).handle
    st = nat.stream_of(DEV)
    buf = torch.zeros(1 << 20, dtype=torch.uint8, device=DEV)
    p = nat.ptr(buf)
    for n, crop, n_psi in [(512, 12, 3), (128, 16, 3), (80, 12, 3), (256, 8, 3)]:
        with pytest.raises(ValueError):
            nat.call("gisapr_correlate_tc_batch", ctx, st, p, 0, 1, 1, p, p, p, p, p, 1, 1, n_psi, n, crop, 1,
                     p, p, p, p)
    with pytest.raises(ValueError):  # more than 128 candidates in one call
        nat.call("gisapr_correlate_tc_batch", ctx, st, p, 1 << 10, 129, 1, p, p, p, p, p, 1, 1, 3, 128, 12, 1,
                 p, p, p, p)
    _ = C


def test_split_box256_crop14_matches_plain():
    """The box-256 precision configuration (crop 14, psi groups of two) on a
    small particle set: tensor-core split maps against the plain FP32 maps."""
    spec = syn.WORKLOADS["box256_20kp"]
    data = syn.make_job(spec, seed=3, device=DEV, n_particles=24)
    job = ScoringJob(_cfg(spec), data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                     records_from_job(data), data.images, fsc_values=data.fsc, device=DEV)
    assert job.cfg.crop == 14 and job.cfg.new_box == 256
    poses = list(syn.candidate_poses(3, 41, 5.0, 3.0))
    plain, tc, want, got, err = _compare_to_plain(job, poses, "fp16x3", SPLIT_MAP_REL)
    np.testing.assert_allclose(got, want, rtol=1e-6)
    assert int(tc.tc_status.item()) == 0


@pytest.mark.parametrize("precision,map_rel", [("bf16x3", 1e-4), ("bf16", 1e-2)])
def test_bf16_forms_match_plain_golden32(golden32, precision, map_rel):
    """The bf16 operand forms (8 significant bits per part): the split form
    within 1e-4 of the plain maps' scale, the single form within 1e-2."""
    g = golden32
    job = _golden32_job(g)
    poses = [g["pose"]] + list(syn.candidate_poses(3, 9, 5.0, 3.0))
    plain = BatchScoringJob(job, len(poses), use_graph=False)
    tc = BatchScoringJob(job, len(poses), use_graph=False, precision=precision)
    want = plain.score_batch(poses)
    got = tc.score_batch(poses)
    ps, ts = plain.score_buf.cpu().numpy(), tc.score_buf.cpu().numpy()
    err = float(np.max(np.abs(ts - ps))) / float(np.max(np.abs(ps)))
    print(f"{precision}: map error {err:.2e} of the map scale")
    assert err <= map_rel, err
    np.testing.assert_allclose(got, want, rtol=1e-5 if precision == "bf16x3" else 1e-3)
    assert int(tc.tc_status.item()) == 0


def test_column_scales_are_powers_of_two_within_range(golden32):
    g = golden32
    job = _golden32_job(g)
    ts, ps = BatchScoringJob.column_scales(job)
    for s in (ts.cpu().numpy(), ps.cpu().numpy()):
        e = np.log2(s)
        assert np.all(e == np.round(e))
    assert np.all(ts.cpu().numpy() >= 1.0) and np.all(ts.cpu().numpy() <= 256.0)
    # particle columns scaled to at most 1/2 (times the global 2^13)
    pmax = job.stack.abs().amax(dim=(0, 1, 2)).cpu().numpy()
    assert np.all(pmax * ps.cpu().numpy() <= 0.5 + 1e-6)


def test_wait_limit_runs_out_and_reports_status(golden32):
    """With the on-chip hand-off waits bounded at one attempt the kernel
    gives up at once: it reports status 1, waits for its own copies in
    flight, frees its TMEM and returns, so the context stays usable and the
    next call with the default bound gives the normal scores."""
    g = golden32
    job = _golden32_job(g)
    poses = list(syn.candidate_poses(3, 13, 5.0, 3.0))
    ref = BatchScoringJob(job, len(poses), use_graph=False, precision="fp16x3").score_active(poses)
    b = BatchScoringJob(job, len(poses), use_graph=False, precision="fp16x3")
    b.tc_wait_limit = 1
    with pytest.raises(RuntimeError, match="ran out"):
        b.score_active(poses)
    assert int(b.tc_status.item()) == 1
    b.tc_status.zero_()
    b.tc_wait_limit = 0
    np.testing.assert_array_equal(b.score_active(poses), ref)
    assert int(b.tc_status.item()) == 0
