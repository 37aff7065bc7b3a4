"""The launch-shape autotuner: it times every valid choice, caches the
winner, and its choices leave scores unchanged beyond float32 summation
order."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import _native as nat  # noqa: E402
from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.autotune import Autotuner  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from tests.helpers import records_from_golden  # noqa: E402

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


def test_tune_caches_and_keeps_scores(golden32, tmp_path):
    g = golden32
    spec = syn.WORKLOADS["box32_tiny"]
    cfg = JobConfig(box=32, apix=3.0, crop=spec.crop, psi_step=spec.psi_step, local_range=spec.local_range,
                    mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, str(g["pdb_text"]), model_angles_from_lists(g["model_rot"], g["model_tilt"]),
                     records_from_golden(g), g["images"], fsc_values=g["fsc"], device=DEV)
    poses = list(syn.candidate_poses(8, 77, 5.0, 3.0))
    ref = BatchScoringJob(job, 8, use_graph=False).score_active(poses)
    ref_tc = BatchScoringJob(job, 8, use_graph=False, precision="fp16x3").score_active(poses)
    try:
        tuner = Autotuner(tmp_path / "tuning.json", trials=1)
        r = tuner.tune(job, n_cand=8, precision="fp16x3")
        assert r.corr_cluster in (1, 2, 3, 4, 5, 6, 8)
        assert r.tc_chunk in (8,) or r.tc_chunk <= 8
        assert any(k.startswith("plain_cluster_") for k in r.times_ms)
        assert any(k.startswith("tc_chunk_") for k in r.times_ms)
        assert any(k.startswith("tc_rings_") for k in r.times_ms)
        assert (r.tc_a_stages, r.tc_b_stages) in ((4, 2), (3, 2), (6, 2), (4, 3))
        assert r.dirs_per_tile == 128 // 8
        assert r.template_lanes in (1, 2, 3)
        assert any(k.startswith("template_lanes_") for k in r.times_ms)
        assert (tmp_path / "tuning.json").exists()
        r2 = Autotuner(tmp_path / "tuning.json").tune(job, n_cand=8, precision="fp16x3")
        assert (r2.corr_cluster, r2.tc_chunk, r2.times_ms) == (r.corr_cluster, r.tc_chunk, r.times_ms)
        got = BatchScoringJob(job, 8, use_graph=False).score_active(poses)
        np.testing.assert_allclose(got, ref, rtol=1e-6)
        got_tc = BatchScoringJob(job, 8, use_graph=False, precision="fp16x3", tc_chunk=r.tc_chunk).score_active(poses)
        np.testing.assert_allclose(got_tc, ref_tc, rtol=1e-6)
        # every cluster size gives the same maps up to float32 summation order
        ctx = nat.Context.for_device(DEV)
        for k in (1, 2, 3):
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_CORR_CLUSTER, 32, k)
            np.testing.assert_allclose(BatchScoringJob(job, 8, use_graph=False).score_active(poses), ref, rtol=1e-6)
        with pytest.raises(ValueError):
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_CORR_CLUSTER, 32, 9)
        with pytest.raises(ValueError):
            nat.call("gisapr_set_tuning", ctx.handle, 77, 32, 1)
        # every ring depth gives bitwise the same tensor-core maps
        tc_ref = BatchScoringJob(job, 8, use_graph=False, precision="fp16x3", tc_chunk=r.tc_chunk)
        tc_ref.score_active(poses)
        maps = tc_ref.score_buf.cpu().numpy()
        for sa, sb in ((2, 2), (3, 3), (8, 2)):
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_A_STAGES, 32, sa)
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_B_STAGES, 32, sb)
            b = BatchScoringJob(job, 8, use_graph=False, precision="fp16x3", tc_chunk=r.tc_chunk)
            b.score_active(poses)
            np.testing.assert_array_equal(b.score_buf.cpu().numpy(), maps)
        with pytest.raises(ValueError):
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_A_STAGES, 32, 9)
        with pytest.raises(ValueError):
            nat.call("gisapr_set_tuning", ctx.handle, nat.TUNE_TC_B_STAGES, 48, 2)
    finally:
        nat.set_default_tuning(nat.TUNE_CORR_CLUSTER, 32, 0)
        nat.set_default_tuning(nat.TUNE_TC_A_STAGES, 32, 0)
        nat.set_default_tuning(nat.TUNE_TC_B_STAGES, 32, 0)
