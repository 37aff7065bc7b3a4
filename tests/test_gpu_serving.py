"""The request loop on the GPU: each request's scores are the same alone and
in a concurrent mix of jobs and drivers (bitwise), and match the
per-candidate path."""
import threading

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.serving import ScoringServer  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from tests.helpers import records_from_golden, records_from_job  # noqa: E402

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


def _cfg(spec):
    return JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                     local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)


@pytest.fixture(scope="module")
def factories(golden32):
    g = golden32
    s32 = syn.WORKLOADS["box32_tiny"]
    s64 = syn.WORKLOADS["box64_small"]
    d64 = syn.make_job(s64, seed=5, n_particles=24)

    def f32():
        return ScoringJob(_cfg(s32), str(g["pdb_text"]), model_angles_from_lists(g["model_rot"], g["model_tilt"]),
                          records_from_golden(g), g["images"], fsc_values=g["fsc"], device=DEV)

    def f64():
        return ScoringJob(_cfg(s64), d64.model.pdb_text, model_angles_from_lists(d64.model_rot, d64.model_tilt),
                          records_from_job(d64), d64.images, fsc_values=d64.fsc, device=DEV)

    return {"b32": f32, "b64": f64}


def _requests(n, seed):
    rng = np.random.default_rng(seed)
    jobs = ("b32", "b64")
    return [(jobs[i % 2], syn.candidate_poses(int(rng.integers(1, 6)), seed * 100 + i, 5.0, 3.0))
            for i in range(n)]


@pytest.mark.parametrize("precision", ["fp32", "fp16x3"])
def test_results_alone_equal_results_in_the_mix(factories, precision):
    reqs = _requests(18, 7 if precision == "fp32" else 8)
    # alone: one request at a time through the job's own batch
    alone = []
    jobs = {k: f() for k, f in factories.items()}
    batches = {k: BatchScoringJob(j, 8, use_graph=False, precision=precision) for k, j in jobs.items()}
    for jid, p in reqs:
        alone.append(batches[jid].score_active(list(p)))
    # the same requests from three driver threads, two workers, jobs mixed
    with ScoringServer(DEV, max_batch=8, n_workers=2, precision=precision) as srv:
        for k, f in factories.items():
            srv.register(k, f, 1 << 30)
        futs = [None] * len(reqs)

        def driver(d):
            for i in range(d, len(reqs), 3):
                futs[i] = srv.submit(*reqs[i])

        ts = [threading.Thread(target=driver, args=(d,)) for d in range(3)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        srv.drain(timeout=600)
        st = srv.stats()
    for a, f in zip(alone, futs):
        np.testing.assert_array_equal(f.result(), a)
    assert st.requests == len(reqs) and st.latency_ms_p99 >= st.latency_ms_p50 > 0
    if precision == "fp32":
        # and the per-candidate path agrees
        for (jid, p), a in zip(reqs[:4], alone[:4]):
            np.testing.assert_array_equal(a, np.asarray([jobs[jid].score(q) for q in p]))
