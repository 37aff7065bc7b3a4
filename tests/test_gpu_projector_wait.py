"""Failure path of the shared-memory projector, without a GPU fault.

Each template's plane reaches shared memory by bulk copies whose wait is
bounded. With the bound set to zero attempts every CTA gives up at once:
the context's status word reports it, the templates are NaN and the engine's
check raises; with the default bound restored the same context builds the
templates again, bitwise equal to the ones it built before."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import _native as nat  # noqa: E402
from gisapr_gb300.engine import projector_check  # noqa: E402
from gisapr_gb300.search import IntegratedProjector, PackedFourierLayout  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from oracle import gisapr_oracle as O  # noqa: E402

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).to(DEV)


def _status(ctx) -> int:
    st = C.c_int(-1)
    nat.call("gisapr_projector_status", ctx.handle, nat.stream_of(DEV), C.byref(st))
    return st.value


def test_projector_wait_bound_reports_and_recovers(golden32):
    g = golden32
    angles = model_angles_from_lists(g["model_rot"], g["model_tilt"])
    fsc = _t(O.centered_to_packed(O.radial_map(g["fsc"], 32)))
    proj = IntegratedProjector(DEV, 32, 32, PackedFourierLayout(32, 8, DEV), _t(g["mask"]), fsc)
    dens = _t(g["density"])
    ctx = nat.Context(0)
    with nat.Context.using(ctx):
        assert _status(ctx) == 0  # no projector call yet
        base = proj.build_templates(dens, angles).cpu().numpy()
        assert np.isfinite(base).all()
        assert _status(ctx) == 0
        nat.call("gisapr_set_projector_wait", ctx.handle, 0)
        try:
            bad = proj.build_templates(dens, angles).cpu().numpy()
            assert _status(ctx) == 1
            assert _status(ctx) == 0  # the query reset the word
            assert np.isnan(bad).all()
            proj.build_templates(dens, angles)
            with pytest.raises(RuntimeError, match="projector"):
                projector_check(ctx.handle)
        finally:
            nat.call("gisapr_set_projector_wait", ctx.handle, -1)
        again = proj.build_templates(dens, angles).cpu().numpy()
        assert _status(ctx) == 0
        projector_check(ctx.handle)
    np.testing.assert_array_equal(again, base)


def test_scoring_job_raises_when_the_projector_gives_up(golden32):
    """ScoringJob.score reads the status word after each call: a projector
    that gave up raises instead of returning a score over NaN templates, and
    the next call with the default bound returns the earlier score bitwise."""
    from gisapr_gb300.engine import JobConfig, ScoringJob
    from gisapr_gb300 import synthetic as syn
    from tests.helpers import records_from_golden
    g = golden32
    spec = syn.WORKLOADS["box32_tiny"]
    cfg = JobConfig(box=32, apix=3.0, crop=spec.crop, psi_step=spec.psi_step, local_range=spec.local_range,
                    mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, str(g["pdb_text"]), model_angles_from_lists(g["model_rot"], g["model_tilt"]),
                     records_from_golden(g), g["images"], fsc_values=g["fsc"], device=DEV)
    job.use_graph = False
    base = job.score(g["pose"])
    ctx = nat.Context.for_device(DEV)
    nat.call("gisapr_set_projector_wait", ctx.handle, 0)
    try:
        with pytest.raises(RuntimeError, match="projector"):
            job.score(g["pose"])
    finally:
        nat.call("gisapr_set_projector_wait", ctx.handle, -1)
    assert job.score(g["pose"]) == base
