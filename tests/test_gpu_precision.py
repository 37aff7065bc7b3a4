"""PRECISION at the box-256 precision configuration's shapes (box 256 at
0.85 A/px, HEALPix order 4 within +-6 degrees, psi step 3.75, crop 14) on a
particle subset: every tensor-core form and the plain FP32 form against an
FP64 evaluation of the same contraction (the oracle's closed form of the
reference's crop-window irfft2, on the job's own float32 templates and
particle spectra), so the comparison isolates the contraction's
arithmetic. Bars: candidate score within 1e-4 relative and the
per-particle argmax (direction, psi, y, x) identical or tied within 1e-5 on
at least 99.9% of particles."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from oracle import gisapr_oracle as O  # noqa: E402
from tests.helpers import SCORE_REL, TIE_REL, records_from_job  # noqa: E402

DEV = "cuda:0"
N_PARTICLES = 40


@pytest.fixture(scope="module")
def case256():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    spec = syn.WORKLOADS["box256_20kp"]
    data = syn.make_job(spec, seed=7, device=DEV, n_particles=N_PARTICLES)
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                    local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                     records_from_job(data), data.images, fsc_values=data.fsc, device=DEV)
    poses = list(syn.candidate_poses(2, 43, 5.0, 3.0))
    plain = BatchScoringJob(job, len(poses), use_graph=False)
    plain.score_batch(poses)
    banks = plain.banks.cpu().numpy()
    stack = job.stack.cpu().numpy()
    ptr = job.local_ptr.cpu().numpy()
    idx = job.local_idx.cpu().numpy()
    # FP64 maxima of every (candidate, entry, psi) map, first maximum order
    fp64 = []
    for c in range(len(poses)):
        sc, ys, xs = [], [], []
        for i in range(len(job.records)):
            if ptr[i + 1] > ptr[i]:
                s, y, x = O.correlate(banks[c][idx[ptr[i]:ptr[i + 1]]], stack[i], cfg.crop)
                sc.append(s.reshape(-1)); ys.append(y.reshape(-1)); xs.append(x.reshape(-1))
        fp64.append((np.concatenate(sc), np.concatenate(ys), np.concatenate(xs)))
    return spec, job, poses, fp64


def _score64(job, maps):
    """sum_i exp(peak_i / 1024) from FP64 map maxima, and per-particle argmax."""
    ptr = job.local_ptr.cpu().numpy()
    n_psi = job.n_psi
    total, best = 0.0, []
    for i in range(len(job.records)):
        a, b = ptr[i] * n_psi, ptr[i + 1] * n_psi
        if b > a:
            k = int(np.argmax(maps[0][a:b]))
            total += float(np.exp(maps[0][a + k] / 1024.0))
            best.append((a, k))
        else:
            best.append(None)
    return total, best


@pytest.mark.parametrize("precision", ["fp32", "fp16x3", "bf16x3", "fp16", "bf16"])
def test_form_vs_fp64(case256, precision):
    spec, job, poses, fp64 = case256
    b = BatchScoringJob(job, len(poses), use_graph=False, precision=precision)
    got = b.score_batch(poses)
    n_psi = job.n_psi
    ptr = job.local_ptr.cpu().numpy()
    agree = total = 0
    worst = 0.0
    for c in range(len(poses)):
        want, best = _score64(job, fp64[c])
        rel = abs(got[c] / want - 1.0)
        worst = max(worst, rel)
        assert rel < SCORE_REL, (precision, c, rel)
        be = b.best_entry[c].cpu().numpy()
        bp = b.best_psi[c].cpu().numpy()
        py, px = b.peak_y[c].cpu().numpy(), b.peak_x[c].cpu().numpy()
        sc, ys, xs = fp64[c]
        for i, bk in enumerate(best):
            if bk is None:
                continue
            a, k = bk
            total += 1
            mine = int(be[i] - ptr[i]) * n_psi + int(bp[i])
            hit = mine == k and int(py[i]) == int(ys[a + k]) and int(px[i]) == int(xs[a + k])
            if not hit:  # a tie within 1e-5 of the FP64 maxima
                hit = abs(sc[a + mine] - sc[a + k]) <= TIE_REL * abs(sc[a + k])
            agree += int(hit)
    print(f"{precision}: score error {worst:.2e} vs FP64, argmax agreement {agree}/{total}")
    assert agree / total >= 0.999, (precision, agree, total)
    if precision != "fp32":
        assert int(b.tc_status.item()) == 0
