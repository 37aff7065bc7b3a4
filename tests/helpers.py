"""Shared helpers of the test suite (inputs from fixtures, error measures)."""
from __future__ import annotations

import numpy as np

from gisapr_gb300 import synthetic as syn
from gisapr_gb300.tables import ParticleRecord

# Tolerances. Density, particle spectra and scores follow the stated parity
# bar; templates carry the reference's own float32 whitening error (its
# templates differ from the FP64 oracle by up to 6e-5 relative RMS, checked in
# test_oracle_golden), so the template bar sits above that floor.
DENSITY_RRMS = 1e-5
SPECTRUM_RRMS = 1e-5
TEMPLATE_RRMS = 3e-4
CTF_ABS = 2e-5
SCORE_REL = 1e-4
PEAK_REL = 1e-4
TIE_REL = 1e-5


def rrms(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.sqrt(np.sum(np.abs(a - b) ** 2) / np.sum(np.abs(b) ** 2)))


def records_from_arrays(line, rot, tilt, psi, dfu, dfv, dfa):
    return [ParticleRecord(int(line[i]), f"{i + 1}@stack.mrcs", float(rot[i]), float(tilt[i]), float(psi[i]),
                           float(dfu[i]), float(dfv[i]), float(dfa[i])) for i in range(len(rot))]


def records_from_golden(g):
    return records_from_arrays(g["rec_line"], g["rec_rot"], g["rec_tilt"], g["rec_psi"], g["rec_dfu"],
                               g["rec_dfv"], g["rec_dfa"])


def records_from_job(job: syn.SearchJob):
    r = job.records
    return records_from_arrays(r.line_index, r.rot, r.tilt, r.psi, r.defocus_u, r.defocus_v, r.defocus_angle)


def argmax_agrees(scores_a, scores_b, idx_a, idx_b, tie_rel=TIE_REL) -> bool:
    """Same first maximum, or both maxima within ``tie_rel`` of each other."""
    if idx_a == idx_b:
        return True
    va, vb = float(scores_b[idx_a]), float(scores_b[idx_b])
    return abs(va - vb) <= tie_rel * max(abs(vb), 1e-30)
