"""Candidate score modes over search text (new_method_to_fit_the_2nd_Gaussian_PEAK_v4.py).

The refinement drivers score a candidate from the search text its
evaluation wrote: per particle the z-score of the ``cc:`` record and the
raw correlation of the ``rawCC:`` record (divided by 1024 here). Four modes:

* CC + simple sum (``do_run_CC=1, do_simple_sum=1``): sum_i exp(rawCC_i) --
  the score the GPU path reduces on the device (csrc/correlate.cu
  score_sum), reached here from text;
* CC + fit (``do_run_CC=1, do_simple_sum=0``): a 1000-bin density histogram
  of rawCC over [0, 1), smoothed by a Gaussian of sigma 2 bins, fitted with a
  sum of two Gaussians; with the larger fitted mean m, the score is
  count(rawCC > m) * m + sum(rawCC > m);
* z-score + fit / simple sum (``do_run_CC=0``): the same over the z-scores
  (histogram over their own range, other initial guesses), the simple sum
  being the plain sum of z-scores.

When the fit raises, the plain sum of the values is returned, as the
reference does (v4:105-110, 144-149). Parsing splits each record at commas
exactly as the reference's reader (v4:57-88), so files it reads parse the
same here. The fit itself is scipy's curve_fit, as in the reference.
"""
from __future__ import annotations

from typing import Iterable, List, Sequence, Tuple

import numpy as np

__all__ = ["gaussian", "double_gaussian", "parse_search_values", "score_values", "run_this", "main"]


def gaussian(x, amp, mean, stddev):
    return amp * np.exp(-((x - mean) ** 2) / (2 * stddev ** 2))


def double_gaussian(x, amp1, mean1, stddev1, amp2, mean2, stddev2):
    return gaussian(x, amp1, mean1, stddev1) + gaussian(x, amp2, mean2, stddev2)


def parse_search_values(lines: Iterable[str]) -> Tuple[np.ndarray, np.ndarray]:
    """(z-scores of ``cc:`` records below 9999, rawCC / 1024 of ``rawCC:``
    records) in file order (v4:57-88)."""
    z, raw = [], []
    for line in lines:
        parts = line.split(",")
        tag = parts[0]
        if tag == "['cc: '":
            value = float(parts[2])
            if value < 9999:
                z.append(value)
        elif tag == "['rawCC: '":
            raw.append(float(parts[-1].split("]")[0]) / 1024.0)
    return np.asarray(z), np.asarray(raw)


def _fit_score(values: np.ndarray, hist_range, guess_sigma: Tuple[float, float], guess_offset: float,
               amp2_div: float):
    """refined_x and count(v > x) * x + sum(v > x), or None if the fit raises."""
    from scipy.ndimage import gaussian_filter
    from scipy.optimize import curve_fit
    if hist_range is None:
        hist, edges = np.histogram(values, bins=1000, density=True)
    else:
        hist, edges = np.histogram(values, bins=1000, range=hist_range, density=True)
    smooth = gaussian_filter(hist, sigma=2)
    centers = (edges[:-1] + edges[1:]) / 2
    peak = centers[np.unravel_index(np.argmax(smooth), smooth.shape)]
    p0 = [max(smooth), peak, guess_sigma[0], max(smooth) / amp2_div, peak + guess_offset, guess_sigma[1]]
    try:
        params, _ = curve_fit(double_gaussian, centers, smooth, p0=p0)
    except Exception:  # noqa: BLE001 - the reference falls back on any failure of the fit
        return None
    refined = params[4]
    if params[1] > params[4]:
        refined = params[1]
    above = values > refined
    return refined, np.sum(above) * refined + np.sum(values[above])


def score_values(z: np.ndarray, raw: np.ndarray, do_run_CC, do_simple_sum) -> Tuple[float, float, float, float]:
    """(thres, CC_value, ZSCORE_value, total_estimated_sum_cc) as run_this
    returns them (v4:49-172): CC_value holds the fitted peak position."""
    z = np.asarray(z, dtype=np.float64)
    raw = np.asarray(raw, dtype=np.float64)
    if len(raw) < 1:
        return 0.0, 0.0, 0.0, 0.0
    if do_run_CC > 0:
        fit = _fit_score(raw, (0, 1.0), (0.02, 0.1), 0.05, 2.0)
        if fit is None:
            return 0.0, 0.0, 0.0, np.sum(raw)
        refined, total = fit
        if do_simple_sum > 0:
            total = np.sum(np.exp(raw))
        return 0.0, refined, 0.0, total
    if len(z) == 0:
        return 0.0, 0.0, 0.0, 0.0
    fit = _fit_score(z, None, (0.3, 4.0), 2.0, 4.0)
    if fit is None:
        return 0.0, 0.0, 0.0, np.sum(z)
    refined, total = fit
    if do_simple_sum > 0:
        total = np.sum(z)
    return 0.0, refined, 0.0, total


def run_this(results_file: str, do_run_CC, do_simple_sum):
    """Score one search text file (v4:49-172)."""
    with open(results_file, "r") as fh:
        z, raw = parse_search_values(fh.readlines())
    return score_values(z, raw, do_run_CC, do_simple_sum)


def main(argv: Sequence[str] = None) -> None:
    """``<index file> <do_run_CC> <do_simple_sum> <output file>``: for every
    search text named in the index file, write its name and then
    ``total ZSCORE_value CC_value`` (v4:34-47)."""
    import sys
    args = list(sys.argv[1:] if argv is None else argv)
    if len(args) < 4:
        print("<Results file> <do_run_CC = 1, zscore = 0> <do_simple_sum = 1> <output filename>")
        raise SystemExit(-1)
    index, do_cc, do_sum, out_name = args[0], float(args[1]), float(args[2]), args[3]
    with open(index, "r") as fh:
        names: List[str] = [line.strip() for line in fh.readlines()]
    with open(out_name, "w") as out:
        for name in names:
            out.write(name + "\n")
            _, cc_value, z_value, total = run_this(name, do_cc, do_sum)
            out.write(str(total) + " " + str(z_value) + " " + str(cc_value) + "\n")

