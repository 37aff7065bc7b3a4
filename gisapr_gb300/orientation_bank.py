"""Top-K direction banks: calibrate once, then score each particle against
its K best directions only (Lite orientation_bank_v1.py:41-108, v7 search
flags --keep-orientations / --orientations-in / --orientations-out).

A bank is a JSON object in the Lite tree's format, so banks move between the
two programs in either direction:

* ``settings``: the schema name ``gisapr-orientations-v1``, the SHA-256 of
  the particle STAR's and the angle STAR's bytes, K (``keep``), whether the
  search was local, the local range and the psi step;
* ``rows``: per particle STAR line (the line number as a string) the image
  name and up to K ``[direction, rot, tilt, peak]`` entries, best first (a
  calibration whose peaks were NaN marks the row ``invalid_rawcc``);
* optional origin fields (the calibration writes the model's ``mrc`` path);
* ``sha256``: the SHA-256 of the compact, key-sorted JSON of everything
  else, which a reader recomputes before it trusts the bank.
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import tempfile
from pathlib import Path
from typing import Dict, List, Optional, Sequence

import numpy as np

SCHEMA = "gisapr-orientations-v1"

__all__ = ["SCHEMA", "bank_settings", "bank_digest", "pack_bank", "check_bank", "read_bank", "write_bank",
           "restricted_indices", "ranked_row"]


def _sha256_of_file(path) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as fh:
        while True:
            block = fh.read(1 << 20)
            if not block:
                return h.hexdigest()
            h.update(block)


def bank_settings(particle_star, angle_star, keep: int, local: bool, local_range: float, psi_step: float) -> dict:
    """The settings a bank is valid for: both input files by content, K and
    the search window."""
    return {"schema": SCHEMA, "particle_sha256": _sha256_of_file(particle_star),
            "angle_sha256": _sha256_of_file(angle_star), "keep": int(keep), "local": bool(local),
            "local_range": float(local_range), "psi_step": float(psi_step)}


def bank_digest(bank: dict) -> str:
    """SHA-256 (hex) of the bank without its ``sha256`` field, serialised as
    compact JSON with sorted keys (no NaN or infinity allowed)."""
    body = dict(bank)
    body.pop("sha256", None)
    text = json.dumps(body, sort_keys=True, allow_nan=False, separators=(",", ":"))
    return hashlib.sha256(text.encode("utf-8")).hexdigest()


def pack_bank(settings: dict, rows: Dict[str, dict], **origin) -> dict:
    """A bank object from settings and rows, with its digest."""
    bank = {"settings": settings, "rows": rows}
    bank.update(origin)
    bank["sha256"] = bank_digest(bank)
    return bank


def check_bank(bank: dict, settings: dict) -> None:
    """ValueError unless the bank was written for exactly these settings and
    its digest matches its content."""
    if not isinstance(bank, dict):
        raise ValueError("orientation bank: not a JSON object")
    if bank.get("settings") != settings:
        raise ValueError("orientation bank: written for other inputs, K or search settings")
    if bank.get("sha256") != bank_digest(bank):
        raise ValueError("orientation bank: digest does not match its content")


def read_bank(path, settings: dict) -> Dict[str, dict]:
    """The rows of a bank file, after check_bank."""
    bank = json.loads(Path(path).read_text(encoding="utf-8"))
    check_bank(bank, settings)
    return bank["rows"]


def write_bank(path, bank: dict) -> None:
    """Write a bank atomically: a temporary file in the same directory,
    then a rename over ``path``."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=path.name + ".", suffix=".tmp", dir=path.parent)
    try:
        with os.fdopen(fd, "w", encoding="utf-8") as fh:
            json.dump(bank, fh, allow_nan=False, ensure_ascii=False, indent=2)
            fh.write("\n")
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


def restricted_indices(row: Optional[dict], rec, allowed: Sequence[int], angles, keep: int) -> List[int]:
    """The directions a bank row lets one particle search, ascending (the
    search's tie order follows the angle file).

    The row must name the particle's image and hold at most min(K, allowed)
    entries, none if and only if the particle has no allowed directions.
    Each entry is ``[direction, rot, tilt, peak]``: an int direction among
    the particle's allowed ones, the grid's own (rot, tilt) of that
    direction, no (rot, tilt) twice, a finite peak. Anything else raises
    ValueError naming the STAR line, so a bank from other inputs never
    silently narrows a search."""
    line = rec.line_index
    if row is None or row.get("image") != rec.image_name:
        raise ValueError(f"orientation bank: no entry for the image of STAR line {line}")
    entries = row.get("directions")
    allowed_set = set(int(a) for a in allowed)
    if not isinstance(entries, list) or len(entries) > min(int(keep), len(allowed_set)) \
            or (len(entries) == 0) != (len(allowed_set) == 0):
        raise ValueError(f"orientation bank: wrong number of directions at STAR line {line}")
    chosen: List[int] = []
    pairs = set()
    for entry in entries:
        ok = isinstance(entry, list) and len(entry) == 4
        if ok:
            d, rot, tilt, peak = entry
            ok = (type(d) is int and d in allowed_set and (rot, tilt) not in pairs
                  and rot == angles.rot[d] and tilt == angles.tilt[d]
                  and isinstance(peak, (int, float)) and math.isfinite(peak))
        if not ok:
            raise ValueError(f"orientation bank: invalid direction entry at STAR line {line}")
        pairs.add((rot, tilt))
        chosen.append(d)
    chosen.sort()
    return chosen


def ranked_row(rec, indices: Sequence[int], angles, peaks, keep: int) -> dict:
    """One particle's bank row: its K best distinct (rot, tilt) directions
    by peak (already maximised over psi and translation), best first, equal
    peaks in list order. A NaN peak marks the row invalid; an infinite one
    raises ValueError."""
    if hasattr(peaks, "detach"):
        peaks = peaks.detach().cpu().numpy()
    p = np.asarray(peaks, dtype=np.float32).reshape(-1)
    if np.isinf(p).any():
        raise ValueError(f"orientation bank: infinite peak at STAR line {rec.line_index}")
    if np.isnan(p).any():
        return {"image": rec.image_name, "directions": [], "invalid_rawcc": True}
    order = sorted(range(len(p)), key=lambda j: -float(p[j]))  # stable: equal peaks keep list order
    best: Dict[tuple, list] = {}
    for j in order:
        d = int(indices[j])
        pair = (angles.rot[d], angles.tilt[d])
        if pair not in best:
            best[pair] = [d, pair[0], pair[1], float(p[j])]
            if len(best) == keep:
                break
    return {"image": rec.image_name, "directions": list(best.values())}
