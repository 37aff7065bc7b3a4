"""Host-side tables of the search (v606:75-541): STAR rows, Euler matrices,
local orientation lists, soft mask, FSC map, packed layout indices, psi
sampling, psi rotation table and the static CTF terms.

These are computed once per job on the host, exactly as the reference does
(the float32 numpy expressions are kept where the kernels depend on their
bits), and handed to the kernels as small device tables.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

_PI_REF = 3.14159265359  # literal used by the reference's Euler code (v606:170-172)


# ---------------------------------------------------------------------------
# STAR parsing (gisapr_star.py / v606:75-224)
#
# Every line is classified once; a table is then a "loop_" line, the label
# lines after it and the data rows after those. The rules follow the
# reference's reader, which the search's line indices depend on (records
# are keyed by their STAR line): blank and "#" lines are skipped anywhere; a
# label is "_name" optionally followed by "#k" (1-based column), otherwise
# it takes the next column in order; rows end at the next "loop_", "data_"
# or label line once a row has been seen (before the first row those lines
# are skipped); a loop without every requested label is passed over.
# ---------------------------------------------------------------------------

_SKIP, _LOOP, _LABEL, _BLOCK, _ROW = range(5)


def _line_kind(line: str) -> int:
    s = line.strip()
    if not s or s[0] == "#":
        return _SKIP
    low = s.lower()
    if low == "loop_":
        return _LOOP
    if s[0] == "_":
        return _LABEL
    if low.startswith("data_"):
        return _BLOCK
    return _ROW


def _label_column(tokens: Sequence[str], default: int) -> int:
    """0-based column of a label line's tokens: the first "#k" token with
    an integer k gives k - 1, else ``default``."""
    for tok in tokens[1:]:
        if tok[:1] != "#":
            continue
        try:
            return int(tok[1:]) - 1
        except ValueError:
            continue
    return default


@dataclass
class StarTable:
    """One STAR loop: the file's lines, each label's column and the line
    indices of its data rows (``first_row`` is the first of them)."""

    lines: List[str]
    columns: Dict[str, int]
    row_lines: List[int]
    first_row: int

    def tokens(self, line_index: int) -> List[str]:
        return self.lines[line_index].split()


def find_star_table(lines: List[str], required_labels: Sequence[str]) -> StarTable:
    """The first loop whose labels include every one of ``required_labels``
    (v606:96-143). ValueError when no loop has them all, or when that loop
    has no data rows."""
    kinds = [_line_kind(ln) for ln in lines]
    n = len(lines)
    need = set(required_labels)
    pos = 0
    while True:
        try:
            head = kinds.index(_LOOP, pos)
        except ValueError:
            raise ValueError("no STAR loop has all of the labels " + ", ".join(required_labels)) from None
        columns: Dict[str, int] = {}
        k, n_labels = head + 1, 0
        while k < n and kinds[k] in (_SKIP, _LABEL):
            if kinds[k] == _LABEL:
                toks = lines[k].split()
                columns[toks[0]] = _label_column(toks, n_labels)  # a repeated label keeps its last column
                n_labels += 1
            k += 1
        if not need <= columns.keys():
            pos = max(k, head + 1)
            continue
        rows: List[int] = []
        while k < n:
            kind = kinds[k]
            if kind == _ROW:
                rows.append(k)
            elif kind != _SKIP and rows:
                break
            k += 1
        if not rows:
            raise ValueError("the STAR loop with labels " + ", ".join(required_labels) + " has no data rows")
        return StarTable(lines, columns, rows, rows[0])


# the reference's name of the same lookup
find_star_loop = find_star_table


def read_text_lines(filename: str) -> List[str]:
    """Lines of a text file with their line ends (bad bytes replaced)."""
    with open(filename, "r", encoding="utf-8", errors="replace") as fh:
        return fh.readlines()


def euler_angles_to_matrix(alpha: float, beta: float, gamma: float) -> List[List[float]]:
    """v605/project3d Euler convention (v606:168-187)."""
    a = alpha / 180.0 * _PI_REF
    b = beta / 180.0 * _PI_REF
    g = gamma / 180.0 * _PI_REF
    ca, cb, cg = math.cos(a), math.cos(b), math.cos(g)
    sa, sb, sg = math.sin(a), math.sin(b), math.sin(g)
    cc, cs, sc, ss = cb * ca, cb * sa, sb * ca, sb * sa
    return [[cg * cc - sg * sa, cg * cs + sg * ca, -cg * sb],
            [-sg * cc - cg * sa, -sg * cs + cg * ca, sg * sb],
            [sc, ss, cb]]


@dataclass
class ModelAngles:
    rot: List[float]
    tilt: List[float]
    psi: List[float]
    rotation_matrices_t: np.ndarray  # (M, 3, 3) float32, transposed (v606:216-218)


def model_angles_from_lists(rot: Sequence[float], tilt: Sequence[float],
                            psi: Optional[Sequence[float]] = None) -> ModelAngles:
    rot = [float(r) for r in rot]
    tilt = [float(t) for t in tilt]
    psi = [0.0] * len(rot) if psi is None else [float(p) for p in psi]
    mats = [np.asarray(euler_angles_to_matrix(r, t, 0.0), dtype=np.float32).T for r, t in zip(rot, tilt)]
    if not mats:
        raise ValueError("No model orientations")
    return ModelAngles(rot, tilt, psi, np.stack(mats).astype(np.float32))


def read_model_angles(angle_star: str) -> ModelAngles:
    """Direction list of a RELION angle STAR (v606:190-224)."""
    lines = read_text_lines(angle_star)
    loop = find_star_table(lines, ["_rlnAngleRot", "_rlnAngleTilt"])
    ri, ti = loop.columns["_rlnAngleRot"], loop.columns["_rlnAngleTilt"]
    pi = loop.columns.get("_rlnAnglePsi", -1)
    rot, tilt, psi = [], [], []
    for li in loop.row_lines:
        toks = loop.tokens(li)
        if max(ri, ti) >= len(toks):
            continue
        rot.append(float(toks[ri]))
        tilt.append(float(toks[ti]))
        psi.append(float(toks[pi]) if 0 <= pi < len(toks) else 0.0)
    if not rot:
        raise ValueError(f"No model orientations found in {angle_star}")
    return model_angles_from_lists(rot, tilt, psi)


@dataclass
class ParticleRecord:
    line_index: int
    image_name: str
    rot: float
    tilt: float
    psi: float
    defocus_u: float = 0.0
    defocus_v: float = 0.0
    defocus_angle: float = 0.0


@dataclass
class ParticleTable:
    lines: List[str]
    loop: StarTable
    records: List[ParticleRecord]
    records_by_line: Dict[int, ParticleRecord]
    has_ctf: bool


def read_particle_table(particle_star: str) -> ParticleTable:
    """Particle rows of a RELION STAR (v606:227-306)."""
    lines = read_text_lines(particle_star)
    loop = find_star_table(lines, ["_rlnImageName", "_rlnAngleRot", "_rlnAngleTilt"])
    ii = loop.columns["_rlnImageName"]
    ri, ti = loop.columns["_rlnAngleRot"], loop.columns["_rlnAngleTilt"]
    pi = loop.columns.get("_rlnAnglePsi", -1)
    du, dv, da = (loop.columns.get(k, -1) for k in ("_rlnDefocusU", "_rlnDefocusV", "_rlnDefocusAngle"))
    has_ctf = min(du, dv, da) >= 0
    recs: List[ParticleRecord] = []
    by_line: Dict[int, ParticleRecord] = {}
    need = max(ii, ri, ti)
    for li in loop.row_lines:
        toks = loop.tokens(li)
        if need >= len(toks):
            continue
        r = ParticleRecord(li, toks[ii], float(toks[ri]), float(toks[ti]),
                           float(toks[pi]) if 0 <= pi < len(toks) else 0.0)
        if has_ctf:
            r.defocus_u, r.defocus_v, r.defocus_angle = float(toks[du]), float(toks[dv]), float(toks[da])
        recs.append(r)
        by_line[li] = r
    if not recs:
        raise ValueError(f"No particle rows found in {particle_star}")
    return ParticleTable(lines, loop, recs, by_line, has_ctf)


def select_particle_records(table: ParticleTable, start_line: int, end_line: int) -> List[ParticleRecord]:
    """Rows in [start, end) by STAR line (v606:309-318)."""
    first = table.loop.first_row
    start = max(start_line, first) if start_line >= 0 else first
    end = len(table.lines) if end_line < 0 else min(end_line, len(table.lines))
    end = max(end, first)
    return [r for r in table.records if start <= r.line_index < end]


# ---------------------------------------------------------------------------
# Local orientation lists (v606:331-378)
# ---------------------------------------------------------------------------


def calculate_angular_distance(rot1, tilt1, psi1, rot2, tilt2, psi2) -> float:
    e1 = euler_angles_to_matrix(rot1, tilt1, psi1)
    e2 = euler_angles_to_matrix(rot2, tilt2, psi2)
    total = 0.0
    for i in range(3):
        dot = 0.0
        for a, b in zip(e1[i], e2[i]):
            dot += float(a) * float(b)
        dot = min(max(dot, -1.0), 1.0)
        total += math.acos(dot) * 180.0 / _PI_REF
    return total / 3.0


def build_local_orientation_entries(particle_records, model_rot, model_tilt, local_range) -> List[List[int]]:
    """[[line_index, dir, dir, ...], ...] exactly as the reference builds them:
    the wrapped |d rot|, |d tilt| window, then the mean three-axis angle."""
    mr = np.asarray(model_rot, dtype=np.float64)
    mt = np.asarray(model_tilt, dtype=np.float64)
    out: List[List[int]] = []
    for rec in particle_records:
        entry = [rec.line_index]
        rd = np.fabs((mr - rec.rot + 180.0) % 360.0 - 180.0)
        td = np.fabs((mt - rec.tilt + 180.0) % 360.0 - 180.0)
        for k in np.where((rd <= local_range) & (td <= local_range))[0]:
            d = calculate_angular_distance(float(mr[k]), float(mt[k]), 0.0, rec.rot, rec.tilt, 0.0)
            if abs(d) <= local_range:
                entry.append(int(k))
        out.append(entry)
    return out


# ---------------------------------------------------------------------------
# Mask, FSC, packed layout (v606:446-541)
# ---------------------------------------------------------------------------


def _centre_distance(shape: Tuple[int, int]) -> np.ndarray:
    """Distance of every pixel from the centre pixel (shape // 2), float64
    (the square root of the exact integer sum of squares)."""
    cy, cx = int(shape[0]) // 2, int(shape[1]) // 2
    dy = np.arange(int(shape[0]), dtype=np.int64)[:, None] - cy
    dx = np.arange(int(shape[1]), dtype=np.int64)[None, :] - cx
    return np.sqrt(dx * dx + dy * dy)


def generate_soft_mask(shape: Tuple[int, int], radius: int, edge_width: int) -> np.ndarray:
    """Circular mask with a raised-cosine edge (v606:446-457): 1 within
    ``radius`` of the centre pixel, 0.5 (1 + cos(pi (d - radius) / edge))
    out to ``radius + edge``, 0 beyond; float32."""
    d = _centre_distance(shape)
    inside = d <= radius
    if edge_width > 0:
        rim = ~inside & (d <= radius + edge_width)
        taper = 0.5 * (1.0 + np.cos(np.pi * (d - radius) / edge_width))
        m = np.where(inside, 1.0, np.where(rim, taper, 0.0))
    else:
        m = inside.astype(np.float64)
    return m.astype(np.float32)


def expand_radial_values(values, size: int) -> np.ndarray:
    """size x size float32 map whose pixel holds values[k], k the integer
    part of its distance from the centre pixel; 0 where k runs past the
    values (v606:460-468)."""
    v = np.asarray(values, dtype=np.float32).reshape(-1)
    k = _centre_distance((size, size)).astype(np.int64)
    if v.size == 0:
        return np.zeros((size, size), dtype=np.float32)
    return np.where(k < v.size, v[np.minimum(k, v.size - 1)], np.float32(0.0)).astype(np.float32)


def read_fsc_map(fsc_filename: str, original_box: int, new_box: int, ignore_fsc: bool) -> np.ndarray:
    """Centred new_box x new_box FSC weights from an FSC text (the second
    column of every non-blank line is the value of shell 0, 1, ...), all
    ones per shell when ``ignore_fsc`` or without a file (v606:471-491)."""
    if not fsc_filename:
        shells = np.ones(original_box, dtype=np.float32)
    else:
        with open(fsc_filename, "r", encoding="utf-8", errors="replace") as fh:
            rows = [ln.split() for ln in fh]
        shells = np.asarray([1.0 if ignore_fsc else float(r[1]) for r in rows if r], dtype=np.float32)
        if shells.size == 0:
            raise ValueError(f"{fsc_filename} holds no FSC values")
    return expand_radial_values(shells, new_box)


def centered_to_packed_np(centered: np.ndarray) -> np.ndarray:
    n = centered.shape[-1]
    h = n // 2
    rows = np.concatenate((np.arange(h, n), np.arange(0, h)))
    cols = np.concatenate((np.arange(h, n), [0]))
    return centered[..., rows, :][..., cols]


# ---------------------------------------------------------------------------
# psi sampling and rotation table (v606:1163-1247)
# ---------------------------------------------------------------------------


def psi_sampling_for_record(particle_psi, psi_step, do_local_search, local_range):
    num_psi = int(360 // psi_step)
    if num_psi < 1:
        num_psi = 1
    tmp = 999999.0
    if do_local_search:
        tmp = local_range // psi_step
        local_count = int(tmp * 2 + 1)
        if local_count < num_psi:
            num_psi = local_count
    fake, eff = [], []
    nearest = round(((particle_psi + 360.0) % 360.0) / psi_step) * psi_step
    nearest %= 360.0
    for i in range(int(num_psi)):
        a = psi_step * i
        if do_local_search:
            a = nearest - tmp * psi_step + i * psi_step
        fake.append(float(a))
        eff.append(float(0.5 if abs(a) < 0.5 else a))
    return fake, eff


def psi_rotation_entry(size: int, angle: float) -> np.ndarray:
    """(cos, sin, offset_row, offset_col) float32 of one psi grid: the matrix
    [[c, -s], [s, c]] and offset = centre - M @ centre, as PsiGridBank builds
    them in float32 numpy (v606:1224-1236)."""
    center = np.asarray((size, size), dtype=np.float32) / np.float32(2.0)
    theta = np.deg2rad(float(np.round(angle, 6)))
    c = np.float32(np.cos(theta))
    s = np.float32(np.sin(theta))
    M = np.asarray([[c, -s], [s, c]], dtype=np.float32)
    off = (center - M @ center).astype(np.float32)
    return np.asarray([c, s, off[0], off[1]], dtype=np.float32)


# ---------------------------------------------------------------------------
# Static CTF terms (v606:719-777)
# ---------------------------------------------------------------------------


@dataclass
class CtfStatic:
    k1: float
    k2: float
    k3: float
    k5: float
    kk: float
    x: np.ndarray
    y: np.ndarray
    u4: np.ndarray
    ncurve: np.ndarray


def ctf_static_terms(size: int, pixel_size: float, cs: float, voltage: float, kk: float,
                     amp_const: float = 0.1, phase_shift: float = 0.0) -> CtfStatic:
    if not 0.0 <= amp_const <= 1.0:
        raise ValueError("Amplitude contrast must be in [0, 1]")
    local_cs = np.float32(cs) * np.float32(1e7)
    local_kv = np.float32(voltage) * np.float32(1e3)
    lam = np.float32(12.2643247) / np.sqrt(local_kv * (np.float32(1.0) + local_kv * np.float32(0.978466e-6)))
    k1 = float(np.float32(np.pi) * lam)
    k2 = float(np.float32(np.pi / 2.0) * local_cs * lam ** np.float32(3.0))
    k3 = float(np.arctan(np.float32(amp_const) / np.sqrt(np.float32(1.0) - np.float32(amp_const) ** 2))
               .astype(np.float32))
    k5 = float(np.radians(np.float32(phase_shift)).astype(np.float32))
    n = int(size)
    ps = np.float32(pixel_size)
    cf = (np.arange(n, dtype=np.float32) - np.float32(n) / np.float32(2.0)) / (np.float32(n) * ps)
    yf = np.concatenate((cf[n // 2:], cf[:n // 2]))
    xf = np.concatenate((cf[n // 2:], cf[:1]))
    x, y = np.meshgrid(xf, yf, indexing="xy")
    x = x.astype(np.float32, copy=False)
    y = y.astype(np.float32, copy=False)
    u2 = x * x + y * y
    u4 = u2 * u2
    ss = np.sqrt(u2).astype(np.float32, copy=False)
    signal = np.exp(np.float32(-78.7757) * ss * ss + np.float32(-12.9121) * ss + np.float32(1.28732),
                    dtype=np.float32) / (np.float32(kk) + np.float32(1.0))
    ncurve = np.exp(np.float32(-9.32) * ss * ss + np.float32(2.65) * ss + np.float32(0.01908),
                    dtype=np.float32) / signal
    return CtfStatic(k1, k2, k3, k5, float(kk), x, y, u4.astype(np.float32),
                     ncurve.astype(np.float32, copy=False))
