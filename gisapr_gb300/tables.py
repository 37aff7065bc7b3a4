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
# ---------------------------------------------------------------------------


@dataclass
class StarLoop:
    lines: List[str]
    labels: Dict[str, int]
    data_line_indices: List[int]
    data_start: int

    def tokens(self, line_index: int) -> List[str]:
        return self.lines[line_index].split()


def _label_index(tokens: Sequence[str], fallback: int) -> int:
    for tok in tokens[1:]:
        if tok.startswith("#"):
            try:
                return int(tok[1:]) - 1
            except ValueError:
                pass
    return fallback


def find_star_loop(lines: List[str], required_labels: Sequence[str]) -> StarLoop:
    """First loop_ holding every required label (v606:96-143)."""
    required = set(required_labels)
    n = len(lines)
    i = 0
    while i < n:
        if lines[i].strip().lower() != "loop_":
            i += 1
            continue
        labels: Dict[str, int] = {}
        j = i + 1
        fallback = 0
        while j < n:
            s = lines[j].strip()
            if not s or s.startswith("#"):
                j += 1
                continue
            if not s.startswith("_"):
                break
            toks = s.split()
            labels[toks[0]] = _label_index(toks, fallback)
            fallback += 1
            j += 1
        if not required.issubset(labels):
            i = max(j, i + 1)
            continue
        data: List[int] = []
        k = j
        start = -1
        while k < n:
            s = lines[k].strip()
            low = s.lower()
            if low == "loop_" or low.startswith("data_") or s.startswith("_"):
                if data:
                    break
                k += 1
                continue
            if not s or s.startswith("#"):
                k += 1
                continue
            if start < 0:
                start = k
            data.append(k)
            k += 1
        if start < 0:
            raise ValueError("Found a STAR loop with the required labels but no data rows: "
                             + ", ".join(required_labels))
        return StarLoop(lines, labels, data, start)
    raise ValueError("Cannot find a STAR loop containing: " + ", ".join(required_labels))


def read_text_lines(filename: str) -> List[str]:
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
    loop = find_star_loop(lines, ["_rlnAngleRot", "_rlnAngleTilt"])
    ri, ti = loop.labels["_rlnAngleRot"], loop.labels["_rlnAngleTilt"]
    pi = loop.labels.get("_rlnAnglePsi", -1)
    rot, tilt, psi = [], [], []
    for li in loop.data_line_indices:
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
    loop: StarLoop
    records: List[ParticleRecord]
    records_by_line: Dict[int, ParticleRecord]
    has_ctf: bool


def read_particle_table(particle_star: str) -> ParticleTable:
    """Particle rows of a RELION STAR (v606:227-306)."""
    lines = read_text_lines(particle_star)
    loop = find_star_loop(lines, ["_rlnImageName", "_rlnAngleRot", "_rlnAngleTilt"])
    ii = loop.labels["_rlnImageName"]
    ri, ti = loop.labels["_rlnAngleRot"], loop.labels["_rlnAngleTilt"]
    pi = loop.labels.get("_rlnAnglePsi", -1)
    du, dv, da = (loop.labels.get(k, -1) for k in ("_rlnDefocusU", "_rlnDefocusV", "_rlnDefocusAngle"))
    has_ctf = min(du, dv, da) >= 0
    recs: List[ParticleRecord] = []
    by_line: Dict[int, ParticleRecord] = {}
    need = max(ii, ri, ti)
    for li in loop.data_line_indices:
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
    start = max(start_line, table.loop.data_start) if start_line >= 0 else table.loop.data_start
    end = len(table.lines) if end_line < 0 else min(end_line, len(table.lines))
    if end < table.loop.data_start:
        end = table.loop.data_start
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


def generate_soft_mask(shape: Tuple[int, int], radius: int, edge_width: int) -> np.ndarray:
    center = np.asarray(shape) // 2
    y, x = np.indices(shape)
    d = np.sqrt((x - center[1]) ** 2 + (y - center[0]) ** 2)
    m = np.zeros_like(d)
    m[d <= radius] = 1.0
    if edge_width > 0:
        e = (d > radius) & (d <= radius + edge_width)
        m[e] = 0.5 * (1.0 + np.cos(np.pi * (d[e] - radius) / edge_width))
    return m.astype(np.float32, copy=False)


def expand_radial_values(values, size: int) -> np.ndarray:
    v = np.asarray(values, dtype=np.float32).reshape(-1)
    c = size // 2
    y, x = np.indices((size, size))
    r = np.sqrt((y - c) ** 2 + (x - c) ** 2).astype(np.int64)
    out = np.zeros((size, size), dtype=np.float32)
    ok = r < v.shape[0]
    out[ok] = v[r[ok]]
    return out


def read_fsc_map(fsc_filename: str, original_box: int, new_box: int, ignore_fsc: bool) -> np.ndarray:
    if not fsc_filename:
        values = np.ones(original_box, dtype=np.float32)
    else:
        parsed = []
        with open(fsc_filename, "r", encoding="utf-8", errors="replace") as fh:
            for line in fh:
                toks = line.split()
                if toks:
                    parsed.append(1.0 if ignore_fsc else float(toks[1]))
        if not parsed:
            raise ValueError(f"No FSC values found in {fsc_filename}")
        values = np.asarray(parsed, dtype=np.float32)
    return expand_radial_values(values, new_box)


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
