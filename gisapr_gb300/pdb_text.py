"""PDB coordinates and the rigid-body pose of one chain (pdb_text.py of the
reference: element inference :26-46, reader :78-120, transform :123-142;
Lite tree: quantize_coordinates :33-58, transformed_density_atoms :204-223).

Only the host-side parsing lives here. The pose transform and the PDB 8.3
round trip of the moved chain run on the GPU inside the splat launch
(gisapr_deposit_moved); ``transform_coordinates`` and
``quantize_coordinates`` are kept for callers that want the coordinates.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

_ELEMENTS = set((
    "H HE LI BE B C N O F NE NA MG AL SI P S CL AR K CA SC TI V CR MN FE "
    "CO NI CU ZN GA GE AS SE BR KR RB SR Y ZR NB MO TC RU RH PD AG CD IN "
    "SN SB TE I XE CS BA LA CE PR ND PM SM EU GD TB DY HO ER TM YB LU HF "
    "TA W RE OS IR PT AU HG TL PB BI PO AT RN FR RA AC TH PA U NP PU AM "
    "CM BK CF ES FM MD NO LR RF DB SG BH HS MT DS RG CN NH FL MC LV TS OG D").split())


def infer_element(line: str) -> str:
    explicit = line[76:78].strip().upper()
    if explicit in _ELEMENTS:
        return explicit
    name = line[12:16].ljust(4).upper()
    letters = "".join(ch for ch in name if ch.isalpha())
    if not letters:
        return ""
    if name[0].isspace() or name[0].isdigit():
        return letters[0] if letters[0] in _ELEMENTS else ""
    if line[:6] == "ATOM  " and letters[0] in "CNOHPS":
        return letters[0]
    if letters[:2] in _ELEMENTS:
        return letters[:2]
    return letters[0] if letters[0] in _ELEMENTS else ""


@dataclass
class PDBText:
    lines: list
    coords: np.ndarray          # [n, 3] float32
    elements: np.ndarray        # [n] U2
    chains: np.ndarray          # [n] U1
    atom_line_indices: np.ndarray


def parse_pdb_lines(lines, include_hetatm=True, first_model_only=True, source="<text>") -> PDBText:
    first_model = next((i for i, l in enumerate(lines) if l[:6].strip() == "MODEL"), None)
    active = first_model is None
    coords, els, chains, idx = [], [], [], []
    kinds = ("ATOM", "HETATM") if include_hetatm else ("ATOM",)
    for i, line in enumerate(lines):
        rec = line[:6].strip()
        if rec == "MODEL":
            if first_model_only and i != first_model:
                break
            active = True
            continue
        if rec == "ENDMDL" and first_model is not None:
            if first_model_only:
                break
            active = False
            continue
        if not active or rec not in kinds:
            continue
        try:
            xyz = [float(line[s:s + 8]) for s in (30, 38, 46)]
        except ValueError as exc:
            raise ValueError("Invalid PDB coordinates in %s, line %d" % (source, i + 1)) from exc
        if not np.all(np.isfinite(xyz)):
            raise ValueError("Non-finite PDB coordinates in %s, line %d" % (source, i + 1))
        coords.append(xyz)
        els.append(infer_element(line))
        chains.append(line[21:22] or " ")
        idx.append(i)
    return PDBText(lines, np.asarray(coords, dtype=np.float32).reshape(-1, 3),
                   np.asarray(els, dtype="U2"), np.asarray(chains, dtype="U1"),
                   np.asarray(idx, dtype=np.int64))


def read_pdb(path, include_hetatm=True, first_model_only=True) -> PDBText:
    with open(path, "r", encoding="utf-8", errors="surrogateescape", newline="") as fh:
        lines = fh.readlines()
    return parse_pdb_lines(lines, include_hetatm, first_model_only, os.fspath(path))


def read_pdb_text(text: str, include_hetatm=True, first_model_only=True) -> PDBText:
    return parse_pdb_lines(text.splitlines(keepends=True), include_hetatm, first_model_only)


def rotation_matrix(pose) -> np.ndarray:
    """Row-convention matrix of the pose's rotation vector (degrees)."""
    from scipy.spatial.transform import Rotation
    pose = np.asarray(pose, dtype=np.float64)
    if pose.shape != (6,) or not np.all(np.isfinite(pose)):
        raise ValueError("Pose must contain six finite rotation/translation values")
    return Rotation.from_rotvec(np.deg2rad(pose[:3])).as_matrix()


def transform_coordinates(coords, pose, pivot=None) -> np.ndarray:
    coords = np.asarray(coords)
    if coords.ndim != 2 or coords.shape[1] != 3 or not len(coords):
        raise ValueError("A nonempty (N, 3) coordinate array is required")
    center = np.mean(coords, axis=0) if pivot is None else np.asarray(pivot, dtype=np.float64)
    return (coords - center) @ rotation_matrix(pose) + center + np.asarray(pose, dtype=np.float64)[3:]


def quantize_coordinates(xyz) -> np.ndarray:
    """PDB 8.3 write and reread, float32 result (Lite pdb_text.py:33-58)."""
    values = np.asarray(xyz, dtype=np.float64)
    if values.ndim != 2 or values.shape[1] != 3:
        raise ValueError("Coordinates must have shape (N, 3)")
    if not np.isfinite(values).all():
        raise ValueError("PDB coordinates must be finite")
    if np.any((values < -1001.0) | (values > 10001.0)):
        raise ValueError("Coordinate exceeds the PDB 8.3 field width")
    scaled = values * 1000.0
    rounded = np.rint(scaled) / 1000.0
    dist = np.abs((np.abs(scaled) - np.floor(np.abs(scaled))) - 0.5)
    amb = dist <= 2.0 * np.spacing(np.abs(scaled))
    if amb.any():
        rounded[amb] = [float(f"{float(v):8.3f}") for v in values[amb]]
    if np.any((rounded < -999.999) | (rounded > 9999.999)):
        raise ValueError("Coordinate exceeds the PDB 8.3 field width")
    return rounded.astype(np.float32)


@dataclass
class ChainSplit:
    """Atoms of one moving chain and of its fixed context, as the density
    sees them (all models, ATOM records unless HETATM is requested)."""

    moving_coords: np.ndarray   # [m, 3] float32 (first-model chain rows that are density atoms)
    moving_elements: np.ndarray
    fixed_coords: np.ndarray    # [f, 3] float32
    fixed_elements: np.ndarray
    pivot: np.ndarray           # [3] float32 mean of the chain's first-model atoms (HETATM included)


def split_moving_chain(pdb: PDBText, chain_id: str, include_hetatm: bool = False,
                       density_pdb: PDBText = None) -> ChainSplit:
    """Split density atoms into the moving chain and the fixed rest, keeping
    the pose pivot of transformed_density_atoms (Lite pdb_text.py:204-223):
    the float32 mean over the chain's first-model atoms."""
    first = pdb
    density = density_pdb if density_pdb is not None else first
    sel_first = first.chains == str(chain_id)
    if not np.any(sel_first):
        raise ValueError("Chain %r has no atoms in the first PDB model" % chain_id)
    pivot = np.mean(first.coords[sel_first], axis=0)
    moving_lines = set(int(i) for i in first.atom_line_indices[sel_first])
    moving = np.asarray([int(i) in moving_lines for i in density.atom_line_indices], dtype=bool)
    return ChainSplit(density.coords[moving].copy(), density.elements[moving].copy(),
                      density.coords[~moving].copy(), density.elements[~moving].copy(),
                      np.asarray(pivot, dtype=np.float32))
