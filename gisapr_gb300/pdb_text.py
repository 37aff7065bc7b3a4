"""PDB coordinates and the rigid-body pose of one chain (pdb_text.py of the
reference: element inference :26-46, reader :78-120, transform :123-142;
Lite tree: quantize_coordinates :33-58, transformed_density_atoms :204-223).

Only the host-side parsing lives here. The pose transform and the PDB 8.3
round trip of the moved chain run on the GPU inside the splat launch
(gisapr_deposit_moved); ``transform_coordinates`` and
``quantize_coordinates`` are kept for callers that want the coordinates.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass
from functools import lru_cache

import numpy as np

# Element symbols by period of the periodic table (Z = 1..118), plus "D"
# for deuterium. The element column and the atom-name rules below pick from
# this set; anything else counts as no element (weight 0 in the density).
_PERIODS = (
    "H He",
    "Li Be B C N O F Ne",
    "Na Mg Al Si P S Cl Ar",
    "K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr",
    "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe",
    "Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn",
    "Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr Rf Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og",
)
KNOWN_ELEMENTS = frozenset(sym.upper() for period in _PERIODS for sym in period.split()) | {"D"}

# Atom names that start in column 13 with one of these letters are that
# element in ATOM records (protein and nucleic-acid atom names), even when
# the first two letters would spell another element (" CA " vs "CA  ").
_ORGANIC_LEADS = frozenset("CNOHPS")


@lru_cache(maxsize=4096)
def _element_of(element_field: str, name_field: str, is_atom: bool) -> str:
    """Element of one atom from its element columns (77-78), its atom-name
    columns (13-16) and whether the record is ATOM. Decision order:

    1. a recognised symbol in the element columns wins;
    2. the alphabetic characters of the name decide otherwise, none -> "";
    3. a name whose first column is blank or a digit is aligned as a
       one-letter element: its first letter;
    4. in ATOM records a leading C, N, O, H, P or S is that element;
    5. else the first two letters if they spell an element, else the first.
    """
    sym = element_field.strip().upper()
    if sym in KNOWN_ELEMENTS:
        return sym
    name = name_field.ljust(4).upper()
    alpha = [ch for ch in name if ch.isalpha()]
    if not alpha:
        return ""
    lead = name[0]
    if lead.isspace() or lead.isdigit():
        choices = (alpha[0],)
    elif is_atom and alpha[0] in _ORGANIC_LEADS:
        choices = (alpha[0],)
    else:
        choices = ("".join(alpha[:2]), alpha[0])
    return next((c for c in choices if c in KNOWN_ELEMENTS), "")


def infer_element(line: str) -> str:
    """Element of one ATOM/HETATM line (upper case, "" when unknown)."""
    return _element_of(line[76:78], line[12:16], line[:6] == "ATOM  ")


@dataclass(frozen=True)
class PdbAtoms:
    """The selected atom records of a PDB text, in file order: the text's
    lines, xyz (float32), element, chain id and the line each atom came from.
    Identifiers other than the chain are never interpreted."""

    lines: list
    coords: np.ndarray             # [n, 3] float32
    elements: np.ndarray           # [n] U2
    chains: np.ndarray             # [n] U1
    atom_line_indices: np.ndarray  # [n] int64

    def __len__(self) -> int:
        return int(self.coords.shape[0])


# the reference's name for the same record set
PDBText = PdbAtoms


def _selected_line_mask(tags, first_model_only: bool) -> np.ndarray:
    """Lines inside the selected models. ``tags`` are the stripped record
    names (columns 1-6). Without MODEL records the whole text is one model.
    Otherwise lines count only inside a MODEL ... ENDMDL span; with
    ``first_model_only`` reading ends at the first ENDMDL or at the second
    MODEL, whichever comes first."""
    n = len(tags)
    model_at = [i for i, t in enumerate(tags) if t == "MODEL"]
    if not model_at:
        return np.ones(n, dtype=bool)
    inside = np.zeros(n, dtype=bool)
    if first_model_only:
        ends = [i for i, t in enumerate(tags) if t == "ENDMDL"] + model_at[1:2]
        stop = min(ends) if ends else n
        if stop > model_at[0]:
            inside[model_at[0] + 1:stop] = True
        return inside
    state = False
    for i, t in enumerate(tags):
        if t == "MODEL":
            state = True
        elif t == "ENDMDL":
            state = False
        else:
            inside[i] = state
    return inside


def parse_pdb_lines(lines, include_hetatm=True, first_model_only=True, source="<text>") -> PdbAtoms:
    """Atom records of ``lines`` (ATOM, and HETATM unless excluded) in the
    selected models. Raises ValueError naming the line when a coordinate
    field does not parse or is not finite."""
    tags = [ln[:6].strip() for ln in lines]
    wanted = {"ATOM", "HETATM"} if include_hetatm else {"ATOM"}
    inside = _selected_line_mask(tags, first_model_only)
    rows = [i for i, t in enumerate(tags) if inside[i] and t in wanted]
    xyz = np.empty((len(rows), 3), dtype=np.float64)
    for k, i in enumerate(rows):
        ln = lines[i]
        try:
            v = (float(ln[30:38]), float(ln[38:46]), float(ln[46:54]))
        except ValueError as exc:
            raise ValueError(f"{source}, line {i + 1}: columns 31-54 do not hold three coordinates") from exc
        if not all(map(math.isfinite, v)):
            raise ValueError(f"{source}, line {i + 1}: coordinates are not finite")
        xyz[k] = v
    elements = [infer_element(lines[i]) for i in rows]
    chains = [lines[i][21:22] or " " for i in rows]
    return PdbAtoms(list(lines), xyz.astype(np.float32).reshape(-1, 3), np.asarray(elements, dtype="U2"),
                    np.asarray(chains, dtype="U1"), np.asarray(rows, dtype=np.int64))


def read_pdb(path, include_hetatm=True, first_model_only=True) -> PdbAtoms:
    """Atom records of a PDB file (see parse_pdb_lines); the text is kept
    byte for byte (undecodable bytes survive as surrogates)."""
    with open(path, "r", encoding="utf-8", errors="surrogateescape", newline="") as fh:
        lines = fh.readlines()
    return parse_pdb_lines(lines, include_hetatm, first_model_only, os.fspath(path))


def read_pdb_text(text: str, include_hetatm=True, first_model_only=True) -> PdbAtoms:
    return parse_pdb_lines(text.splitlines(keepends=True), include_hetatm, first_model_only)


def rotation_matrix(pose) -> np.ndarray:
    """Row-convention matrix of the pose's rotation vector (degrees)."""
    from scipy.spatial.transform import Rotation
    pose = np.asarray(pose, dtype=np.float64)
    if pose.shape != (6,) or not np.all(np.isfinite(pose)):
        raise ValueError("Pose must contain six finite rotation/translation values")
    return Rotation.from_rotvec(np.deg2rad(pose[:3])).as_matrix()


def rotation_matrices(poses) -> np.ndarray:
    """rotation_matrix of every row of a (k, 6) pose array in one call,
    element for element the same matrices."""
    from scipy.spatial.transform import Rotation
    poses = np.asarray(poses, dtype=np.float64)
    if poses.ndim != 2 or poses.shape[1] != 6 or not np.all(np.isfinite(poses)):
        raise ValueError("Poses must be a (k, 6) array of finite rotation/translation values")
    if len(poses) == 0:
        return np.zeros((0, 3, 3))
    return Rotation.from_rotvec(np.deg2rad(poses[:, :3])).as_matrix().reshape(-1, 3, 3)


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


def split_moving_chain(pdb: PdbAtoms, chain_id: str, include_hetatm: bool = False,
                       density_pdb: PdbAtoms = None) -> ChainSplit:
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
