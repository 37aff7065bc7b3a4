"""Seeded synthetic search jobs with the shapes of GisAPR's published use.

The reference's timing dataset (EMPIAR-11241 particles and a user model) is
not available, so every workload here is generated from a seed:

* two chains of a confined, self-avoiding 3.8 A C-alpha walk, each residue
  expanded to N/CA/C/O/CB plus an S atom in 5 % of residues, centred on the
  origin and written as column-aligned PDB text that ``pdb_text.read_pdb``
  parses (chain in column 22, element in columns 77-78);
* HEALPix NEST directions written as RELION angles: rot = fmod(phi+360, 360)
  - 180 and tilt = acos(z), both in degrees (the reference's
  generate_healpix_order_and_relion_star.py:74-97 writes the same values);
* particles projected from the unperturbed model at uniform random SO(3)
  orientations, rotated in-plane, multiplied by a -sin(gamma) CTF (amplitude
  contrast 0.1), shifted by whole pixels, given white Gaussian noise at a
  stated SNR and whitened by radial amplitude, plane removal and
  normalisation (the reference's particle whitening in
  read_star_shift_crop_and_generate_new_star_v5.py:42-75 does the same);
* STAR-equivalent particle records whose angles are the true ones perturbed
  inside the local search window.

The projection used to make particles is a plain Fourier-slice projector in
PyTorch (CPU or CUDA). It is data generation, not the scoring path.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# ---------------------------------------------------------------------------
# Model atoms
# ---------------------------------------------------------------------------


def _ca_walk(n_res: int, rng: np.random.Generator, radius: float,
             start: Optional[np.ndarray] = None, step: float = 3.8,
             tries: int = 60) -> np.ndarray:
    """Self-avoiding 3.8 A walk kept inside a sphere of ``radius``."""
    pts = np.zeros((n_res, 3))
    pts[0] = start if start is not None else rng.normal(size=3) * radius * 0.2
    cell = step
    grid: Dict[Tuple[int, int, int], List[int]] = {}

    def key(p):
        return (int(math.floor(p[0] / cell)), int(math.floor(p[1] / cell)),
                int(math.floor(p[2] / cell)))

    grid.setdefault(key(pts[0]), []).append(0)
    for i in range(1, n_res):
        best = None
        for _ in range(tries):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            cand = pts[i - 1] + step * d
            if np.linalg.norm(cand) > radius:
                continue
            k = key(cand)
            clash = False
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                            if j != i - 1 and np.sum((pts[j] - cand) ** 2) < step * step:
                                clash = True
                                break
                        if clash:
                            break
                    if clash:
                        break
                if clash:
                    break
            if not clash:
                best = cand
                break
            if best is None:
                best = cand
        if best is None:  # every try left the sphere: step towards the centre
            d = -pts[i - 1] / max(np.linalg.norm(pts[i - 1]), 1e-9)
            best = pts[i - 1] + step * d
        pts[i] = best
        grid.setdefault(key(best), []).append(i)
    return pts


def _residue_atoms(ca: np.ndarray, rng: np.random.Generator, s_fraction: float):
    """Expand a C-alpha trace to N, CA, C, O, CB (+ SG) at ideal-ish offsets."""
    n = len(ca)
    coords, names, elements = [], [], []
    for i in range(n):
        prev_ = ca[i - 1] if i > 0 else ca[i] - (ca[i + 1] - ca[i])
        next_ = ca[i + 1] if i + 1 < n else ca[i] + (ca[i] - ca[i - 1])
        t = next_ - prev_
        t /= max(np.linalg.norm(t), 1e-9)
        u = np.cross(t, rng.normal(size=3))
        u /= max(np.linalg.norm(u), 1e-9)
        v = np.cross(t, u)
        a = ca[i]
        atoms = [
            ("N", "N", a - 1.20 * t + 0.80 * u),
            ("CA", "C", a),
            ("C", "C", a + 1.25 * t + 0.85 * u),
            ("O", "O", a + 1.60 * t + 1.95 * u + 0.30 * v),
            ("CB", "C", a - 0.55 * t - 0.75 * u + 1.25 * v),
        ]
        if rng.random() < s_fraction:
            atoms.append(("SG", "S", a - 0.90 * t - 1.30 * u + 2.60 * v))
        for name, el, xyz in atoms:
            coords.append(xyz)
            names.append(name)
            elements.append(el)
    return np.asarray(coords), names, elements


@dataclass
class SyntheticModel:
    """Atoms of a moving chain A and a fixed chain B, plus their PDB text."""

    coords: np.ndarray            # [n, 3] float64, chain A first
    elements: List[str]
    chains: List[str]
    pdb_text: str

    @property
    def moving(self) -> np.ndarray:
        return np.asarray([c == "A" for c in self.chains])


def _pdb_line(serial, name, resname, chain, resseq, xyz, element):
    nm = (" " + name).ljust(4) if len(name) < 4 else name
    return ("ATOM  %5d %-4s %3s %1s%4d    %8.3f%8.3f%8.3f%6.2f%6.2f          %2s\n"
            % (serial % 100000, nm, resname, chain, resseq % 10000,
               xyz[0], xyz[1], xyz[2], 1.0, 0.0, element.rjust(2)))


def make_model(n_moving_res: int, n_fixed_res: int, seed: int,
               radius: Optional[float] = None, s_fraction: float = 0.05) -> SyntheticModel:
    """Two seeded chains, each centred on the origin."""
    rng = np.random.default_rng(seed)
    chains_xyz = []
    for n_res in (n_moving_res, n_fixed_res):
        r = radius if radius is not None else max(12.0, 1.25 * (31.0 * n_res) ** (1.0 / 3.0))
        ca = _ca_walk(n_res, rng, r)
        xyz, names, els = _residue_atoms(ca, rng, s_fraction)
        xyz = xyz - xyz.mean(axis=0)
        chains_xyz.append((xyz, names, els))
    lines, coords, elements, chains = [], [], [], []
    serial = 1
    for chain, (xyz, names, els) in zip("AB", chains_xyz):
        res = 0
        for k, (p, nm, el) in enumerate(zip(xyz, names, els)):
            if nm == "N":
                res += 1
            # Round through the PDB field so text and arrays agree exactly.
            p = np.asarray([float(f"{v:8.3f}") for v in p])
            lines.append(_pdb_line(serial, nm, "ALA" if nm != "SG" else "CYS", chain, res, p, el))
            coords.append(p)
            elements.append(el)
            chains.append(chain)
            serial += 1
        lines.append("TER\n")
    lines.append("END\n")
    return SyntheticModel(np.asarray(coords), elements, chains, "".join(lines))


def residues_for_atoms(n_atoms: int, s_fraction: float = 0.05) -> int:
    return max(2, int(round(n_atoms / (5.0 + s_fraction))))


# ---------------------------------------------------------------------------
# Directions (HEALPix NEST), restated from the published pixelisation scheme
# ---------------------------------------------------------------------------

_JRLL = (2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4)
_JPLL = (1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7)


def _compress_bits(v: int) -> int:
    """Keep the even bits of v packed together (de-interleave)."""
    out = 0
    bit = 0
    while v:
        out |= (v & 1) << bit
        v >>= 2
        bit += 1
    return out


def healpix_nest_angles(order: int) -> Tuple[np.ndarray, np.ndarray]:
    """(phi, theta) in degrees of every NEST pixel centre (Gorski et al. 2005)."""
    nside = 1 << order
    npface = nside * nside
    npix = 12 * npface
    fact2 = 4.0 / npix
    fact1 = (nside << 1) * fact2
    nl4 = 4 * nside
    phi = np.empty(npix)
    theta = np.empty(npix)
    for pix in range(npix):
        face = pix >> (2 * order)
        p = pix & (npface - 1)
        ix = _compress_bits(p)
        iy = _compress_bits(p >> 1)
        jr = (_JRLL[face] << order) - ix - iy - 1
        if jr < nside:
            nr = jr
            z = 1 - nr * nr * fact2
            kshift = 0
        elif jr > 3 * nside:
            nr = nl4 - jr
            z = nr * nr * fact2 - 1
            kshift = 0
        else:
            nr = nside
            z = (2 * nside - jr) * fact1
            kshift = (jr - nside) & 1
        jp = (_JPLL[face] * nr + ix - iy + 1 + kshift) // 2
        if jp > nl4:
            jp -= nl4
        if jp < 1:
            jp += nl4
        ph = (jp - (kshift + 1) * 0.5) * (0.5 * np.pi / nr)
        phi[pix] = np.rad2deg(ph)
        theta[pix] = np.rad2deg(np.arccos(z))
    return phi, theta


def healpix_directions(order: int) -> Tuple[List[float], List[float]]:
    """RELION (rot, tilt) lists as the reference's direction STAR holds them."""
    phi, theta = healpix_nest_angles(order)
    rot = [math.fmod(float(p) + 360.0, 360.0) - 180.0 for p in phi]
    tilt = [math.fmod(float(t) + 360.0, 360.0) for t in theta]
    return rot, tilt


# ---------------------------------------------------------------------------
# Search jobs
# ---------------------------------------------------------------------------


@dataclass
class ParticleRecords:
    """STAR-equivalent particle rows (rlnAngleRot/Tilt/Psi, defocus)."""

    line_index: np.ndarray
    rot: np.ndarray
    tilt: np.ndarray
    psi: np.ndarray
    defocus_u: np.ndarray
    defocus_v: np.ndarray
    defocus_angle: np.ndarray


@dataclass
class WorkloadSpec:
    name: str
    box: int
    apix: float
    n_moving_atoms: int
    n_fixed_atoms: int
    n_particles: int
    healpix_order: int
    local_range: float
    psi_step: float
    trans_range: int
    snr: float = 0.05
    defocus_range: Tuple[float, float] = (10000.0, 25000.0)
    fsc_half_res: Optional[float] = 4.0       # None = unit FSC
    voltage: float = 300.0
    cs: float = 2.7
    kk: float = 3.0
    newbox: Optional[int] = None
    mask_edge: int = 6
    pose_rotation_deg: float = 3.0
    pose_translation: float = 1.5

    @property
    def crop(self) -> int:
        return 2 * self.trans_range + 2

    @property
    def new_box(self) -> int:
        return self.newbox or self.box

    @property
    def mask_radius(self) -> int:
        return int(round(0.43 * self.box))

    @property
    def res(self) -> float:
        return 2.0 * self.apix


WORKLOADS = {
    # configs of the published use, one per mode
    "box64_200p": WorkloadSpec("box64_200p", 64, 1.5, 760, 3030, 200, 2, 15.0, 15.0, 4,
                               snr=0.05, fsc_half_res=None),
    "box128_5kp": WorkloadSpec("box128_5kp", 128, 1.1, 3000, 20000, 5000, 3, 10.0, 7.5, 5),
    "box256_20kp": WorkloadSpec("box256_20kp", 256, 0.85, 8000, 60000, 20000, 4, 6.0, 3.75, 6,
                                snr=0.03, defocus_range=(8000.0, 30000.0)),
    # small cases for tests
    "box32_tiny": WorkloadSpec("box32_tiny", 32, 3.0, 200, 600, 24, 1, 30.0, 15.0, 3,
                               fsc_half_res=None, mask_edge=3),
    "box64_small": WorkloadSpec("box64_small", 64, 1.5, 760, 3030, 48, 2, 15.0, 15.0, 4,
                                fsc_half_res=8.0),
    "box96_tiny": WorkloadSpec("box96_tiny", 96, 2.0, 300, 900, 16, 1, 30.0, 15.0, 3,
                               fsc_half_res=8.0, mask_edge=3),
    # the serving stream's other box sizes (3 * 2^k)
    "box96_serve": WorkloadSpec("box96_serve", 96, 1.1, 1000, 8000, 1000, 3, 10.0, 7.5, 5),
    "box192_serve": WorkloadSpec("box192_serve", 192, 1.1, 6000, 20000, 2000, 3, 10.0, 7.5, 5),
}


def logistic_fsc(box: int, apix: float, half_res: Optional[float]) -> np.ndarray:
    """FSC per shell k (resolution box*apix/k), logistic, 0.5 at ``half_res``."""
    if half_res is None:
        return np.ones(box, dtype=np.float32)
    k = np.arange(box, dtype=np.float64)
    res = np.where(k > 0, box * apix / np.maximum(k, 1e-9), np.inf)
    freq = np.where(np.isfinite(res), 1.0 / res, 0.0)
    f0 = 1.0 / half_res
    return (1.0 / (1.0 + np.exp((freq - f0) / (0.08 * f0)))).astype(np.float32)


def blob_density(n: int, seed: int) -> np.ndarray:
    """Six Gaussian blobs around the box centre plus 0.2 white noise, float32
    [z, y, x], from ``seed``. The noise keeps every radial shell of the
    spectrum well above float32 rounding (the whitening rescales each shell
    to unit mean amplitude), so template comparisons at any box measure the
    arithmetic, not rounding noise in empty shells."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float64),) * 3, indexing="ij")
    v = 0.2 * rng.standard_normal((n, n, n))
    for _ in range(6):
        c = n / 2 + rng.normal(scale=n / 10, size=3)
        s = rng.uniform(1.5, n / 16)
        v += rng.uniform(0.5, 2.0) * np.exp(-((z - c[0]) ** 2 + (y - c[1]) ** 2 + (x - c[2]) ** 2) / (2 * s * s))
    return v.astype(np.float32)


def random_rotations(n: int, rng: np.random.Generator):
    """Uniform SO(3) as RELION (rot, tilt, psi) degrees."""
    rot = rng.uniform(-180.0, 180.0, n)
    tilt = np.rad2deg(np.arccos(rng.uniform(-1.0, 1.0, n)))
    psi = rng.uniform(0.0, 360.0, n)
    return rot, tilt, psi


def candidate_poses(n: int, seed: int, max_rot_deg: float, max_trans: float,
                    exact: bool = False) -> np.ndarray:
    """Rigid-body perturbations [n, 6]: rotvec in degrees about random axes,
    then a translation in A. ``exact`` uses the full magnitudes."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 6))
    for i in range(n):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        tr = rng.normal(size=3)
        tr /= np.linalg.norm(tr)
        a = max_rot_deg if exact else rng.uniform(-max_rot_deg, max_rot_deg)
        t = max_trans if exact else rng.uniform(0.0, max_trans)
        out[i, :3] = a * ax
        out[i, 3:] = t * tr
    return out


def ctf_full(size: int, pixel: float, dfu, dfv, dfa_deg, voltage=300.0, cs=2.7, amp=0.1):
    """Centered full-grid -sin(gamma) CTF, float64 (data generation only)."""
    kv = voltage * 1e3
    lam = 12.2643247 / math.sqrt(kv * (1.0 + kv * 0.978466e-6))
    k1 = math.pi * lam
    k2 = math.pi / 2.0 * cs * 1e7 * lam ** 3
    k3 = math.atan(amp / math.sqrt(1.0 - amp * amp))
    f = (np.arange(size) - size / 2.0) / (size * pixel)
    x, y = np.meshgrid(f, f, indexing="xy")
    a = math.radians(dfa_deg)
    sa, ca = math.sin(a), math.cos(a)
    axx = -dfu * ca * ca - dfv * sa * sa
    ayy = -dfu * sa * sa - dfv * ca * ca
    axy = -dfu * sa * ca + dfv * sa * ca
    u2 = x * x + y * y
    g = k1 * (axx * x * x + 2 * axy * x * y + ayy * y * y) + k2 * u2 * u2 - k3
    return -np.sin(g)


def whiten_particle(img: np.ndarray) -> np.ndarray:
    """Radial amplitude flattening, least-squares plane removal, normalisation."""
    n = img.shape[-1]
    F = np.fft.fftshift(np.fft.fft2(img))
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    d = np.round(np.sqrt((j - n // 2) ** 2 + (i - n // 2) ** 2)).astype(int)
    spec = np.bincount(d.ravel(), weights=np.abs(F).ravel())
    cnt = np.bincount(d.ravel())
    div = np.ones_like(spec)
    nz = (cnt > 0) & (spec > 0)
    div[nz] = cnt[nz] / spec[nz]
    div[0] = 1.0
    out = np.fft.ifft2(np.fft.ifftshift(F * div[d])).real
    A = np.stack([i.ravel(), j.ravel(), np.ones(n * n)], 1).astype(np.float64)
    coef, *_ = np.linalg.lstsq(A, out.ravel(), rcond=None)
    out = out - (coef[0] * i + coef[1] * j + coef[2])
    s = out.std()
    return (out - out.mean()) / s if s > 0 else out - out.mean()


def _project_fourier(volume: np.ndarray, rot, tilt, device="cpu", batch=256) -> np.ndarray:
    """Fourier-slice projections at euler(rot, tilt, 0) in the template geometry."""
    import torch
    import torch.nn.functional as F
    dev = torch.device(device)
    n = volume.shape[0]
    m = 2 * n
    v = torch.as_tensor(np.asarray(volume, dtype=np.float32), device=dev)
    v = F.pad(v, [n // 2] * 6)
    dft = torch.fft.fftshift(torch.fft.rfftn(torch.fft.fftshift(v)), dim=(0, 1))
    dre = torch.view_as_real(dft).permute(3, 0, 1, 2).unsqueeze(0).contiguous()
    del v, dft
    fy = torch.fft.fftshift(torch.fft.fftfreq(m, device=dev))
    fx = torch.fft.rfftfreq(m, device=dev)
    yy, xx = torch.meshgrid(fy, fx, indexing="ij")
    out = np.empty((len(rot), n, n), dtype=np.float32)
    shape = torch.tensor([m, m, n + 1], dtype=torch.float32, device=dev)
    for s in range(0, len(rot), batch):
        e = min(s + batch, len(rot))
        mats = []
        for r, t in zip(rot[s:e], tilt[s:e]):
            a, b = math.radians(r), math.radians(t)
            ca, sa, cb, sb = math.cos(a), math.sin(a), math.cos(b), math.sin(b)
            M = np.array([[cb * ca, cb * sa, -sb], [-sa, ca, 0.0], [sb * ca, sb * sa, cb]])
            mats.append(M.T)
        R = torch.as_tensor(np.asarray(mats, dtype=np.float32), device=dev)
        rx = R[:, 0, 0, None, None] * xx + R[:, 0, 1, None, None] * yy
        ry = R[:, 1, 0, None, None] * xx + R[:, 1, 1, None, None] * yy
        rz = R[:, 2, 0, None, None] * xx + R[:, 2, 1, None, None] * yy
        neg = rx < 0
        sgn = torch.where(neg, -1.0, 1.0)
        cz = rz * sgn * m + m // 2
        cy = ry * sgn * m + m // 2
        cx = rx * sgn * m
        grid = torch.stack((cx, cy, cz), -1) / (0.5 * shape.flip(0) - 0.5) - 1.0
        smp = F.grid_sample(dre, grid.unsqueeze(0), mode="bilinear", padding_mode="border",
                            align_corners=True)[0]
        c = torch.complex(smp[0], smp[1])
        c = torch.where(neg, torch.conj(c), c)
        p = torch.fft.irfftn(torch.fft.ifftshift(c, dim=-2), dim=(-2, -1))
        p = torch.fft.ifftshift(p, dim=(-2, -1))[:, n // 2:n // 2 + n, n // 2:n // 2 + n]
        out[s:e] = p.float().cpu().numpy()
    return out


def _rotate_bilinear(img: np.ndarray, angle_deg: float) -> np.ndarray:
    """Inverse of the search's psi rotation: out(q) = img(R(-a)(q - c) + c)."""
    n = img.shape[0]
    c = n / 2.0
    th = math.radians(-angle_deg)
    co, si = math.cos(th), math.sin(th)
    yy, xx = np.meshgrid(np.arange(n, dtype=np.float64), np.arange(n, dtype=np.float64),
                         indexing="ij")
    sy = co * (yy - c) - si * (xx - c) + c
    sx = si * (yy - c) + co * (xx - c) + c
    y0, x0 = np.floor(sy).astype(int), np.floor(sx).astype(int)
    ty, tx = sy - y0, sx - x0
    out = np.zeros_like(yy)
    for dy, wy in ((0, 1 - ty), (1, ty)):
        for dx, wx in ((0, 1 - tx), (1, tx)):
            yi, xi = y0 + dy, x0 + dx
            ok = (yi >= 0) & (yi < n) & (xi >= 0) & (xi < n)
            out += np.where(ok, wy * wx * img[np.clip(yi, 0, n - 1), np.clip(xi, 0, n - 1)], 0.0)
    return out


@dataclass
class SearchJob:
    """Everything one refinement job holds while candidates are scored."""

    spec: WorkloadSpec
    model: SyntheticModel
    model_rot: List[float]
    model_tilt: List[float]
    images: np.ndarray              # [n_particles, box, box] float32
    records: ParticleRecords
    fsc: np.ndarray                 # per-shell values, len box
    true_angles: np.ndarray = field(default=None)  # [n, 3] rot, tilt, psi
    true_shifts: np.ndarray = field(default=None)  # [n, 2] y, x pixels


def make_job(spec: WorkloadSpec, seed: int = 1, device: str = "cpu",
             n_particles: Optional[int] = None, truth_volume: Optional[np.ndarray] = None,
             model: Optional[SyntheticModel] = None) -> SearchJob:
    """Build the seeded job for ``spec``. ``truth_volume`` is the density of
    the unperturbed model; it is computed here with a plain float64 splat if
    not given."""
    rng = np.random.default_rng(seed)
    if model is None:
        model = make_model(residues_for_atoms(spec.n_moving_atoms),
                           residues_for_atoms(spec.n_fixed_atoms), seed)
    if truth_volume is None:
        truth_volume = reference_density(model.coords, model.elements, spec.box, spec.apix, spec.res)
    n = spec.box
    n_p = spec.n_particles if n_particles is None else int(n_particles)
    rot, tilt, psi = random_rotations(n_p, rng)
    proj = _project_fourier(truth_volume, rot, tilt, device=device)
    dfu = rng.uniform(*spec.defocus_range, n_p)
    dfv = np.clip(dfu + rng.uniform(-1500.0, 1500.0, n_p), spec.defocus_range[0], spec.defocus_range[1])
    dfa = rng.uniform(0.0, 180.0, n_p)
    tmax = max(1, spec.trans_range - 1)
    shifts = rng.integers(-tmax, tmax + 1, size=(n_p, 2))
    images = np.empty((n_p, n, n), dtype=np.float32)
    for i in range(n_p):
        p = _rotate_bilinear(proj[i].astype(np.float64), psi[i])
        ctf = ctf_full(n, spec.apix, dfu[i], dfv[i], dfa[i], spec.voltage, spec.cs)
        p = np.fft.ifft2(np.fft.ifftshift(np.fft.fftshift(np.fft.fft2(p)) * ctf)).real
        p = np.roll(p, (int(shifts[i, 0]), int(shifts[i, 1])), axis=(0, 1))
        sig = p.var()
        noise = rng.normal(size=p.shape) * math.sqrt(sig / spec.snr) if sig > 0 else 0.0
        images[i] = whiten_particle(p + noise).astype(np.float32)
    half = spec.local_range * 0.5
    rec = ParticleRecords(
        line_index=np.arange(n_p, dtype=np.int64) + 20,
        rot=rot + rng.uniform(-half, half, n_p),
        tilt=np.clip(tilt + rng.uniform(-half, half, n_p), 0.0, 180.0),
        psi=(psi + rng.uniform(-0.5 * spec.psi_step, 0.5 * spec.psi_step, n_p)) % 360.0,
        defocus_u=dfu, defocus_v=dfv, defocus_angle=dfa)
    mrot, mtilt = healpix_directions(spec.healpix_order)
    return SearchJob(spec, model, mrot, mtilt, images, rec,
                     logistic_fsc(n, spec.apix, spec.fsc_half_res),
                     np.stack([rot, tilt, psi], 1), shifts)


def job_from_pool(pool: SearchJob, n_particles: int, seed: int) -> SearchJob:
    """A job of ``n_particles`` particles drawn (with repeats) from a pool
    job of the same model and box: each drawn particle keeps its image, its
    STAR angles and defocus, and gets its own STAR line. Large serving jobs
    (up to 20,000 particles) are built this way in seconds; the search work
    per particle has the pool's distribution."""
    rng = np.random.default_rng(seed)
    n_pool = len(pool.records.rot)
    pick = np.arange(int(n_particles)) % n_pool if n_particles <= n_pool else \
        np.concatenate([np.arange(n_pool), rng.integers(0, n_pool, size=int(n_particles) - n_pool)])
    r = pool.records
    rec = ParticleRecords(line_index=np.arange(len(pick), dtype=np.int64) + 20, rot=r.rot[pick],
                          tilt=r.tilt[pick], psi=r.psi[pick], defocus_u=r.defocus_u[pick],
                          defocus_v=r.defocus_v[pick], defocus_angle=r.defocus_angle[pick])
    return SearchJob(pool.spec, pool.model, pool.model_rot, pool.model_tilt, pool.images[pick], rec, pool.fsc,
                     None if pool.true_angles is None else pool.true_angles[pick],
                     None if pool.true_shifts is None else pool.true_shifts[pick])


def reference_density(coords, elements, box, apix, res) -> np.ndarray:
    """Plain float64 Gaussian splat used only to make particles."""
    z = np.asarray([{"H": 1, "C": 6, "N": 7, "O": 8, "P": 15, "S": 16}.get(e.upper(), 0)
                    for e in elements], dtype=np.float64)
    width = int(round(res * 3.0 / apix))
    rp = (math.pi / (res / apix)) ** 2
    kn = (rp / math.pi) ** 1.5
    pos = np.asarray(coords, dtype=np.float64) / apix + box // 2
    vol = np.zeros(box ** 3)
    ax = np.arange(-width, width + 1)
    oz, oy, ox = np.meshgrid(ax, ax, ax, indexing="ij")
    off = np.stack([ox.ravel(), oy.ravel(), oz.ravel()], 1)
    for s in range(0, len(pos), 1024):
        p = pos[s:s + 1024]
        base = np.round(p).astype(int)
        v = base[:, None, :] + off[None]
        ok = ((v >= 0) & (v < box)).all(2)
        r = np.sqrt(((v - p[:, None, :]) ** 2).sum(2))
        val = z[s:s + 1024, None] * kn * np.exp(-r * rp)
        idx = v[..., 0] + box * (v[..., 1] + box * v[..., 2])
        vol += np.bincount(idx[ok], weights=val[ok], minlength=box ** 3)
    return vol.reshape(box, box, box).astype(np.float32)


def make_models_shared_fixed(moving_atoms: Sequence[int], n_fixed_atoms: int, seed: int,
                             s_fraction: float = 0.05) -> List[SyntheticModel]:
    """Models that share one fixed chain B and differ in the moving chain A
    (the mixed 1,500 / 3,000 / 6,000-atom batches). Chain B comes from its
    own seeded generator, so it is identical in every model."""
    rng_b = np.random.default_rng(seed + 7919)
    nb = residues_for_atoms(n_fixed_atoms, s_fraction)
    rb = max(12.0, 1.25 * (31.0 * nb) ** (1.0 / 3.0))
    xb, names_b, els_b = _residue_atoms(_ca_walk(nb, rng_b, rb), rng_b, s_fraction)
    xb = xb - xb.mean(axis=0)
    models = []
    for k, n_atoms in enumerate(moving_atoms):
        rng_a = np.random.default_rng(seed + 104729 * (k + 1))
        na = residues_for_atoms(n_atoms, s_fraction)
        ra = max(12.0, 1.25 * (31.0 * na) ** (1.0 / 3.0))
        xa, names_a, els_a = _residue_atoms(_ca_walk(na, rng_a, ra), rng_a, s_fraction)
        xa = xa - xa.mean(axis=0)
        lines, coords, elements, chains = [], [], [], []
        serial = 1
        for chain, (xyz, names, els) in zip("AB", ((xa, names_a, els_a), (xb, names_b, els_b))):
            res = 0
            for p, nm, el in zip(xyz, names, els):
                if nm == "N":
                    res += 1
                p = np.asarray([float(f"{v:8.3f}") for v in p])
                lines.append(_pdb_line(serial, nm, "ALA" if nm != "SG" else "CYS", chain, res, p, el))
                coords.append(p)
                elements.append(el)
                chains.append(chain)
                serial += 1
            lines.append("TER\n")
        lines.append("END\n")
        models.append(SyntheticModel(np.asarray(coords), elements, chains, "".join(lines)))
    return models
