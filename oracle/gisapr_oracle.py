"""CPU oracle for GisAPR's candidate-scoring path -- TEST INFRASTRUCTURE ONLY.

This module checks the product and is never part of it. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it. The ``gisapr_gb300`` package never imports it and has no CPU fallback.

It restates, in numpy, what the reference computes for one candidate pose:

* a1  pose transform and PDB 8.3 round trip   pdb_text.py:123-142,
      ZL pdb_text.py:33-58 and 204-223
* a2  Gaussian atom splat                      pdb2mrc_gpu_ver_fp32_v3.py:41-98
* a3  pad, real-space sinc^2, 3-D R2C          v606:837-853, 1063-1073
* a4  central-slice trilinear gather           v606:856-896, 1094-1113
* a5  per-orientation template tail            v606:899-992, 1115-1147
* a6  packed CTF with ISSPA weight             v606:549-692 and 695-829
* a7  psi sampling, rotation grids, particle   v606:1163-1256, 1321-1374
* a8  pruned inverse transform + crop maximum  v606:1418-1449
* a9  per-particle result record               v606:1452-1516
* a10 host tables (Euler, local map, mask, FSC, packed layout)
                                               v606:168-187, 331-378, 446-541
* a11 candidate score sum(exp(rawCC/1024))     ZL gisapr_batch_search.py:361

"v606" is test1_with_isspa_weight_varingKK_search_translation_also_v606_torch_
optimized_standalone.py; "ZL" is the GisAPR-Lite-v1.3.2 tree.

Precision policy. Where the reference's own float32 rounding decides the
result (CTF phase gamma, which reaches hundreds of radians; splat positions,
voxel bounds and exponent arguments; slice and psi-rotation sampling
coordinates) this module repeats the reference's float32 operations in the
same order. Everything else (FFTs, sums, solves, interpolation arithmetic) is
float64, so the oracle is at least as accurate as the reference.

Pinning. tests/golden/make_golden.py runs the reference itself on seeded
inputs and stores its outputs; tests/test_oracle_golden.py checks this module
against those fixtures.
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np
import scipy.fft as sfft

f32 = np.float32
f64 = np.float64

# --------------------------------------------------------------------------
# a1: pose transform and PDB 8.3 round trip
# --------------------------------------------------------------------------

ELEMENT_Z = {"H": 1.0, "C": 6.0, "N": 7.0, "O": 8.0, "P": 15.0, "S": 16.0}


def atomic_numbers(elements: Sequence[str]) -> np.ndarray:
    """Z per element, 0 for anything else (pdb2mrc_gpu_ver_fp32_v3.py:13-22)."""
    return np.asarray([ELEMENT_Z.get(str(e).upper(), 0.0) for e in elements], dtype=f64)


def transform_coordinates(coords, pose, pivot=None) -> np.ndarray:
    """(c - pivot) @ R(rotvec deg) + pivot + t, float64 (pdb_text.py:123-142)."""
    from scipy.spatial.transform import Rotation

    coords = np.asarray(coords)
    pose = np.asarray(pose, dtype=f64)
    center = np.mean(coords, axis=0) if pivot is None else np.asarray(pivot, dtype=f64)
    matrix = Rotation.from_rotvec(np.deg2rad(pose[:3])).as_matrix()
    return (coords - center) @ matrix + center + pose[3:]


def quantize_8_3(xyz) -> np.ndarray:
    """Write each coordinate with "%8.3f" and read it back as float32.

    This is the PDB write/reread of the moved chain (pdb_text.py:65-71 writes,
    ZL pdb_text.py:204-223 rereads). Python's formatter rounds the exact binary
    value half-to-even, which is what this restatement uses, one value at a time.
    """
    values = np.asarray(xyz, dtype=f64)
    out = np.empty(values.shape, dtype=f32)
    flat_in = values.reshape(-1)
    flat_out = out.reshape(-1)
    for i, v in enumerate(flat_in):
        field = f"{float(v):8.3f}"
        if len(field) != 8:
            raise ValueError("Coordinate exceeds the PDB 8.3 field width")
        flat_out[i] = f32(float(field))
    return out


# --------------------------------------------------------------------------
# a2: Gaussian atom splat
# --------------------------------------------------------------------------


def density_parameters(apix: float, res: float) -> Tuple[int, float, float]:
    """Cube half-width w, rp = (pi*apix/res)^2, kn = (rp/pi)^1.5 (pdb2mrc:54-58)."""
    width = int(round(res * 3.0 / apix))
    rp = float(np.power(np.pi / (res / apix), 2))
    kn = float(np.power(rp / np.pi, 1.5))
    return width, rp, kn


def _round_away(v: np.ndarray) -> np.ndarray:
    v = v.astype(f64)
    return (np.sign(v) * np.floor(np.abs(v) + 0.5)).astype(np.int64)


def splat_density(coords, numbers, box: int, apix: float, res: float,
                  initial=None, chunk_atoms: int = 2048) -> np.ndarray:
    """Density [z, y, x] with a float64 accumulator (pdb2mrc:41-98).

    Per atom: p = f32(f64(xyz)/apix + box//2); voxel bounds are
    round-half-away(f32(p -/+ w)), lower clipped at 0, upper clipped at box-1
    and exclusive; per voxel r = sqrtf((dx*dx + dy*dy) + dz*dz) in float32,
    value = f32(f64(Z)*kn * f64(expf(f32(-f64(r)*rp)))). Atoms with Z = 0 or
    wholly outside the box add nothing. ``initial`` is the fixed-context
    density the moving atoms are added onto (ZL pdb2mrc v4:71-75).
    """
    width, rp, kn = density_parameters(apix, res)
    if width < 3:
        raise ValueError("You do not have sufficient sampling for this resolution. Decrease apix.")
    xyz = np.asarray(coords, dtype=f32).reshape(-1, 3)
    z = np.asarray(numbers, dtype=f32).reshape(-1)
    acc = np.zeros(box ** 3, dtype=f64)
    if initial is not None:
        acc += np.asarray(initial, dtype=f64).reshape(-1)
    if len(xyz) == 0:
        return acc.reshape(box, box, box)
    if not np.isfinite(xyz).all():
        raise ValueError("PDB coordinates must be finite")
    pos = (xyz.astype(f64) / apix + box // 2).astype(f32)
    lower = _round_away((pos - f32(width)))
    upper = _round_away((pos + f32(width)))
    keep = (lower < box).all(1) & (upper >= 0).all(1) & (z != 0)
    pos, z, lower, upper = pos[keep], z[keep], lower[keep], upper[keep]
    lower = np.maximum(lower, 0)
    upper = np.minimum(upper, box - 1)
    axis = np.arange(2 * width + 1)
    oz, oy, ox = np.meshgrid(axis, axis, axis, indexing="ij")
    offsets = np.stack((ox.ravel(), oy.ravel(), oz.ravel()), axis=1)  # x, y, z
    zk = z.astype(f64) * kn
    for s in range(0, len(pos), chunk_atoms):
        e = s + chunk_atoms
        vox = lower[s:e, None, :] + offsets[None]
        valid = (vox < upper[s:e, None, :]).all(2)
        d = vox.astype(f32) - pos[s:e, None, :]
        sq = d * d
        r = np.sqrt((sq[..., 0] + sq[..., 1]) + sq[..., 2])
        expo = (-(r.astype(f64)) * rp).astype(f32)
        val = (zk[s:e, None] * np.exp(expo).astype(f64)).astype(f32)
        idx = vox[..., 0] + box * (vox[..., 1] + box * vox[..., 2])
        acc += np.bincount(idx[valid], weights=val[valid].astype(f64), minlength=box ** 3)
    return acc.reshape(box, box, box)


# --------------------------------------------------------------------------
# a10: host tables
# --------------------------------------------------------------------------

_PI_REF = 3.14159265359  # the reference's own literal (v606:170-172)


def euler_angles_to_matrix(alpha: float, beta: float, gamma: float):
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


def rotation_matrices_t(rot: Sequence[float], tilt: Sequence[float]) -> np.ndarray:
    """float32 transpose of euler(rot, tilt, 0) per direction (v606:216-218)."""
    return np.stack([np.asarray(euler_angles_to_matrix(r, t, 0.0), dtype=f32).T
                     for r, t in zip(rot, tilt)]).astype(f32)


def angular_distance(r1, t1, p1, r2, t2, p2) -> float:
    """Mean per-axis angle between two Euler frames, degrees (v606:331-348)."""
    e1 = euler_angles_to_matrix(r1, t1, p1)
    e2 = euler_angles_to_matrix(r2, t2, p2)
    total = 0.0
    for i in range(3):
        dot = 0.0
        for a, b in zip(e1[i], e2[i]):
            dot += float(a) * float(b)
        dot = min(max(dot, -1.0), 1.0)
        total += math.acos(dot) * 180.0 / _PI_REF
    return total / 3.0


def local_orientations(p_rot, p_tilt, m_rot, m_tilt, local_range) -> List[List[int]]:
    """Directions within +-range of each particle's angles (v606:351-378)."""
    m_rot = np.asarray(m_rot)
    m_tilt = np.asarray(m_tilt)
    out = []
    for pr, pt in zip(p_rot, p_tilt):
        rd = np.fabs((m_rot - pr + 180.0) % 360.0 - 180.0)
        td = np.fabs((m_tilt - pt + 180.0) % 360.0 - 180.0)
        sel = []
        for k in np.where((rd <= local_range) & (td <= local_range))[0]:
            d = angular_distance(float(m_rot[k]), float(m_tilt[k]), 0.0, pr, pt, 0.0)
            if abs(d) <= local_range:
                sel.append(int(k))
        out.append(sel)
    return out


def soft_mask(size: int, radius: int, edge: int) -> np.ndarray:
    """Cosine-edged disc (v606:446-457)."""
    c = size // 2
    y, x = np.indices((size, size))
    d = np.sqrt((x - c) ** 2 + (y - c) ** 2)
    m = np.zeros_like(d)
    m[d <= radius] = 1.0
    if edge > 0:
        e = (d > radius) & (d <= radius + edge)
        m[e] = 0.5 * (1.0 + np.cos(np.pi * (d[e] - radius) / edge))
    return m.astype(f32)


def radial_map(values, size: int) -> np.ndarray:
    """Centered map of values[int(radius)] (v606:460-469)."""
    v = np.asarray(values, dtype=f32).reshape(-1)
    c = size // 2
    y, x = np.indices((size, size))
    r = np.sqrt((y - c) ** 2 + (x - c) ** 2).astype(np.int64)
    out = np.zeros((size, size), dtype=f32)
    ok = r < v.shape[0]
    out[ok] = v[r[ok]]
    return out


def centered_to_packed(centered: np.ndarray) -> np.ndarray:
    """fftshift(full)[:, :n//2+1] index permutation (v606:494-533)."""
    n = centered.shape[-1]
    h = n // 2
    rows = np.concatenate((np.arange(h, n), np.arange(0, h)))
    cols = np.concatenate((np.arange(h, n), [0]))
    return centered[..., rows, :][..., cols]


def pre_shift(packed: np.ndarray) -> np.ndarray:
    """fftshift over both packed dims (v606:535-537)."""
    return np.fft.fftshift(packed, axes=(-2, -1))


# --------------------------------------------------------------------------
# a3-a5: projector
# --------------------------------------------------------------------------


def volume_spectrum(volume) -> np.ndarray:
    """Pad N/2 per side, multiply by sinc^2(|f|), fftshift, rfftn, fftshift(z,y).

    Returns the (2N, 2N, N+1) complex128 half volume in the reference's layout
    (v606:1063-1073, filter v606:837-853).
    """
    vol = np.asarray(volume, dtype=f64)
    n = vol.shape[0]
    m = 2 * n
    padded = np.pad(vol, n // 2)
    f = np.fft.fftshift(np.fft.fftfreq(m))
    r = np.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + f[None, None, :] ** 2)
    padded *= np.sinc(r) ** 2
    dft = sfft.rfftn(np.fft.fftshift(padded))
    return np.fft.fftshift(dft, axes=(0, 1))


def _fftfreq_f32(m: int) -> np.ndarray:
    k = np.concatenate((np.arange(0, (m + 1) // 2), np.arange(-(m // 2), 0))).astype(f32)
    return k * f32(1.0 / m)


def slice_pixel_coordinates(rot_t: np.ndarray, n: int):
    """Sampling positions of one central slice, float32 as the reference.

    Base grid (z=0, y=fftshift(fftfreq(2N)), x=rfftfreq(2N)); rotate by the
    stored transposed matrix; negate where x<0 (and conjugate later); scale
    to voxel units; normalise for grid_sample and un-normalise it again with
    align_corners=True; clamp for border padding (v606:856-896, 1099-1105).
    Returns (iz, iy, ix) float32 voxel coordinates and the conjugate mask.
    """
    m = 2 * n
    fy = np.fft.fftshift(_fftfreq_f32(m))
    fx = (np.arange(n + 1).astype(f32) * f32(1.0 / m))
    yy, xx = np.meshgrid(fy, fx, indexing="ij")
    R = np.asarray(rot_t, dtype=f32)
    # The reference's batched 3x3 matmul rounds each product and the sum in
    # float32 (no fused multiply-add). Points where R00*x + R01*y cancels sit
    # on the conjugation boundary, so the rounding order decides the sample.
    rx = (R[0, 0] * xx + R[0, 1] * yy).astype(f32)
    ry = (R[1, 0] * xx + R[1, 1] * yy).astype(f32)
    rz = (R[2, 0] * xx + R[2, 1] * yy).astype(f32)
    conj = rx < 0
    rx = np.where(conj, -rx, rx)
    ry = np.where(conj, -ry, ry)
    rz = np.where(conj, -rz, rz)
    dims = (m, m, n + 1)  # dft shape z, y, x
    cz = rz * f32(m) + f32(m // 2)
    cy = ry * f32(m) + f32(m // 2)
    cx = rx * f32(m)
    out = []
    for c, size in zip((cz, cy, cx), dims):
        norm = c / (f32(0.5) * f32(size) - f32(0.5)) - f32(1.0)
        pix = ((norm + f32(1.0)) / f32(2.0)) * f32(size - 1)
        out.append(np.minimum(f32(size - 1), np.maximum(pix, f32(0.0))).astype(f32))
    return out[0], out[1], out[2], conj


def trilinear_border(dft: np.ndarray, iz, iy, ix) -> np.ndarray:
    """grid_sample trilinear on already-clamped voxel coordinates, float64."""
    D, H, W = dft.shape
    iz, iy, ix = (np.asarray(a, dtype=f64) for a in (iz, iy, ix))
    z0, y0, x0 = np.floor(iz), np.floor(iy), np.floor(ix)
    tz, ty, tx = iz - z0, iy - y0, ix - x0
    z0, y0, x0 = z0.astype(np.int64), y0.astype(np.int64), x0.astype(np.int64)
    out = np.zeros(iz.shape, dtype=np.complex128)
    for dz, wz in ((0, 1 - tz), (1, tz)):
        for dy, wy in ((0, 1 - ty), (1, ty)):
            for dx, wx in ((0, 1 - tx), (1, tx)):
                zz, yy, xx = z0 + dz, y0 + dy, x0 + dx
                ok = (zz < D) & (yy < H) & (xx < W)
                w = wz * wy * wx
                vals = dft[np.minimum(zz, D - 1), np.minimum(yy, H - 1), np.minimum(xx, W - 1)]
                out += np.where(ok, w * vals, 0)
    return out


def central_slice(dft: np.ndarray, rot_t: np.ndarray, n: int) -> np.ndarray:
    """(2N, N+1) complex slice with conjugation where x<0 (v606:1099-1113)."""
    iz, iy, ix, conj = slice_pixel_coordinates(rot_t, n)
    s = trilinear_border(dft, iz, iy, ix)
    return np.where(conj, np.conj(s), s)


def whiten(image: np.ndarray) -> np.ndarray:
    """Radial amplitude whitening, plane removal, normalisation (v606:938-992).

    The plane is fitted over (row, column) = (coord_x, coord_y): the reference
    swaps the names at its call site (v606:916-918).
    """
    img = np.asarray(image, dtype=f64)
    n = img.shape[0]
    c = n // 2
    yy, xx = np.meshgrid(np.arange(n, dtype=f64), np.arange(n, dtype=f64), indexing="ij")
    rad = np.round(np.sqrt((yy - c) ** 2 + (xx - c) ** 2)).astype(np.int64)
    F = np.fft.fftshift(sfft.fft2(img))
    nb = rad.max() + 1
    spec = np.bincount(rad.ravel(), weights=np.abs(F).ravel(), minlength=nb)
    cnt = np.bincount(rad.ravel(), minlength=nb).astype(f64)
    div = np.ones(nb)
    nz = cnt > 0
    div[nz] = cnt[nz] / spec[nz]
    div[0] = 1.0
    F = F * div[rad]
    img = sfft.ifft2(np.fft.ifftshift(F)).real
    x, y, z = yy.ravel(), xx.ravel(), img.ravel()
    A = np.array([[np.sum(x * x), np.sum(x * y), np.sum(x)],
                  [np.sum(x * y), np.sum(y * y), np.sum(y)],
                  [np.sum(x), np.sum(y), float(x.size)]])
    b = np.array([np.sum(x * z), np.sum(y * z), np.sum(z)])
    coeff = np.linalg.solve(A, b)
    img = img - (coeff[0] * yy + coeff[1] * xx + coeff[2])
    mean = img.mean()
    std = img.std()
    return (img - mean) / std if std > 1e-12 else img - mean


def template_from_slice(slice_c: np.ndarray, n: int, newbox: int, mask, packed_fsc) -> np.ndarray:
    """ifftshift rows, irfft2 to (2N)^2, ifftshift, crop N^2, whiten, mask,
    fft2, fftshift, Fourier crop, pack, FSC, L2 normalise, pre-shift
    (v606:1121-1147)."""
    pad = n // 2
    proj = np.fft.ifftshift(slice_c, axes=0)
    proj = sfft.irfftn(proj, s=(2 * n, 2 * n), axes=(0, 1))
    proj = np.fft.ifftshift(proj)[pad:pad + n, pad:pad + n]
    proj = whiten(proj)
    if mask is not None:
        proj = proj * np.asarray(mask, dtype=f64)
    F = np.fft.fftshift(sfft.fft2(proj))
    if newbox != n:
        lo = n // 2 - newbox // 2
        F = F[lo:lo + newbox, lo:lo + newbox]
    packed = centered_to_packed(F) * np.asarray(packed_fsc, dtype=f64)
    packed = packed / np.linalg.norm(packed.ravel())
    return pre_shift(packed)


def build_templates(volume, rot_t: np.ndarray, newbox: int, mask, packed_fsc,
                    dft: np.ndarray = None) -> np.ndarray:
    """All templates of one volume: [n_dir, newbox, newbox//2+1] complex128."""
    n = np.asarray(volume).shape[0]
    if dft is None:
        dft = volume_spectrum(volume)
    out = np.empty((len(rot_t), newbox, newbox // 2 + 1), dtype=np.complex128)
    for i, R in enumerate(rot_t):
        out[i] = template_from_slice(central_slice(dft, R, n), n, newbox, mask, packed_fsc)
    return out


# --------------------------------------------------------------------------
# a6: packed CTF with ISSPA weighting (float32, operation order of v606:778-829)
# --------------------------------------------------------------------------


class PackedCTF:
    """float32 CTF*ISSPA table in the packed layout (v606:695-777 set-up)."""

    def __init__(self, size, pixel_size, cs, voltage, kk, amp_const=0.1):
        self.size = int(size)
        self.kk = float(kk)
        local_cs = f32(cs) * f32(1e7)
        local_kv = f32(voltage) * f32(1e3)
        lam = f32(12.2643247) / np.sqrt(local_kv * (f32(1.0) + local_kv * f32(0.978466e-6)))
        self.k1 = f32(f32(np.pi) * lam)
        self.k2 = f32(f32(np.pi / 2.0) * local_cs * lam ** f32(3.0))
        self.k3 = f32(np.arctan(f32(amp_const) / np.sqrt(f32(1.0) - f32(amp_const) ** 2)))
        self.k5 = f32(0.0)
        n = self.size
        ps = f32(pixel_size)
        cf = (np.arange(n, dtype=f32) - f32(n) / f32(2.0)) / (f32(n) * ps)
        yf = np.concatenate((cf[n // 2:], cf[:n // 2]))
        xf = np.concatenate((cf[n // 2:], cf[:1]))
        x, y = np.meshgrid(xf, yf, indexing="xy")
        self.x = x.astype(f32)
        self.y = y.astype(f32)
        u2 = self.x * self.x + self.y * self.y
        self.u4 = (u2 * u2).astype(f32)
        ss = np.sqrt(u2).astype(f32)
        signal = np.exp(f32(-78.7757) * ss * ss + f32(-12.9121) * ss + f32(1.28732),
                        dtype=f32) / (f32(self.kk) + f32(1.0))
        self.ncurve = (np.exp(f32(-9.32) * ss * ss + f32(2.65) * ss + f32(0.01908),
                              dtype=f32) / signal).astype(f32)

    def one(self, dfu, dfv, dfa) -> np.ndarray:
        """CTF * ISSPA weight for one particle (v606:781-829)."""
        dfu, dfv = f32(dfu), f32(dfv)
        ang = f32(dfa) * f32(math.pi / 180.0)
        s, c = np.sin(ang, dtype=f32), np.cos(ang, dtype=f32)
        axx = (-dfu) * c * c - dfv * s * s
        ayy = (-dfu) * s * s - dfv * c * c
        axy = (-dfu) * s * c + dfv * s * c
        x, y = self.x, self.y
        t = (axx * x * x + f32(2.0) * axy * x * y) + ayy * y * y
        gamma = self.k1 * t + self.k2 * self.u4 - self.k5 - self.k3
        v = -np.sin(gamma.astype(f32), dtype=f32)
        v = np.where(np.abs(v) < f32(1e-8), np.sign(v) * f32(1e-8), v).astype(f32)
        return (v * np.sqrt(f32(1.0) / (self.ncurve + f32(self.kk) * v * v), dtype=f32)).astype(f32)


# --------------------------------------------------------------------------
# a7: psi sampling and particle spectra
# --------------------------------------------------------------------------


def psi_sampling(particle_psi, psi_step, do_local, local_range):
    """(searched psi, effective psi) lists (v606:1163-1190)."""
    num = int(360 // psi_step)
    if num < 1:
        num = 1
    tmp = 999999.0
    if do_local:
        tmp = local_range // psi_step
        local_count = int(tmp * 2 + 1)
        if local_count < num:
            num = local_count
    fake, eff = [], []
    nearest = round(((particle_psi + 360.0) % 360.0) / psi_step) * psi_step
    nearest %= 360.0
    for i in range(int(num)):
        a = psi_step * i
        if do_local:
            a = nearest - tmp * psi_step + i * psi_step
        fake.append(float(a))
        eff.append(float(0.5 if abs(a) < 0.5 else a))
    return fake, eff


def _fma32(a, b, c):
    """float32 fused multiply-add: one rounding of a*b + c (exact in float64)."""
    return (f64(a) * np.asarray(b, dtype=f64) + np.asarray(c, dtype=f32).astype(f64)).astype(f32)


def psi_grid_pixels(size: int, angle_deg: float):
    """Source pixel (row, col) of each output pixel, float32 (v606:1213-1247,
    then grid_sample's align_corners=True un-normalisation)."""
    yy, xx = np.meshgrid(np.arange(size, dtype=f32), np.arange(size, dtype=f32), indexing="ij")
    center = np.asarray((size, size), dtype=f32) / f32(2.0)
    th = np.deg2rad(float(np.round(angle_deg, 6)))
    c, s = f32(np.cos(th)), f32(np.sin(th))
    M = np.asarray([[c, -s], [s, c]], dtype=f32)
    off = (center - M @ center).astype(f32)
    # The reference's (1,S,2)@(B,2,2) matmul forms fl(M[i,0]*row) and then
    # fuses the second product: fma(M[i,1], col, fl(M[i,0]*row)).
    sy = _fma32(M[0, 1], xx, M[0, 0] * yy) + off[0]
    sx = _fma32(M[1, 1], xx, M[1, 0] * yy) + off[1]
    yn = f32(2.0) * sy / f32(size - 1) - f32(1.0)
    xn = f32(2.0) * sx / f32(size - 1) - f32(1.0)
    # torch's vectorised 2-D CPU grid_sample un-normalises as (g + 1) * ((size-1)/2).
    half = f32(size - 1) / f32(2.0)
    py = (yn + f32(1.0)) * half
    px = (xn + f32(1.0)) * half
    return py.astype(f32), px.astype(f32)


def bilinear_zeros(image: np.ndarray, py, px) -> np.ndarray:
    """grid_sample bilinear with zero padding on voxel coordinates, float64."""
    H, W = image.shape
    img = np.asarray(image, dtype=f64)
    py, px = np.asarray(py, dtype=f64), np.asarray(px, dtype=f64)
    y0, x0 = np.floor(py), np.floor(px)
    ty, tx = py - y0, px - x0
    y0, x0 = y0.astype(np.int64), x0.astype(np.int64)
    out = np.zeros(py.shape)
    for dy, wy in ((0, 1 - ty), (1, ty)):
        for dx, wx in ((0, 1 - tx), (1, tx)):
            yy, xx = y0 + dy, x0 + dx
            ok = (yy >= 0) & (yy < H) & (xx >= 0) & (xx < W)
            v = img[np.clip(yy, 0, H - 1), np.clip(xx, 0, W - 1)]
            out += np.where(ok, wy * wx * v, 0.0)
    return out


def prepare_particle(image, effective_psi, ctf, mask, newbox: int) -> np.ndarray:
    """[n_psi, newbox, newbox//2+1] pre-shifted, conjugated, normalised
    particle spectra (v606:1340-1374)."""
    img = np.asarray(image, dtype=f64)
    n = img.shape[0]
    out = []
    for a in effective_psi:
        py, px = psi_grid_pixels(n, a)
        rot = bilinear_zeros(img, py, px)
        if mask is not None:
            rot = rot * np.asarray(mask, dtype=f64)
        F = np.fft.fftshift(sfft.fft2(rot))
        if newbox != n:
            lo = n // 2 - newbox // 2
            F = F[lo:lo + newbox, lo:lo + newbox]
        p = np.conj(centered_to_packed(F) * np.asarray(ctf, dtype=f64))
        p = p / np.linalg.norm(p.ravel())
        out.append(pre_shift(p))
    return np.stack(out)


# --------------------------------------------------------------------------
# a8: correlation maximum over the translation window
# --------------------------------------------------------------------------


def crop_offsets(crop: int) -> np.ndarray:
    """Signed shift of each crop index: crop index i reads ccg[(i - crop/2) mod N]
    (v606:518-529, 539-541)."""
    return np.arange(crop) - crop // 2


def correlation_window(templates: np.ndarray, particle: np.ndarray, crop: int) -> np.ndarray:
    """raw[a, b, iy, ix] = N^2 * irfft2(T_a * P_b)[y, x] on the crop window.

    Closed form of irfft2 on the stored (pre-shifted) arrays, as pocketfft and
    torch evaluate it: a complex inverse along rows, then a C2R along columns
    that keeps only the real part of columns 0 and N/2:
        raw(y, x) = sum_{r,c} w_c Re[Q(r,c) e^{2 pi i (r y + c x)/N}],
        w_c = 1 for c in {0, N/2}, 2 otherwise (v606:1437-1442).
    """
    T = np.asarray(templates, dtype=np.complex128)
    P = np.asarray(particle, dtype=np.complex128)
    n, h = T.shape[-2], T.shape[-1]
    off = crop_offsets(crop)
    Ey = np.exp(2j * np.pi * np.outer(np.arange(n), off) / n)          # [r, iy]
    w = np.full(h, 2.0)
    w[0] = 1.0
    w[n // 2] = 1.0
    Ex = w[:, None] * np.exp(2j * np.pi * np.outer(np.arange(h), off) / n)  # [c, ix]
    Q = T[:, None] * P[None]                                            # [a, b, r, c]
    Z = np.einsum("ry,abrc->abyc", Ey, Q)
    return np.einsum("abyc,cx->abyx", Z, Ex).real


def correlate(templates, particle, crop: int):
    """(scores, y, x) as correlate_templates_and_particle returns them
    (v606:1418-1449): score = 1024 * max raw, first maximum in row-major
    crop order."""
    raw = correlation_window(templates, particle, crop)
    a, b = raw.shape[:2]
    flat = raw.reshape(a, b, -1)
    idx = np.argmax(flat, axis=-1)
    best = np.take_along_axis(flat, idx[..., None], -1)[..., 0]
    return best * 1024.0, idx // crop, idx % crop


# --------------------------------------------------------------------------
# a9 / a11: per-particle record and candidate score
# --------------------------------------------------------------------------


def result_record(line_index, p_rot, p_tilt, p_psi, fake_psi, m_rot, m_tilt,
                  model_indices, scores, ys, xs, crop, trans_scale,
                  cc_threshold=3.0, accuracy=11.0):
    """The three output records of one particle (v606:1452-1516)."""
    s = np.asarray(scores, dtype=f64)
    flat = s.reshape(-1)
    k = int(np.argmax(flat))
    n_psi = s.shape[1]
    li, pi = k // n_psi, k % n_psi
    peak = s[li, pi]
    py, px = int(ys[li, pi]), int(xs[li, pi])
    rem_x = float(crop // 2 - px) / trans_scale
    rem_y = float(crop // 2 - py) / trans_scale
    g = int(model_indices[li])
    ang = angular_distance(m_rot[g], m_tilt[g], 0.0, p_rot, p_tilt, 0.0)
    z = (peak - flat.mean()) / flat.std()
    return [
        ["cc: ", line_index, float(z), 1 if z > cc_threshold else 0,
         1 if ang < accuracy else 0, m_rot[g], m_tilt[g], ang,
         round(rem_x), round(rem_y), 0, 0],
        ["psi: ", line_index, float(fake_psi[pi]), float((p_psi + 360.0) % 360.0)],
        ["rawCC: ", line_index, float(peak)],
    ]


def candidate_score(raw_cc) -> float:
    """sum(exp(rawCC / 1024)) in float64 (ZL gisapr_batch_search.py:361)."""
    return float(np.sum(np.exp(np.asarray(raw_cc, dtype=f64) / 1024.0)))


# --------------------------------------------------------------------------
# PDB text (pdb_text.py:26-46 element inference, 78-120 reader)
# --------------------------------------------------------------------------

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


def read_pdb_text(text: str, include_hetatm=True, first_model_only=True):
    """(coords float32 [n,3], elements, chains) of the selected records."""
    lines = text.splitlines(keepends=True)
    first_model = next((i for i, l in enumerate(lines) if l[:6].strip() == "MODEL"), None)
    active = first_model is None
    coords, els, chains = [], [], []
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
        coords.append([float(line[s:s + 8]) for s in (30, 38, 46)])
        els.append(infer_element(line))
        chains.append(line[21:22] or " ")
    return (np.asarray(coords, dtype=f32).reshape(-1, 3), np.asarray(els, dtype="U2"),
            np.asarray(chains, dtype="U1"))


# --------------------------------------------------------------------------
# One candidate, end to end, in the order of run_search (v606:1594-1825)
# --------------------------------------------------------------------------


def moved_density_atoms(pdb_text: str, chain_id: str, pose, include_hetatm=False):
    """Coordinates and Z of every density atom with the chain moved and
    8.3-rounded (Z3 pdb_text.py:179-198): the pivot is the float32 mean of
    the chain's first-model atoms (HETATM included)."""
    fc, fe, fch = read_pdb_text(pdb_text, include_hetatm=True, first_model_only=True)
    dc, de, dch = read_pdb_text(pdb_text, include_hetatm=include_hetatm, first_model_only=False)
    sel = fch == chain_id
    moved = transform_coordinates(fc[sel], pose)
    q = quantize_8_3(moved)
    coords = dc.copy()
    # Files written by the synthetic generator hold one model in file order,
    # so the selected first-model rows are the density rows with this chain.
    dsel = np.where(dch == chain_id)[0]
    coords[dsel[:len(q)]] = q[:len(dsel)]
    return coords, atomic_numbers(de), dch


def evaluate_candidate(pdb_text, pose, box, apix, res, model_rot, model_tilt, images,
                       rec_line, rec_rot, rec_tilt, rec_psi, rec_dfu, rec_dfv, rec_dfa,
                       fsc_values, mask_radius, mask_edge, psi_step, local_range, crop,
                       kk=3.0, voltage=300.0, cs=2.7, newbox=None, chain_id="A",
                       keep_templates=True):
    """Score one candidate pose; returns every intermediate the tests check."""
    n = int(box)
    nb = int(newbox or box)
    coords, z, _ = moved_density_atoms(pdb_text, chain_id, pose)
    density = splat_density(coords, z, n, apix, res)
    rot_t = rotation_matrices_t(model_rot, model_tilt)
    mask = soft_mask(n, mask_radius, mask_edge)
    packed_fsc = centered_to_packed(radial_map(fsc_values, nb))
    local = local_orientations(rec_rot, rec_tilt, model_rot, model_tilt, local_range)
    needed = sorted({k for l in local for k in l})
    dft = volume_spectrum(density)
    templates = {}
    for k in needed:
        templates[k] = template_from_slice(central_slice(dft, rot_t[k], n), n, nb, mask, packed_fsc)
    del dft
    new_apix = n / nb * apix
    ctfgen = PackedCTF(nb, new_apix, cs, voltage, kk)
    per = []
    raw = []
    for i in range(len(rec_line)):
        fake, eff = psi_sampling(float(rec_psi[i]), psi_step, True, local_range)
        ctf = ctfgen.one(rec_dfu[i], rec_dfv[i], rec_dfa[i])
        spec = prepare_particle(images[i], eff, ctf, mask, nb)
        idx = local[i]
        if not idx:
            per.append(dict(spectra=spec, local=idx))
            continue
        T = np.stack([templates[k] for k in idx])
        s, y, x = correlate(T, spec, crop)
        recs = result_record(int(rec_line[i]), float(rec_rot[i]), float(rec_tilt[i]),
                             float(rec_psi[i]), fake, model_rot, model_tilt, idx, s, y, x,
                             crop, apix / new_apix)
        raw.append(recs[2][2])
        per.append(dict(spectra=spec, local=idx, scores=s, ys=y, xs=x, records=recs,
                        ctf=ctf, fake=fake, eff=eff))
    return dict(density=density, templates=templates if keep_templates else None,
                particles=per, score=candidate_score(raw), raw=np.asarray(raw), local=local)
