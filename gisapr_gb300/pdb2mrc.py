"""Gaussian density of PDB atoms on the GPU (pdb2mrc_gpu_ver_fp32_v3.py and
the Lite tree's pdb2mrc_gpu_ver_fp32_v4.py, same entry points and
conventions). Every density is produced by the splat kernels of
libgisapr_gb300.so; the output is float32 [z, y, x] on the given CUDA device.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .pdb_text import read_pdb, rotation_matrices, rotation_matrix, split_moving_chain

element_data = {
    "H": (1.0, 1.00794), "C": (6.0, 12.0107), "N": (7.0, 14.00674),
    "O": (8.0, 15.9994), "P": (15.0, 30.973761), "S": (16.0, 32.066),
}


def atoms_to_atomic_numbers_and_masses(atoms):
    values = np.asarray([element_data.get(str(a).upper(), (0.0, 0.0)) for a in atoms],
                        dtype=np.float64).reshape(-1, 2)
    return values[:, 0], values[:, 1]


def density_parameters(apix: float, res: float):
    """(width, rp, kn) of pdb2mrc_gpu_ver_fp32_v3.py:53-58, with its checks."""
    apix, res = float(apix), float(res)
    if not np.isfinite(apix) or not np.isfinite(res) or apix <= 0 or res <= 0:
        raise ValueError("boxsize, apix and resolution must be positive and finite")
    width = int(round(res * 3.0 / apix))
    if width < 3:
        raise ValueError("You do not have sufficient sampling for this resolution. Decrease apix.")
    rp = float(np.power(np.pi / (res / apix), 2))
    kn = float(np.power(rp / np.pi, 1.5))
    return width, rp, kn


def _dev(device) -> torch.device:
    d = torch.device(device)
    if d.type != "cuda":
        raise ValueError(f"GisAPR GB300 density kernels need a CUDA device, got {d}")
    return d if d.index is not None else torch.device("cuda", torch.cuda.current_device())


def density_from_coords(coordinates, atomic_numbers, boxsize, apix, res, device="cuda",
                        max_chunk_voxels=524288, _initial_volume=None, backend="cuda",
                        backend_metrics=None):
    """Return a float32 [z, y, x] density (pdb2mrc v3:41-98, v4:41-118).

    Atoms add per voxel in input order onto ``_initial_volume`` (never
    modified; a fresh tensor is returned) or onto zeros. ``max_chunk_voxels``
    and ``backend`` are accepted for signature compatibility: there is one
    kernel, and it has no chunking.
    """
    if backend not in ("auto", "torch", "cuda"):
        raise ValueError("density backend must be auto, torch or cuda")
    boxsize = int(boxsize)
    if boxsize < 1:
        raise ValueError("boxsize, apix and resolution must be positive and finite")
    width, rp, kn = density_parameters(apix, res)
    dev = _dev(device)
    xyz = torch.as_tensor(np.asarray(coordinates, dtype=np.float32) if not torch.is_tensor(coordinates)
                          else coordinates, dtype=torch.float32, device=dev).reshape(-1, 3).contiguous()
    z = torch.as_tensor(np.asarray(atomic_numbers, dtype=np.float32) if not torch.is_tensor(atomic_numbers)
                        else atomic_numbers, dtype=torch.float32, device=dev).reshape(-1).contiguous()
    if len(xyz) != len(z):
        raise ValueError("Coordinate and atom count differ")
    if _initial_volume is None:
        volume = torch.zeros((boxsize,) * 3, dtype=torch.float32, device=dev)
    else:
        if (tuple(_initial_volume.shape) != (boxsize,) * 3 or _initial_volume.dtype != torch.float32
                or _initial_volume.device != dev):
            raise ValueError("Initial density must match the box, float32 dtype and device")
        volume = _initial_volume.clone(memory_format=torch.contiguous_format)
    if len(xyz) == 0:
        return volume
    if not bool(torch.isfinite(xyz).all()):
        raise ValueError("PDB coordinates must be finite")
    nat.call("gisapr_deposit", nat.Context.for_device(dev).handle, nat.stream_of(dev), nat.ptr(xyz),
             nat.ptr(z), len(xyz), nat.ptr(volume), boxsize, width, float(apix), rp, kn)
    if backend_metrics is not None:
        backend_metrics["density_fused_calls"] = backend_metrics.get("density_fused_calls", 0) + 1
    return volume


def yflip_vectorized(arr):
    """EMAN y-flip, even boxes keep row zero (pdb2mrc v3:101-112)."""
    ny = arr.shape[1]
    idx = np.arange(ny)
    j1 = np.arange(ny // 2, ny)
    j2 = ny - j1 + (-1 if ny % 2 else 0)
    ok = j1 > j2
    idx[j1[ok]], idx[j2[ok]] = j2[ok], j1[ok]
    if isinstance(arr, np.ndarray):
        return arr[:, idx, :].copy()
    return arr.index_select(1, torch.as_tensor(idx, device=arr.device))


class MovedChainDensity:
    """Fixed-context density computed once, moving chain splatted per pose:
    RigidDensityCache (Lite gisapr_batch_density.py:57-117) with the pose
    transform and PDB 8.3 round trip of transformed_density_atoms on the GPU.
    """

    def __init__(self, pdb_path_or_text, chain_id, boxsize, apix, res, device="cuda",
                 include_hetatm=False, from_text=False):
        from .pdb_text import read_pdb_text
        self.device = _dev(device)
        self.box = int(boxsize)
        self.apix = float(apix)
        self.width, self.rp, self.kn = density_parameters(apix, res)
        if from_text:
            first = read_pdb_text(pdb_path_or_text)
            dens = read_pdb_text(pdb_path_or_text, include_hetatm=include_hetatm, first_model_only=False)
        else:
            first = read_pdb(pdb_path_or_text)
            dens = read_pdb(pdb_path_or_text, include_hetatm=include_hetatm, first_model_only=False)
        split = split_moving_chain(first, chain_id, include_hetatm, dens)
        zm, _ = atoms_to_atomic_numbers_and_masses(split.moving_elements)
        zf, _ = atoms_to_atomic_numbers_and_masses(split.fixed_elements)
        f = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=self.device)
        self.moving_xyz = f(split.moving_coords).reshape(-1, 3)
        self.moving_z = f(zm)
        self.pivot = f(split.pivot)
        self.n_moving = int(len(zm))
        self.fixed = density_from_coords(split.fixed_coords, zf, self.box, apix, res, device=self.device)
        self.fixed_atom_count = int(len(zf))
        self._pose = torch.zeros(12, dtype=torch.float64, device=self.device)

    def pose_tensor(self, pose) -> torch.Tensor:
        """[rot (9, row-major), shift (3)] float64 on the host."""
        m = rotation_matrix(pose)
        return torch.from_numpy(np.concatenate([m.reshape(-1), np.asarray(pose, dtype=np.float64)[3:]]))

    @staticmethod
    def pose_tensors(poses) -> torch.Tensor:
        """pose_tensor of every pose, [k, 12] float64 on the host, from one
        vectorized rotation call (a batch of 64 poses takes about 0.05 ms
        instead of 1.8 ms pose by pose)."""
        p = np.asarray(poses, dtype=np.float64).reshape(-1, 6)
        m = rotation_matrices(p)
        return torch.from_numpy(np.concatenate([m.reshape(-1, 9), p[:, 3:]], axis=1))

    def generate(self, pose, out=None, write_padded=False, pose_device=None) -> torch.Tensor:
        """Density of the moved chain on the fixed context (``out`` may be a
        preallocated [box]^3 tensor; ``write_padded`` also fills the FFT input)."""
        if pose_device is None:
            self._pose.copy_(self.pose_tensor(pose), non_blocking=True)
            pose_device = self._pose
        if out is None and not write_padded:
            out = torch.empty((self.box,) * 3, dtype=torch.float32, device=self.device)
        nat.call("gisapr_deposit_moved", nat.Context.for_device(self.device).handle,
                 nat.stream_of(self.device), nat.ptr(self.moving_xyz), nat.ptr(self.moving_z),
                 self.n_moving, nat.ptr(self.pivot), nat.ptr(pose_device),
                 nat.c_ptr_offset(pose_device, 9 * 8), nat.ptr(self.fixed), nat.ptr(out),
                 1 if write_padded else 0, self.box, self.width, self.apix, self.rp, self.kn)
        return out


def generate_volume(pdb_path, boxsize, apix, res, device="cuda", do_center=False, do_yflip=False,
                    include_hetatm=False, source_pdb=None, chain_id=None, pose=None,
                    density_backend="cuda", backend_metrics=None):
    """Density of a PDB file, or of ``source_pdb`` with chain ``chain_id``
    moved by ``pose`` (Z3 pdb2mrc v3:115-133, Lite v4:135-155)."""
    if source_pdb is None:
        pdb = read_pdb(pdb_path, include_hetatm=include_hetatm, first_model_only=False)
        z, masses = atoms_to_atomic_numbers_and_masses(pdb.elements)
        coords = pdb.coords
        if do_center and len(coords):
            if masses.sum() <= 0:
                raise ValueError("Cannot center PDB: no supported atoms with nonzero mass")
            coords = coords - np.sum(coords * masses[:, None], axis=0) / masses.sum()
        vol = density_from_coords(coords, z, boxsize, apix, res, device=device,
                                  backend=density_backend, backend_metrics=backend_metrics)
    else:
        if do_center:
            raise ValueError("do_center with a moved chain is not supported")
        vol = MovedChainDensity(source_pdb, chain_id, boxsize, apix, res, device, include_hetatm).generate(pose)
    if do_yflip:
        vol = yflip_vectorized(vol)
    return vol
