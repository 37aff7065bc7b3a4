"""Geometric restraint of a moved chain (func_check_boundary_for_testing_v8.py).

``GeometryRestraint(pdb_path, chain_id, device, boxsize=256, apix=1.5,
threshold=1.0, include_hetatm=False).evaluate(pose, pivot=None)`` returns
(overlapping voxel count, minimum chain to main-body separation in
Angstrom), as the reference's class of the same name does (v8:62-126): the
main body (every atom not in the chain) is splatted once at ``apix`` with
resolution 2*apix, thresholded into a mask, and its exact distance
transform is kept on the device as integer squared voxel distances. A pose
moves the chain with the reference's float32 row-vector rotation about its
mean (v8:33-45, on the host, as the reference computes it), the moved chain
is splatted onto an all-zero scratch volume, and one reduction over the
chain's bounding box counts overlap voxels and takes the minimum squared
distance (the scratch is zeroed as it is read). ``evaluate_many`` scores a
list of poses with one upload of every pose's coordinates, one splat and
one reduction launch per pose, and one read-back of all results.

The kernels are in csrc/restraint.cu; the densities use the same splat as
the scoring path. There is no CPU path.
"""
from __future__ import annotations

import argparse
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat
from .pdb2mrc import atoms_to_atomic_numbers_and_masses, density_from_coords, density_parameters
from .pdb_text import read_pdb

__all__ = ["OUT_OF_BOUNDARY", "IN_BOUNDARY", "GeometryRestraint", "read_pdb_split_chain_and_rest",
           "rotate_coords_rotvec", "create_BOUNDARY_CHECK_parser", "convert_float_into_my_format", "main"]

OUT_OF_BOUNDARY = False
IN_BOUNDARY = True


def read_pdb_split_chain_and_rest(pdb_filename, target_chain_id, do_include_HETATM=False):
    """(chain coords, chain elements, rest coords, rest elements) over every
    model of the file (v8:24-30)."""
    pdb = read_pdb(pdb_filename, include_hetatm=do_include_HETATM, first_model_only=False)
    selected = pdb.chains == target_chain_id
    if not np.any(selected):
        raise ValueError(f"Cannot find chain {target_chain_id}")
    return pdb.coords[selected], pdb.elements[selected], pdb.coords[~selected], pdb.elements[~selected]


def rotate_coords_rotvec(coordinates, rot, tilt, psi, xshift, yshift, zshift, pivot=None):
    """(c - centre) @ R + centre + shift in float32, R = the rotation vector
    (rot, tilt, psi) in degrees as a float32 matrix, centre = the float32
    mean of the coordinates unless ``pivot`` is given (v8:33-45)."""
    from scipy.spatial.transform import Rotation
    coordinates = np.asarray(coordinates)
    if coordinates.shape[0] == 0:
        return coordinates.copy()
    center = np.mean(coordinates, axis=0) if pivot is None else np.asarray(pivot, dtype=np.float32)
    if center.shape != (3,) or not np.isfinite(center).all():
        raise ValueError("pivot must contain three finite coordinates in Angstrom")
    omega = np.asarray([rot, tilt, psi], dtype=np.float32)
    matrix = Rotation.from_rotvec(np.deg2rad(omega)).as_matrix().astype(np.float32, copy=False)
    shift = np.asarray([xshift, yshift, zshift], dtype=np.float32)
    return ((coordinates - center) @ matrix + center + shift).astype(np.float32, copy=False)


class GeometryRestraint:
    """Main-body mask and distance transform of one chain split, on the device."""

    def __init__(self, pdb_path, chain_id, device="cuda", boxsize=256, apix=1.5, threshold=1.0,
                 include_hetatm=False):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("GeometryRestraint needs a CUDA device")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.boxsize = int(boxsize)
        self.apix = float(apix)
        self.threshold = float(threshold)
        self.res = 2.0 * self.apix
        self.width, self.rp, self.kn = density_parameters(self.apix, self.res)
        self.chain_coords, chain_atoms, rest_coords, rest_atoms = read_pdb_split_chain_and_rest(
            pdb_path, chain_id, do_include_HETATM=include_hetatm)
        numbers, _ = atoms_to_atomic_numbers_and_masses(chain_atoms)
        self.chain_numbers = torch.as_tensor(np.asarray(numbers, np.float32), device=self.device)
        rest_numbers, _ = atoms_to_atomic_numbers_and_masses(rest_atoms)
        rest = density_from_coords(rest_coords, rest_numbers, self.boxsize, self.apix, self.res,
                                   device=self.device)
        n = self.boxsize
        self.mainbody_mask = torch.empty((n, n, n), dtype=torch.uint8, device=self.device)
        self.mainbody_d2 = torch.empty((n, n, n), dtype=torch.int32, device=self.device)
        scratch = torch.empty((n, n, n), dtype=torch.int32, device=self.device)
        ctx = nat.Context.for_device(self.device).handle
        nat.call("gisapr_restraint_edt", ctx, nat.stream_of(self.device), nat.ptr(rest), n, self.threshold,
                 nat.ptr(self.mainbody_mask), nat.ptr(self.mainbody_d2), nat.ptr(scratch))
        del rest, scratch
        self.has_mainbody = bool(torch.count_nonzero(self.mainbody_mask).item())
        self._volume = torch.zeros((n, n, n), dtype=torch.float32, device=self.device)
        self._empty_chain_distance: Optional[float] = None

    # -------------------------------------------------------------------
    @property
    def mainbody_distance(self) -> torch.Tensor:
        """Distance transform in voxels (float64), as the reference keeps it."""
        return torch.sqrt(self.mainbody_d2.to(torch.float64))

    def _bounds(self, xyz: np.ndarray) -> np.ndarray:
        """Half-open (z, y, x) voxel box that holds every voxel the splat of
        ``xyz`` can touch."""
        n, w = self.boxsize, self.width
        if len(xyz) == 0:
            return np.zeros(6, dtype=np.int32)
        pos = (xyz.astype(np.float64) / self.apix + n // 2).astype(np.float32)
        lo = np.floor(pos.min(axis=0).astype(np.float64) - w) - 1
        hi = np.ceil(pos.max(axis=0).astype(np.float64) + w) + 2
        lo = np.clip(lo, 0, n).astype(np.int64)[::-1]
        hi = np.clip(hi, 0, n).astype(np.int64)[::-1]
        hi = np.maximum(hi, lo)
        return np.ascontiguousarray(np.concatenate([lo, hi]), dtype=np.int32)

    def _empty_distance(self) -> float:
        # No chain voxel above the threshold: the reference's distance
        # transform then measures to the implicit point (-1, 0, 0) (v8:119-126).
        if self._empty_chain_distance is None:
            zz, yy, xx = np.nonzero(self.mainbody_mask.cpu().numpy())
            squared = (zz.astype(np.int64) + 1) ** 2 + yy.astype(np.int64) ** 2 + xx.astype(np.int64) ** 2
            self._empty_chain_distance = float(np.sqrt(np.min(squared))) * self.apix
        return self._empty_chain_distance

    def evaluate(self, pose, pivot=None) -> Tuple[int, float]:
        """(overlapping voxel count, minimum separation in Angstrom); pose =
        [rot, tilt, psi, xshift, yshift, zshift]."""
        return self.evaluate_many([pose], pivot)[0]

    def evaluate_many(self, poses: Sequence, pivot=None) -> List[Tuple[int, float]]:
        poses = np.asarray(poses, dtype=np.float64)
        if poses.ndim != 2 or poses.shape[1] != 6 or not np.isfinite(poses).all():
            raise ValueError("pose must contain six finite rotation/translation values")
        if not self.has_mainbody:
            return [(0, 0.0)] * len(poses)
        k, n_atoms = len(poses), len(self.chain_coords)
        moved = np.stack([rotate_coords_rotvec(self.chain_coords, *p, pivot=pivot) for p in poses]) \
            if n_atoms else np.zeros((k, 0, 3), np.float32)
        bounds = [self._bounds(m) for m in moved]
        dev = self.device
        xyz_host = torch.from_numpy(np.ascontiguousarray(moved, dtype=np.float32)).pin_memory()
        xyz = xyz_host.to(dev, non_blocking=True)
        out = torch.empty((k, 3), dtype=torch.int32, device=dev)
        ctx = nat.Context.for_device(dev).handle
        st = nat.stream_of(dev)
        n = self.boxsize
        nat.call("gisapr_restraint_init", st, nat.ptr(out), k)
        try:
            for c in range(k):
                if n_atoms:
                    nat.call("gisapr_deposit", ctx, st, nat.c_ptr_offset(xyz, c * n_atoms * 12),
                             nat.ptr(self.chain_numbers), n_atoms, nat.ptr(self._volume), n, self.width,
                             self.apix, self.rp, self.kn)
                nat.call("gisapr_restraint_eval", ctx, st, nat.ptr(self._volume), nat.ptr(self.mainbody_mask),
                         nat.ptr(self.mainbody_d2), n, bounds[c].ctypes.data, self.threshold,
                         nat.c_ptr_offset(out, c * 12))
            res = out.cpu().numpy()
        except BaseException:
            self._volume.zero_()
            raise
        results = []
        for count, d2, any_voxel in res:
            if count:
                results.append((int(count), 0.0))
            elif any_voxel:
                results.append((0, float(np.sqrt(np.float64(d2))) * self.apix))
            else:
                results.append((0, self._empty_distance()))
        return results


def create_BOUNDARY_CHECK_parser():
    """Arguments of the restraint command (v8:129-151)."""
    p = argparse.ArgumentParser(description="Check whether a subunit hits a physical boundary.")
    p.add_argument("--i", required=True)
    p.add_argument("--chainID", required=True)
    p.add_argument("--rot", type=float, required=True)
    p.add_argument("--tilt", type=float, required=True)
    p.add_argument("--psi", type=float, required=True)
    p.add_argument("--centerX", type=float, default=0.)
    p.add_argument("--centerY", type=float, default=0.)
    p.add_argument("--centerZ", type=float, default=0.)
    p.add_argument("--pivot", type=float, nargs=3, metavar=("X", "Y", "Z"))
    p.add_argument("--maskBoxsize", type=int, default=256)
    p.add_argument("--apix", type=float, default=1.5)
    p.add_argument("--outputRoot", required=True)
    p.add_argument("--thresholdForMask", type=float, default=1.)
    p.add_argument("--thresholdChainIsTooFar", type=float, default=50.)
    p.add_argument("--thresholdPixelHits", type=int, default=5)
    p.add_argument("--outputFile", required=True)
    p.add_argument("--noUse", action="store_true", help="Legacy placeholder")
    p.add_argument("--gpuid", type=int, default=0)
    p.add_argument("--device", help="CUDA device, e.g. cuda:0; overrides --gpuid")
    p.add_argument("--skip-geometric-restraint", action="store_true")
    return p


def convert_float_into_my_format(number) -> str:
    """12.34 -> '12p3', -0.5 -> 'N0p5' (v8:154-158)."""
    integer_part = int(np.fabs(number))
    decimal_part = abs(number - integer_part)
    dp = f"{decimal_part:.1f}".split(".")[1]
    return ("N" if number < 0 else "") + str(integer_part) + "p" + dp


def main(argv=None) -> None:
    args = create_BOUNDARY_CHECK_parser().parse_args(argv)
    pose = [args.rot, args.tilt, args.psi, args.centerX, args.centerY, args.centerZ]
    if args.skip_geometric_restraint:
        overlap, min_distance = 0, 0.0
    else:
        restraint = GeometryRestraint(args.i, args.chainID, device=args.device or f"cuda:{args.gpuid}",
                                      boxsize=args.maskBoxsize, apix=args.apix, threshold=args.thresholdForMask)
        overlap, min_distance = restraint.evaluate(pose, pivot=args.pivot)
    print("Minimum distance between the rotated chains and mainbody is (in Angstrom):", min_distance)
    values = [args.chainID] + [convert_float_into_my_format(x) for x in pose] + [str(overlap), str(min_distance)]
    with open(args.outputFile, "w") as handle:
        handle.write("\t".join(values) + "\n")


if __name__ == "__main__":
    main()
