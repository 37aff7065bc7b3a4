"""Drop-in search API of GisAPR's v606 engine, backed by the sm_103a kernels.

Names, arguments and return conventions follow
test1_with_isspa_weight_varingKK_search_translation_also_v606_torch_optimized_
standalone.py ("v606"): PackedFourierLayout (v606:494-541), PackedCTFTorch
(v606:695-829), PsiGridBank (v606:1193-1256), ParticleFourierPreparer
(v606:1321-1374), IntegratedProjector (v606:1034-1155),
CorrelationWorkspace / correlate_templates_and_particle (v606:1382-1449) and
make_result_records (v606:1452-1516). Tensors live on a CUDA device; every
numeric step runs in libgisapr_gb300.so and there is no CPU path (a CPU
device raises ValueError).
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat
from .mrc import read_mrc_volume
from .tables import (ModelAngles, ParticleRecord, calculate_angular_distance, ctf_static_terms,
                     psi_rotation_entry)


def _cuda_device(device) -> torch.device:
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError(f"GisAPR GB300 kernels need a CUDA device, got {dev}")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


class PackedFourierLayout:
    """Index tensors of the packed half-plane layout (v606:494-541)."""

    def __init__(self, size: int, crop_size: int, device):
        if size <= 0 or size % 2 != 0:
            raise ValueError("newboxsize must be a positive even integer")
        if crop_size <= 0 or crop_size % 2 != 0 or crop_size > size:
            raise ValueError("CCG crop size must be positive, even and <= newboxsize")
        self.size = int(size)
        self.rfft_size = self.size // 2 + 1
        self.crop_size = int(crop_size)
        half = self.size // 2
        dev = torch.device(device)
        self.centered_row_to_packed = torch.cat((torch.arange(half, self.size, device=dev),
                                                 torch.arange(0, half, device=dev)))
        self.centered_col_to_packed = torch.cat((torch.arange(half, self.size, device=dev),
                                                 torch.zeros(1, dtype=torch.long, device=dev)))
        ch = self.crop_size // 2
        self.unshifted_ccg_crop_indices = torch.cat((torch.arange(self.size - ch, self.size, device=dev),
                                                     torch.arange(0, ch, device=dev)))

    def centered_full_to_packed(self, centered: torch.Tensor) -> torch.Tensor:
        packed = centered.index_select(-2, self.centered_row_to_packed.to(centered.device))
        return packed.index_select(-1, self.centered_col_to_packed.to(centered.device))


class PackedCTFTorch:
    """CTF * ISSPA weights in the packed layout (v606:695-829)."""

    def __init__(self, size, pixel_size, cs, voltage, kk, device, amp_const=0.1, bfactor=0.0,
                 scale=1.0, phase_shift=0.0):
        if float(bfactor) != 0.0 or float(scale) != 1.0:
            raise ValueError("bfactor and scale other than 0 and 1 are not implemented by the GB300 CTF kernel")
        self.size = int(size)
        self.device = _cuda_device(device)
        st = ctf_static_terms(size, pixel_size, cs, voltage, kk, amp_const, phase_shift)
        self.static = st
        self.kk = float(kk)
        self.k1, self.k2, self.k3, self.k5 = st.k1, st.k2, st.k3, st.k5
        to = lambda a: torch.from_numpy(np.ascontiguousarray(a.reshape(-1))).to(self.device)
        self.x, self.y, self.u4, self.ncurve = to(st.x), to(st.y), to(st.u4), to(st.ncurve)

    def batch_arrays(self, dfu, dfv, dfa, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        n = len(dfu)
        K = self.size * (self.size // 2 + 1)
        if out is None:
            out = torch.empty((n, self.size, self.size // 2 + 1), dtype=torch.float32, device=self.device)
        f = lambda v: torch.as_tensor(np.asarray(v, dtype=np.float32), device=self.device).contiguous()
        u, v, a = f(dfu), f(dfv), f(dfa)
        for s in range(0, n, 65535):
            e = min(n, s + 65535)
            nat.call("gisapr_packed_ctf", nat.stream_of(self.device), nat.ptr(u[s:]), nat.ptr(v[s:]),
                     nat.ptr(a[s:]), e - s, nat.ptr(self.x), nat.ptr(self.y), nat.ptr(self.u4),
                     nat.ptr(self.ncurve), K, self.k1, self.k2, self.k3, self.k5, self.kk,
                     nat.ptr(out[s:]))
        return out

    def batch(self, records: Sequence[ParticleRecord], has_ctf: bool) -> torch.Tensor:
        if not has_ctf:
            return torch.ones((len(records), self.size, self.size // 2 + 1), dtype=torch.float32,
                              device=self.device)
        return self.batch_arrays([r.defocus_u for r in records], [r.defocus_v for r in records],
                                 [r.defocus_angle for r in records])


class PsiGridBank:
    """In-plane rotations as (cos, sin, offset) rows (v606:1193-1256). The
    kernel forms each source coordinate on the fly instead of reading a
    stored sampling grid."""

    def __init__(self, size: int, device, unique_angles: Sequence[float], build_batch_size: int = 8):
        self.size = int(size)
        self.device = _cuda_device(device)
        self.angle_keys = [float(np.round(a, 6)) for a in unique_angles]
        self.angle_to_index = {a: i for i, a in enumerate(self.angle_keys)}
        rows = [psi_rotation_entry(self.size, a) for a in self.angle_keys]
        tab = np.stack(rows) if rows else np.zeros((1, 4), np.float32)
        self.table = torch.from_numpy(tab).to(self.device)

    def indices_for_angles(self, effective_angles: Sequence[float]) -> torch.Tensor:
        idx = []
        for a in effective_angles:
            key = float(np.round(a, 6))
            try:
                idx.append(self.angle_to_index[key])
            except KeyError as exc:
                raise KeyError(f"Psi grid angle {key} was not precomputed") from exc
        return torch.tensor(idx, dtype=torch.int32, device=self.device)


class ParticleFourierPreparer:
    """Rotated, masked, CTF-weighted, conjugated, normalised particle spectra
    (v606:1321-1374)."""

    def __init__(self, original_box, new_box, device, layout, real_space_mask, psi_grid_bank):
        self.original_box = int(original_box)
        self.new_box = int(new_box)
        self.device = _cuda_device(device)
        self.layout = layout
        self.real_space_mask = None if real_space_mask is None else \
            real_space_mask.to(self.device, torch.float32).contiguous()
        self.psi_grid_bank = psi_grid_bank

    def prepare_batch(self, images: torch.Tensor, psi_index: torch.Tensor, packed_ctf: torch.Tensor,
                      out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """images [n, box, box] float32, psi_index [n, n_psi] int32 rows of the
        bank, packed_ctf [n, newbox, newbox//2+1] -> [n, n_psi, newbox, H]."""
        n, n_psi = psi_index.shape
        nb, H = self.new_box, self.new_box // 2 + 1
        images = images.to(self.device, torch.float32).contiguous()
        psi_index = psi_index.to(self.device, torch.int32).contiguous()
        packed_ctf = packed_ctf.to(self.device, torch.float32).contiguous()
        if out is None:
            out = torch.empty((n, n_psi, nb, H), dtype=torch.complex64, device=self.device)
        nat.call("gisapr_prepare_particles", nat.Context.for_device(self.device).handle,
                 nat.stream_of(self.device), nat.ptr(images), n, n_psi, nat.ptr(psi_index),
                 nat.ptr(self.psi_grid_bank.table), nat.ptr(self.real_space_mask), nat.ptr(packed_ctf),
                 self.original_box, nb, nat.ptr(out))
        return out

    def prepare(self, image: torch.Tensor, effective_angles: Sequence[float],
                packed_ctf: torch.Tensor) -> torch.Tensor:
        idx = self.psi_grid_bank.indices_for_angles(effective_angles).view(1, -1)
        img = image.reshape(1, self.original_box, self.original_box)
        return self.prepare_batch(img, idx, packed_ctf.reshape(1, self.new_box, -1))[0]


class IntegratedProjector:
    """Fourier central-slice projector with whitening (v606:1034-1155)."""

    def __init__(self, device, original_box, new_box, layout, real_space_mask, packed_fsc,
                 projection_batch_size=8):
        self.device = _cuda_device(device)
        self.original_box = int(original_box)
        self.new_box = int(new_box)
        self.layout = layout
        self.real_space_mask = None if real_space_mask is None else \
            real_space_mask.to(self.device, torch.float32).contiguous()
        self.packed_fsc = packed_fsc.to(self.device, torch.float32).contiguous()
        self.batch_size = max(1, int(projection_batch_size))
        self._rot_cache = None
        # cuFFT spectrum (boxes 96, 192) per native context: the template
        # lanes of a batch run the transform and the projector of different
        # candidates at the same time on their own contexts and streams, so
        # each context writes and samples its own buffer
        self._spectra = {}
        # power-of-two boxes transform the density straight into the blocked
        # copy the slice gather reads (gisapr_volume_spectrum_blocked);
        # False keeps the cuFFT spectrum + blocked copy of volume_spectrum
        n = self.original_box
        self.blocked_fft = n & (n - 1) == 0 and 32 <= n <= 256
        self._from_blocked = False

    def _rot(self, angles: ModelAngles) -> torch.Tensor:
        key = id(angles.rotation_matrices_t)
        if self._rot_cache is None or self._rot_cache[0] != key:
            t = torch.from_numpy(np.ascontiguousarray(angles.rotation_matrices_t, dtype=np.float32))
            self._rot_cache = (key, t.reshape(-1, 9).to(self.device))
        return self._rot_cache[1]

    @property
    def spectrum(self) -> Optional[torch.Tensor]:
        """The last cuFFT spectrum written on this thread's current context."""
        return self._spectra.get(nat.Context.for_device(self.device).handle.value)

    def volume_spectrum(self, volume: Optional[torch.Tensor]) -> torch.Tensor:
        n = self.original_box
        ctx = nat.Context.for_device(self.device).handle
        spec = self._spectra.get(ctx.value)
        if spec is None:
            spec = torch.empty((2 * n, 2 * n, n + 1), dtype=torch.complex64, device=self.device)
            self._spectra[ctx.value] = spec
        nat.call("gisapr_volume_spectrum", ctx, nat.stream_of(self.device), nat.ptr(volume), n, nat.ptr(spec))
        self._from_blocked = False
        return spec

    def volume_spectrum_blocked(self, volume: torch.Tensor) -> None:
        """The density's half-volume spectrum, straight into the context's
        blocked copy (power-of-two boxes); the next project() reads it."""
        nat.call("gisapr_volume_spectrum_blocked", nat.Context.for_device(self.device).handle,
                 nat.stream_of(self.device), nat.ptr(volume), self.original_box)
        self._from_blocked = True

    def prepare(self, volume: torch.Tensor) -> None:
        """The spectrum the projector samples, by the transform of this box."""
        if self.blocked_fft:
            self.volume_spectrum_blocked(volume)
        else:
            self.volume_spectrum(volume)

    def project(self, angles: ModelAngles, dirs: torch.Tensor, out: torch.Tensor,
                out_slot: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Templates of ``dirs`` from the last volume_spectrum (or
        volume_spectrum_blocked) into ``out``."""
        nat.call("gisapr_project_templates", nat.Context.for_device(self.device).handle,
                 nat.stream_of(self.device), nat.ptr(None if self._from_blocked else self.spectrum),
                 self.original_box,
                 nat.ptr(self._rot(angles)), nat.ptr(dirs), int(dirs.numel()), nat.ptr(out_slot),
                 nat.ptr(self.real_space_mask), nat.ptr(self.packed_fsc), self.new_box, nat.ptr(out))
        return out

    def build_templates(self, mrc_volume, angles: ModelAngles, orientation_indices=None) -> torch.Tensor:
        if isinstance(mrc_volume, torch.Tensor):
            volume = mrc_volume
            if volume.dtype != torch.float32 or volume.device != self.device:
                raise ValueError("Model tensor must be float32 on the projector device")
        else:
            volume = torch.from_numpy(read_mrc_volume(mrc_volume)).to(self.device)
        if volume.ndim != 3 or len(set(volume.shape)) != 1:
            raise ValueError(f"Model volume must be cubic; got shape {tuple(volume.shape)}")
        if volume.shape[0] != self.original_box:
            raise ValueError(f"Model volume box {volume.shape[0]} does not match --oriboxsize "
                             f"{self.original_box}")
        selected = (list(range(len(angles.rot))) if orientation_indices is None
                    else sorted(set(map(int, orientation_indices))))
        if any(i < 0 or i >= len(angles.rot) for i in selected):
            raise ValueError("Projection orientation index is outside the angle table")
        out = torch.empty((len(selected), self.new_box, self.layout.rfft_size), dtype=torch.complex64,
                          device=self.device)
        if not selected:
            return out
        self.prepare(volume.contiguous())
        dirs = torch.tensor(selected, dtype=torch.int32, device=self.device)
        slots = torch.arange(len(selected), dtype=torch.int32, device=self.device)
        return self.project(angles, dirs, out, slots)


class CorrelationWorkspace:
    """Reusable output buffers of correlate_templates_and_particle (v606:1382-1415)."""

    def __init__(self, device):
        self.device = _cuda_device(device)
        self.capacity = 0
        self.scores = self.ys = self.xs = None
        self.ptr = torch.zeros(2, dtype=torch.int32, device=self.device)
        self.idx = None

    def ensure(self, n_a: int, n_b: int):
        if n_a * n_b > self.capacity or self.scores is None:
            self.capacity = max(n_a * n_b, self.capacity)
            self.scores = torch.empty(self.capacity, dtype=torch.float32, device=self.device)
            self.ys = torch.empty(self.capacity, dtype=torch.int32, device=self.device)
            self.xs = torch.empty(self.capacity, dtype=torch.int32, device=self.device)
        if self.idx is None or self.idx.numel() < n_a:
            self.idx = torch.arange(max(n_a, 16), dtype=torch.int32, device=self.device)
        return self.scores[:n_a * n_b], self.ys[:n_a * n_b], self.xs[:n_a * n_b]


def correlate_templates_and_particle(templates_pre_shifted: torch.Tensor, particle_pre_shifted: torch.Tensor,
                                     layout: PackedFourierLayout, workspace: CorrelationWorkspace,
                                     chunk_size_a: int = 16, chunk_size_b: int = 32
                                     ) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """(scores [n_a, n_b] float32, y [n_a, n_b] int64, x [n_a, n_b] int64):
    1024 * n^2 * max over the crop window of irfft2(T_a * P_b) and its
    row-major first argmax (v606:1418-1449). The chunk sizes are accepted for
    signature compatibility; the kernel has no chunking."""
    T = templates_pre_shifted.contiguous()
    P = particle_pre_shifted.contiguous()
    n_a, n_b = T.shape[0], P.shape[0]
    s, y, x = workspace.ensure(n_a, n_b)
    ptr = torch.tensor([0, n_a], dtype=torch.int32, device=workspace.device)
    nat.call("gisapr_correlate", nat.Context.for_device(workspace.device).handle,
             nat.stream_of(workspace.device), nat.ptr(T), nat.ptr(P), nat.ptr(ptr),
             nat.ptr(workspace.idx), 1, n_b, layout.size, layout.crop_size, nat.ptr(s), nat.ptr(y),
             nat.ptr(x))
    return s.view(n_a, n_b), y.view(n_a, n_b).long(), x.view(n_a, n_b).long()


def make_result_records(particle: ParticleRecord, fake_psi: Sequence[float], model_rot: Sequence[float],
                        model_tilt: Sequence[float], model_indices: Sequence[int], scores: torch.Tensor,
                        y_positions: torch.Tensor, x_positions: torch.Tensor, crop_size: int,
                        trans_scale_factor: float, cc_threshold: float = 3.0,
                        accuracy: float = 11.0) -> List[List[object]]:
    """The three text records of one particle (v606:1452-1516). The first
    maximum, mean, population sigma and z-score come from the
    particle_results kernel."""
    if scores.numel() == 0:
        return []
    dev = scores.device
    n_a, n_psi = scores.shape
    ptr = torch.tensor([0, n_a], dtype=torch.int32, device=dev)
    s = scores.to(torch.float32).contiguous()
    ys = y_positions.to(torch.int32).contiguous()
    xs = x_positions.to(torch.int32).contiguous()
    outs = [torch.empty(1, dtype=t, device=dev) for t in
            (torch.int32, torch.int32, torch.float32, torch.int32, torch.int32, torch.float32)]
    nat.call("gisapr_particle_results", nat.stream_of(dev), nat.ptr(ptr), nat.ptr(s), nat.ptr(ys),
             nat.ptr(xs), 1, n_psi, *[nat.ptr(o) for o in outs])
    best_e, best_psi, peak, py, px, z = [o.item() for o in outs]
    return format_records(particle, fake_psi, model_rot, model_tilt, model_indices, int(best_e),
                          int(best_psi), float(peak), int(py), int(px), float(z), crop_size,
                          trans_scale_factor, cc_threshold, accuracy)


def format_records(particle, fake_psi, model_rot, model_tilt, model_indices, local_index, psi_index,
                   peak, peak_y, peak_x, z, crop_size, trans_scale_factor, cc_threshold=3.0,
                   accuracy=11.0):
    rem_x = float(crop_size // 2 - peak_x) / trans_scale_factor
    rem_y = float(crop_size // 2 - peak_y) / trans_scale_factor
    g = int(model_indices[local_index])
    ang = calculate_angular_distance(model_rot[g], model_tilt[g], 0.0, particle.rot, particle.tilt, 0.0)
    return [
        ["cc: ", particle.line_index, float(z), 1 if z > cc_threshold else 0,
         1 if ang < accuracy else 0, model_rot[g], model_tilt[g], ang, round(rem_x), round(rem_y), 0, 0],
        ["psi: ", particle.line_index, float(fake_psi[psi_index]), float((particle.psi + 360.0) % 360.0)],
        ["rawCC: ", particle.line_index, float(peak)],
    ]
