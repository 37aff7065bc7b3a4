"""Job-resident candidate scoring on one GPU.

A ScoringJob holds everything that does not depend on the candidate pose on
the device: the particle spectra (CTF * ISSPA weighted, conjugated,
normalised, pre-shifted), the local direction lists as CSR arrays, the
fixed-context density and the output buffers. Scoring a pose then enqueues
six launches on the current stream (splat with fused FFT input, 3-D R2C,
projector, correlation, per-particle records, score sum) and reads back one
float64. This is the in-process form of the reference's worker request
``search_from_pdb`` / ``search_batch_from_pdb`` (Z3 gisapr_worker.py,
Lite gisapr_batch_search.py:142-364) with the Python per-particle loop of
run_search (v606:1749-1810) replaced by batched kernels.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _native as nat
from .pdb2mrc import MovedChainDensity
from .search import (IntegratedProjector, PackedCTFTorch, PackedFourierLayout, ParticleFourierPreparer,
                     PsiGridBank, format_records)
from .tables import (ModelAngles, ParticleRecord, build_local_orientation_entries, centered_to_packed_np,
                     expand_radial_values, generate_soft_mask, psi_sampling_for_record)


@dataclass
class JobConfig:
    box: int
    apix: float
    crop: int
    psi_step: float
    local_range: float
    do_local_search: bool = True
    newbox: Optional[int] = None
    res: Optional[float] = None
    mask_radius: Optional[int] = None
    mask_edge: int = 6
    discard_mask: bool = False
    kk: float = 3.0
    voltage: float = 300.0
    cs: float = 2.7
    chain_id: str = "A"
    include_hetatm: bool = False

    @property
    def new_box(self) -> int:
        return int(self.newbox or self.box)

    @property
    def resolution(self) -> float:
        return float(self.res) if self.res is not None else 2.0 * float(self.apix)


class ScoringJob:
    """One refinement job (model + particles) resident on one CUDA device."""

    def __init__(self, cfg: JobConfig, pdb_text: Optional[str], angles: ModelAngles,
                 records: Sequence[ParticleRecord], images, fsc_values=None, has_ctf: bool = True,
                 device="cuda", local: Optional[Sequence[Sequence[int]]] = None,
                 fsc_map: Optional[np.ndarray] = None):
        """``pdb_text`` None makes a job without a model: densities are then
        given per call (score_volume). ``local`` (one direction list per
        record) replaces the lists built from the local range; ``fsc_map`` (the
        centred new_box x new_box map of read_fsc_map) replaces
        ``fsc_values``."""
        t0 = time.perf_counter()
        self.cfg = cfg
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("ScoringJob needs a CUDA device")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        dev = self.device
        n, nb = int(cfg.box), cfg.new_box
        self.angles = angles
        self.records = list(records)
        self.layout = PackedFourierLayout(nb, cfg.crop, dev)
        new_apix = n / nb * cfg.apix
        self.trans_scale = cfg.apix / new_apix
        # local direction lists -> compact template bank + CSR
        if local is None:
            if cfg.do_local_search:
                entries = build_local_orientation_entries(self.records, angles.rot, angles.tilt, cfg.local_range)
                local = [e[1:] for e in entries]
            else:
                local = [list(range(len(angles.rot))) for _ in self.records]
        self._set_lists(local)
        # mask and FSC
        mask_radius = cfg.mask_radius if cfg.mask_radius is not None else int(round(0.43 * n))
        mask_np = generate_soft_mask((n, n), mask_radius, cfg.mask_edge)
        self.mask = None if cfg.discard_mask else torch.from_numpy(mask_np).to(dev)
        if fsc_map is None:
            fsc = np.ones(n, np.float32) if fsc_values is None else np.asarray(fsc_values, np.float32)
            fsc_map = expand_radial_values(fsc, nb)
        fsc_map = np.asarray(fsc_map, dtype=np.float32)
        if fsc_map.shape != (nb, nb):
            raise ValueError(f"FSC map must be {nb}x{nb}, got {fsc_map.shape}")
        self.packed_fsc = torch.from_numpy(np.ascontiguousarray(centered_to_packed_np(fsc_map))).to(dev)
        # psi sampling
        self.psi_meta = [psi_sampling_for_record(r.psi, cfg.psi_step, cfg.do_local_search, cfg.local_range)
                         for r in self.records]
        self.n_psi = len(self.psi_meta[0][1]) if self.psi_meta else 1
        uniq = list(dict.fromkeys(float(np.round(a, 6)) for _, eff in self.psi_meta for a in eff))
        self.psi_bank = PsiGridBank(n, dev, uniq)
        psi_index = np.asarray([[self.psi_bank.angle_to_index[float(np.round(a, 6))] for a in eff]
                                for _, eff in self.psi_meta], dtype=np.int32).reshape(-1, self.n_psi)
        # particle spectra, once per job
        ctfgen = PackedCTFTorch(nb, new_apix, cfg.cs, cfg.voltage, cfg.kk, dev)
        ctf = ctfgen.batch(self.records, has_ctf)
        imgs = torch.as_tensor(np.asarray(images, dtype=np.float32)) if not torch.is_tensor(images) else images
        imgs = imgs.to(dev, torch.float32).contiguous()
        preparer = ParticleFourierPreparer(n, nb, dev, self.layout, self.mask, self.psi_bank)
        self.stack = preparer.prepare_batch(imgs, torch.from_numpy(psi_index), ctf)
        del imgs, ctf
        # model
        self.density = None if pdb_text is None else MovedChainDensity(
            pdb_text, cfg.chain_id, n, cfg.apix, cfg.resolution, dev, include_hetatm=cfg.include_hetatm,
            from_text=True)
        self.projector = IntegratedProjector(dev, n, nb, self.layout, self.mask, self.packed_fsc)
        # power-of-two boxes: the splat writes the density and the blocked
        # volume transform reads it; other boxes: the splat writes the padded
        # FFT input of the cuFFT transform
        self.vol_buf = torch.empty((n, n, n), dtype=torch.float32, device=dev) \
            if self.projector.blocked_fft else None
        self._alloc_search_buffers()
        np_ = len(self.records)
        self.best_entry = torch.empty(np_, dtype=torch.int32, device=dev)
        self.best_psi = torch.empty(np_, dtype=torch.int32, device=dev)
        self.peak = torch.empty(np_, dtype=torch.float32, device=dev)
        self.peak_y = torch.empty(np_, dtype=torch.int32, device=dev)
        self.peak_x = torch.empty(np_, dtype=torch.int32, device=dev)
        self.zscore = torch.empty(np_, dtype=torch.float32, device=dev)
        self.total = torch.zeros(1, dtype=torch.float64, device=dev)
        self.pose_dev = torch.zeros(12, dtype=torch.float64, device=dev)
        self.pose_host = torch.zeros(12, dtype=torch.float64).pin_memory()
        # score(): per host thread, the candidate's launch sequence is captured
        # as a CUDA graph on the second call and replayed after that
        self.use_graph = True
        self._graphs: Dict[int, tuple] = {}
        # score() and score_volume() write the job's device buffers (density,
        # bank, maps, records, total): calls from several host threads take
        # turns, as the reference's worker serialises requests under a lock
        self._call_lock = threading.RLock()
        self._warm: Dict[int, int] = {}
        self.total_host = torch.zeros(1, dtype=torch.float64).pin_memory()
        torch.cuda.synchronize(dev)
        self.setup_s = time.perf_counter() - t0

    def _set_lists(self, local: Sequence[Sequence[int]]) -> None:
        """Direction lists (one per record) -> needed directions and CSR arrays."""
        if len(local) != len(self.records):
            raise ValueError("local needs one direction list per particle record")
        n_dirs = len(self.angles.rot)
        local = [[int(k) for k in l] for l in local]
        if any(k < 0 or k >= n_dirs for l in local for k in l):
            raise ValueError("a local direction index is outside the angle table")
        dev = self.device
        self.local = local
        needed = sorted({k for l in local for k in l})
        self.needed = needed
        slot = {d: i for i, d in enumerate(needed)}
        ptr = np.zeros(len(local) + 1, dtype=np.int32)
        ptr[1:] = np.cumsum([len(l) for l in local])
        idx = np.asarray([slot[k] for l in local for k in l], dtype=np.int32)
        self.local_ptr = torch.from_numpy(ptr).to(dev)
        self.local_idx = torch.from_numpy(idx if len(idx) else np.zeros(1, np.int32)).to(dev)
        self.nnz = int(ptr[-1])
        self.needed_dirs = torch.tensor(needed if needed else [0], dtype=torch.int32, device=dev)
        self.needed_slots = torch.arange(max(1, len(needed)), dtype=torch.int32, device=dev)

    def _alloc_search_buffers(self) -> None:
        nb, dev = self.cfg.new_box, self.device
        self.bank = torch.empty((max(1, len(self.needed)), nb, nb // 2 + 1), dtype=torch.complex64, device=dev)
        m = max(1, self.nnz) * self.n_psi
        self.score_buf = torch.empty(m, dtype=torch.float32, device=dev)
        self.y_buf = torch.empty(m, dtype=torch.int32, device=dev)
        self.x_buf = torch.empty(m, dtype=torch.int32, device=dev)

    def set_local(self, local: Sequence[Sequence[int]]) -> None:
        """Replace the per-particle direction lists; the prepared particle
        spectra stay resident. Batches built on this job before the call
        must be rebuilt."""
        self._set_lists(local)
        self._alloc_search_buffers()
        self._graphs.clear()
        self._warm.clear()

    # ------------------------------------------------------------------
    # launches of this engine per scored candidate at a power-of-two box up
    # to 128: atoms + splat, the three passes of the volume transform, slice
    # rows + template tail, correlation, records, score sum (at boxes 96 and
    # 192 the volume transform is cuFFT's, whose kernels are not counted)
    KERNELS_PER_CANDIDATE = 10

    @staticmethod
    def projector_launches(box: int, n_build: int = 1) -> int:
        """Kernels of one projector call of ``n_build`` templates, as the
        library reports them: three in the shared-memory path (powers of two
        up to 128), one in the general path (boxes 96 and 192); for box 256
        the blocked spectrum copy, then the gather kernel and the general
        kernel per 4,096 templates."""
        n = int(nat.load().gisapr_project_launches(int(box), max(1, int(n_build))))
        if n < 0:
            raise ValueError(f"unsupported box {box}")
        return n

    def template_launches(self) -> int:
        """Kernels of this library that one candidate's density, volume
        transform and templates enqueue: the splat (2), the blocked volume
        transform (3) and the projector without its blocked copy at
        power-of-two boxes; elsewhere the splat and the projector."""
        proj = self.projector_launches(self.cfg.box, len(self.needed))
        if self.projector.blocked_fft:
            return 2 + 3 + max(0, proj - 1)
        return 2 + proj

    def launches_per_candidate(self) -> int:
        return self.template_launches() + 3
    STAGES = ("density", "volume_fft", "templates", "correlate", "records")

    def enqueue(self, pose_device: torch.Tensor, write_volume: Optional[torch.Tensor] = None,
                stage_events: Optional[Dict[str, list]] = None) -> None:
        """Enqueue one candidate on the current stream; pose_device is
        [rot(9), shift(3)] float64 on the device. The score lands in
        self.total. ``stage_events`` (stage -> list) collects a pair of CUDA
        events around each stage when given."""
        if self.density is None:
            raise ValueError("this job has no model; score densities with score_volume")
        mark = self._marker(stage_events)
        mark("density", False)
        vol = self.model_density(self.density, pose_device, write_volume)
        mark("density", True)
        self._enqueue_search(vol, mark)

    def model_density(self, model, pose_device: torch.Tensor, out: Optional[torch.Tensor] = None):
        """Enqueue one moved-chain density for the projector: into ``out``
        (or the job's buffer) for the blocked transform of power-of-two
        boxes, else into the padded FFT input (returns None)."""
        if self.projector.blocked_fft:
            vol = out if out is not None else self.vol_buf
            model.generate(None, out=vol, write_padded=False, pose_device=pose_device)
            return vol
        model.generate(None, out=out, write_padded=True, pose_device=pose_device)
        return None

    def enqueue_templates(self, volume: Optional[torch.Tensor], bank: torch.Tensor) -> None:
        """Volume spectrum and the needed templates into ``bank`` (``volume``
        None: the padded FFT input the splat wrote)."""
        if self.projector.blocked_fft:
            self.projector.volume_spectrum_blocked(volume)
        else:
            self.projector.volume_spectrum(volume)
        if self.needed:
            self.projector.project(self.angles, self.needed_dirs, bank, self.needed_slots)

    def enqueue_volume(self, volume: torch.Tensor, stage_events: Optional[Dict[str, list]] = None) -> None:
        """Enqueue the search of one given density ([box]^3 float32 on the
        job's device) on the current stream; the score lands in self.total."""
        n = int(self.cfg.box)
        if volume.shape != (n, n, n) or volume.dtype != torch.float32 or volume.device != self.device:
            raise ValueError(f"density must be a float32 [{n}]^3 tensor on {self.device}")
        self._enqueue_search(volume.contiguous(), self._marker(stage_events))

    @staticmethod
    def _marker(stage_events):
        def mark(stage, end):
            if stage_events is None:
                return
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            if end:
                stage_events[stage][-1].append(ev)
            else:
                stage_events.setdefault(stage, []).append([ev])
        return mark

    def _enqueue_search(self, volume: Optional[torch.Tensor], mark) -> None:
        """Volume spectrum (of ``volume``, or of the padded input the splat
        wrote), templates, correlation, per-particle records and score sum."""
        ctx = nat.Context.for_device(self.device).handle
        st = nat.stream_of(self.device)
        mark("volume_fft", False)
        if self.projector.blocked_fft:
            self.projector.volume_spectrum_blocked(volume)
        else:
            self.projector.volume_spectrum(volume)
        mark("volume_fft", True)
        mark("templates", False)
        if self.needed:
            self.projector.project(self.angles, self.needed_dirs, self.bank, self.needed_slots)
        mark("templates", True)
        mark("correlate", False)
        nat.call("gisapr_correlate", ctx, st, nat.ptr(self.bank), nat.ptr(self.stack), nat.ptr(self.local_ptr),
                 nat.ptr(self.local_idx), len(self.records), self.n_psi, self.cfg.new_box, self.cfg.crop,
                 nat.ptr(self.score_buf), nat.ptr(self.y_buf), nat.ptr(self.x_buf))
        mark("correlate", True)
        mark("records", False)
        nat.call("gisapr_particle_results", st, nat.ptr(self.local_ptr), nat.ptr(self.score_buf),
                 nat.ptr(self.y_buf), nat.ptr(self.x_buf), len(self.records), self.n_psi,
                 nat.ptr(self.best_entry), nat.ptr(self.best_psi), nat.ptr(self.peak), nat.ptr(self.peak_y),
                 nat.ptr(self.peak_x), nat.ptr(self.zscore))
        nat.call("gisapr_score_sum", st, nat.ptr(self.local_ptr), nat.ptr(self.peak), len(self.records),
                 nat.ptr(self.total))
        mark("records", True)

    def score(self, pose) -> float:
        """sum_i exp(rawCC_i / 1024) of one pose (degrees, Angstrom)."""
        t = self.density.pose_tensor(pose)
        with self._call_lock:
            return self._score(t)

    def _score(self, pose_tensor: torch.Tensor) -> float:
        self.pose_host.copy_(pose_tensor)
        self.pose_dev.copy_(self.pose_host, non_blocking=True)
        g = self._score_graph()
        if g is not None:
            g.replay()
        else:
            self.enqueue(self.pose_dev)
        self.total_host.copy_(self.total, non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        self._check_projector()
        return float(self.total_host[0])

    def _check_projector(self) -> None:
        """Raise if this call's projector gave up waiting for a template
        plane (the stream is idle here: one 4-byte read)."""
        projector_check(nat.Context.for_device(self.device).handle, torch.cuda.current_stream(self.device))

    def _score_graph(self):
        """The captured launch sequence of score() for this host thread, or
        None while it runs eagerly: the first call on a thread (and the first
        after set_local or a tuning change) creates plans, tables and scratch;
        the second is captured. Replays launch the same kernels on the same
        buffers, so scores are bitwise those of eager calls."""
        if not self.use_graph or self.density is None:
            return None
        key = threading.get_ident()
        ver = nat.tuning_version()
        ent = self._graphs.get(key)
        if ent is not None and ent[1] == ver:
            return ent[0]
        if self._warm.get(key) != ver:
            self._warm[key] = ver
            return None
        cur = torch.cuda.current_stream(self.device)
        side = torch.cuda.Stream(self.device)
        side.wait_stream(cur)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            self.enqueue(self.pose_dev)
        cur.wait_stream(side)
        self._graphs[key] = (g, ver)
        return g

    def score_many(self, poses) -> np.ndarray:
        return np.asarray([self.score(p) for p in poses], dtype=np.float64)

    def score_volume(self, volume) -> float:
        """sum_i exp(rawCC_i / 1024) of one given density (array or tensor, [box]^3)."""
        if not torch.is_tensor(volume):
            volume = torch.from_numpy(np.ascontiguousarray(volume, dtype=np.float32))
        volume = volume.to(self.device, torch.float32)
        with self._call_lock:
            self.enqueue_volume(volume)
            self.total_host.copy_(self.total, non_blocking=True)
            torch.cuda.current_stream(self.device).synchronize()
            self._check_projector()
            return float(self.total_host[0])

    # ------------------------------------------------------------------
    def particle_results(self) -> Dict[str, np.ndarray]:
        """Per-particle arrays of the last scored pose."""
        out = dict(best_entry=self.best_entry, best_psi=self.best_psi, peak=self.peak,
                   peak_y=self.peak_y, peak_x=self.peak_x, zscore=self.zscore)
        return {k: v.cpu().numpy() for k, v in out.items()}

    def result_records(self) -> List[List[object]]:
        """The search text records of the last scored pose, in particle order
        (v606:1494-1516), skipping particles without directions."""
        return self.format_results(self.particle_results())

    def format_results(self, r: Dict[str, np.ndarray]) -> List[List[object]]:
        """Text records from per-particle arrays (best_entry, best_psi, peak,
        peak_y, peak_x, zscore), in particle order; particles without
        directions, or left out of a batch slot's subset (best_entry -1),
        have no record."""
        rows = []
        ptr = self.local_ptr.cpu().numpy()
        for i, rec in enumerate(self.records):
            if ptr[i + 1] <= ptr[i] or r["best_entry"][i] < 0:
                continue
            fake, _ = self.psi_meta[i]
            local_index = int(r["best_entry"][i] - ptr[i])
            rows.extend(format_records(rec, fake, self.angles.rot, self.angles.tilt, self.local[i], local_index,
                                       int(r["best_psi"][i]), float(r["peak"][i]), int(r["peak_y"][i]),
                                       int(r["peak_x"][i]), float(r["zscore"][i]), self.cfg.crop,
                                       self.trans_scale))
        return rows

    def search_text(self) -> str:
        return "".join(str(row) + "\n" for row in self.result_records())


def projector_check(ctx_handle, stream=None) -> None:
    """Raise if a shared-memory projector call on this native context gave
    up waiting for a template plane (those templates are NaN); resets the
    context's status word. Synchronizes ``stream`` (default: the current
    stream)."""
    st = C.c_int(0)
    s = nat.stream_of(torch.cuda.current_device()) if stream is None else C.c_void_p(stream.cuda_stream)
    nat.call("gisapr_projector_status", ctx_handle, s, C.byref(st))
    if st.value != 0:
        raise RuntimeError("projector: a template plane did not arrive within the wait bound; "
                           "its templates are NaN")


def idx_ptr(a: np.ndarray) -> C.c_void_p:
    """Host address of a contiguous numpy array (for the host-side ABI helpers)."""
    return C.c_void_p(a.ctypes.data)


def subset_mask(subsets, n_cand: int, n_particles: int) -> np.ndarray:
    """The [n_cand][n_particles] uint8 mask of per-slot particle subsets.

    ``subsets``: None (every slot scores every particle) or one entry per
    slot (at most n_cand; missing slots score every particle), each None
    (all particles), a sequence of particle indices, or a boolean mask of
    length n_particles. Raises ValueError for an index out of range, a
    repeated index, or a mask of the wrong length."""
    mask = np.ones((n_cand, n_particles), dtype=np.uint8)
    if subsets is None:
        return mask
    subsets = list(subsets)
    if len(subsets) > n_cand:
        raise ValueError(f"{len(subsets)} subsets for {n_cand} slots")
    for c, sub in enumerate(subsets):
        if sub is None:
            continue
        a = np.asarray(sub)
        if a.dtype == np.bool_:
            if a.shape != (n_particles,):
                raise ValueError(f"slot {c}: a boolean subset needs {n_particles} entries, got {a.shape}")
            mask[c] = a
            continue
        a = a.astype(np.int64, copy=False).reshape(-1)
        if a.size and (a.min() < 0 or a.max() >= n_particles):
            raise ValueError(f"slot {c}: particle index out of range 0..{n_particles - 1}")
        if np.unique(a).size != a.size:
            raise ValueError(f"slot {c}: repeated particle index")
        mask[c] = 0
        mask[c, a] = 1
    return mask


class BatchScoringJob:
    """Many candidates per launch sequence, replayed as one CUDA graph.

    A PSO/simplex generation is a batch of candidate poses; each slot of the
    batch is bound to one moving-chain model (models share the job's fixed
    context, so chains of different atom counts mix in one batch). Per slot
    the splat, volume FFT and projector write that candidate's template bank;
    one batched correlation then stages each particle's spectra on chip once
    for all candidates, and batched record and score kernels finish. After a
    warm-up run the whole sequence is captured into a CUDA graph; scoring a
    new generation copies the poses in and replays the graph. This is the
    GPU form of the Lite tree's round-batched evaluation
    (ZL gisapr_batch_search.py:251-364).

    Slots may score different particle subsets (``set_subsets``): a slot's
    score, records and search text are those of a job that holds only its
    particles. The subset mask lives on the device and is read when the
    kernels run, so subsets may change between graph replays. The plain
    correlation skips the (slot, particle) pairs left out; the tensor-core
    correlation computes every slot's rows of a particle tile and the
    records and score leave the pairs out.
    """

    PRECISIONS = ("fp32", "fp16x3", "fp16", "bf16x3", "bf16")
    # precision code of gisapr_correlate_tc_batch_ex (GISAPR_TC_*)
    TC_CODES = {"fp16": 0, "fp16x3": 1, "bf16": 2, "bf16x3": 3}

    def __init__(self, job: ScoringJob, n_cand: int, models: Optional[Sequence] = None,
                 model_of: Optional[Sequence[int]] = None, use_graph: bool = True, precision: str = "fp32",
                 tc_chunk: int = 128, lanes: int = 2):
        if precision not in self.PRECISIONS:
            raise ValueError(f"precision must be one of {self.PRECISIONS}, got {precision!r}")
        self.precision = precision
        if not 1 <= int(tc_chunk) <= self.TC_MAX_CAND:
            raise ValueError(f"tc_chunk must be in 1..{self.TC_MAX_CAND}")
        self.tc_chunk = int(tc_chunk)
        self.job = job
        self.n_cand = int(n_cand)
        if not models and job.density is None:
            raise ValueError("a job without a model needs the batch's models")
        self.models = list(models) if models else [job.density]
        self.model_of = list(model_of) if model_of is not None else [i % len(self.models) for i in range(self.n_cand)]
        if len(self.model_of) != self.n_cand:
            raise ValueError("model_of needs one model index per candidate")
        dev = job.device
        nb = job.cfg.new_box
        n_needed = max(1, len(job.needed))
        self.banks = torch.empty((self.n_cand, n_needed, nb, nb // 2 + 1), dtype=torch.complex64, device=dev)
        self.bank_stride = n_needed * nb * (nb // 2 + 1)
        m = max(1, job.nnz) * job.n_psi
        self.score_buf = torch.empty((self.n_cand, m), dtype=torch.float32, device=dev)
        self.y_buf = torch.empty((self.n_cand, m), dtype=torch.int32, device=dev)
        self.x_buf = torch.empty((self.n_cand, m), dtype=torch.int32, device=dev)
        np_ = len(job.records)
        shape = (self.n_cand, np_)
        self.best_entry = torch.empty(shape, dtype=torch.int32, device=dev)
        self.best_psi = torch.empty(shape, dtype=torch.int32, device=dev)
        self.peak = torch.empty(shape, dtype=torch.float32, device=dev)
        self.peak_y = torch.empty(shape, dtype=torch.int32, device=dev)
        self.peak_x = torch.empty(shape, dtype=torch.int32, device=dev)
        self.zscore = torch.empty(shape, dtype=torch.float32, device=dev)
        self.totals = torch.zeros(self.n_cand, dtype=torch.float64, device=dev)
        self.subset = torch.ones(shape, dtype=torch.uint8, device=dev)
        self.poses_dev = torch.zeros((self.n_cand, 12), dtype=torch.float64, device=dev)
        self.poses_host = torch.zeros((self.n_cand, 12), dtype=torch.float64).pin_memory()
        self.totals_host = torch.zeros(self.n_cand, dtype=torch.float64).pin_memory()
        self.use_graph = bool(use_graph)
        self.graph = None
        self.stream = torch.cuda.Stream(dev)
        self._setup_lanes(int(lanes))
        if precision != "fp32":
            self._setup_tensor_path(n_needed)

    def _setup_lanes(self, lanes: int) -> None:
        """Template lanes: slot c's density, volume transform and projector run
        on lane c % lanes. Lane 0 is the caller's stream and native context;
        each further lane has its own stream, native context (its own
        splat, transform and projector scratch) and density buffer, so the
        slots' template stages overlap on the GPU (one slot's short splat
        and transform launches fill the tail of another's projector)."""
        if lanes < 1:
            raise ValueError("lanes must be at least 1")
        job = self.job
        dev = torch.device(job.device)
        idx = dev.index if dev.index is not None else torch.cuda.current_device()
        self.lanes = [(None, None, None)]
        for _ in range(1, min(lanes, self.n_cand)):
            vol = torch.empty_like(job.vol_buf) if job.vol_buf is not None else None
            self.lanes.append((nat.Context(idx), torch.cuda.Stream(dev), vol))

    TC_MAX_CAND = 128  # candidates per tensor-core launch

    def _setup_tensor_path(self, n_needed: int) -> None:
        """fp16 hi/lo bank scratch, direction-sorted work lists and status word.

        Batches of more than ``tc_chunk`` (at most 128) candidates run as
        equal chunks, one tensor-core launch each (the tile shape depends on
        the chunk size; the autotuner picks tc_chunk)."""
        job = self.job
        lib = nat.load()
        nb = job.cfg.new_box
        self.n_slot = n_needed
        n_chunks = -(-self.n_cand // self.tc_chunk)
        size = -(-self.n_cand // n_chunks)
        self.tc_chunks = [(c0, min(size, self.n_cand - c0)) for c0 in range(0, self.n_cand, size)]
        per_cand = int(lib.gisapr_tc_bank_bytes(n_needed, nb))
        self.tbank = torch.empty(size * per_cand, dtype=torch.uint8, device=job.device)
        ptr = np.ascontiguousarray(job.local_ptr.cpu().numpy(), dtype=np.int32)
        idx = np.ascontiguousarray(job.local_idx.cpu().numpy(), dtype=np.int32)
        np_ = len(job.records)
        self._host_map = (ptr, idx)
        self.tc_plans = {}
        for _, cc in self.tc_chunks:
            self._tc_plan(cc)
        self.tc_status = torch.zeros(1, dtype=torch.int32, device=job.device)
        self.t_scale, self.p_scale = self.column_scales(job)
        self.tc_wait_limit = 0  # default bound of the kernel's on-chip waits

    @staticmethod
    def column_scales(job: ScoringJob):
        """Per stored bank column, the powers of two that multiply the
        template and the particle operands of the tensor-core correlation
        (undone after accumulation), so that weak high-frequency columns
        keep the 16-bit types' normal range. Particle side: from the job's
        largest coefficient of the column (scaled into [0.25, 0.5]).
        Template side: from the column's largest FSC weight (a template
        coefficient is at most its FSC weight times its whitened amplitude
        over the template norm), up to 2^8, only for weights below 1/4.
        Both are job constants; a template value that still leaves fp16's
        range is reported by the kernel's status word."""
        nb = job.cfg.new_box
        h = nb // 2 + 1
        with torch.no_grad():
            pmax = job.stack.abs().amax(dim=(0, 1, 2)).float().cpu().numpy()   # [H] stored columns
        fsc = job.packed_fsc.cpu().numpy().reshape(nb, h)                         # packed (unshifted) columns
        stored_of = (np.arange(h) + h // 2) % h                                    # packed column -> stored
        fmax = np.zeros(h, np.float64)
        fmax[stored_of] = np.abs(fsc).max(axis=0)
        with np.errstate(divide="ignore"):
            pe = np.where(pmax > 0, np.floor(np.log2(0.5 / np.maximum(pmax, 1e-30))), 0.0)
            te = np.where(fmax > 0, np.floor(np.log2(0.25 / np.maximum(fmax, 1e-30))), 8.0)
        pe = np.clip(pe, -8, 12)
        te = np.clip(te, 0, 8)
        dev = job.device
        return (torch.from_numpy(np.exp2(te).astype(np.float32)).to(dev),
                torch.from_numpy(np.exp2(pe).astype(np.float32)).to(dev))

    def _tc_plan(self, cc: int):
        """Work list of the tensor-core kernel for chunks of cc candidates (cached)."""
        if cc not in self.tc_plans:
            job = self.job
            ptr, idx = self._host_map
            np_ = len(job.records)
            count = C.c_int(0)
            nat.call("gisapr_tc_plan_work", idx_ptr(ptr), idx_ptr(idx), np_, cc, job.n_psi, job.cfg.crop, None, 0,
                     C.byref(count))
            work = np.zeros((max(1, count.value), 2), dtype=np.int32)
            nat.call("gisapr_tc_plan_work", idx_ptr(ptr), idx_ptr(idx), np_, cc, job.n_psi, job.cfg.crop,
                     idx_ptr(work), work.shape[0], C.byref(count))
            self.tc_plans[cc] = (torch.from_numpy(work).to(job.device), count.value)
        return self.tc_plans[cc]

    def tc_mma_flops(self) -> float:
        """Tensor-core flops one generation issues: per work item and K step
        (32 rows of a packed column, 64 K elements) four MMAs of
        M = 128 x N x K = 16 per pass (three passes for the split forms),
        N = psi angles per tile x 2 crop (rounded up to 8 per psi, then to 16)."""
        if self.precision == "fp32":
            return 0.0
        nb, crop = self.job.cfg.new_box, self.job.cfg.crop
        psi_group = 3 if crop <= 12 else 2
        kn = -(-psi_group * (-(-2 * crop // 8) * 8) // 16) * 16
        passes = 3 if self.precision in ("fp16x3", "bf16x3") else 1
        steps = (nb // 2 + 1) * (nb // 32)
        items = sum(self._tc_plan(cc)[1] for _, cc in self.tc_chunks)
        return float(items) * steps * passes * 4 * 2.0 * 128 * kn * 16

    def _chunks(self, n_active: int):
        if n_active == self.n_cand:
            return self.tc_chunks
        n_chunks = -(-n_active // self.tc_chunk)
        size = -(-n_active // n_chunks)
        return [(c0, min(size, n_active - c0)) for c0 in range(0, n_active, size)]

    def check_status(self) -> None:
        """Raise if a projector plane wait of any template lane ran out (its
        templates are NaN), an on-chip barrier wait of the tensor-core kernel
        ran out (status 1) or a scaled template value left the operand
        type's range (status 2)."""
        dev = self.job.device
        for lane_ctx, lane_stream, _ in self.lanes:
            ctx = lane_ctx if lane_ctx is not None else nat.Context.for_device(dev)
            projector_check(ctx.handle, lane_stream if lane_stream is not None else self.stream)
        if self.precision == "fp32":
            return
        st = int(self.tc_status.item())
        if st == 1:
            raise RuntimeError("tensor-core correlation: an on-chip barrier wait ran out; results are incomplete")
        if st == 2:
            raise RuntimeError("tensor-core correlation: a scaled template value left the operand range")
        if st != 0:
            raise RuntimeError(f"tensor-core correlation: status {st}")

    KERNELS_PER_BATCH = 3      # correlation, records, score sums

    def launches_per_batch(self) -> int:
        # per slot: splat (2 launches) and the projector; fp16 hi/lo bank copy
        # and tensor-core kernel per chunk instead of one plain kernel
        per_slot = self.job.template_launches()
        extra = 2 * len(self.tc_chunks) - 1 if self.precision != "fp32" else 0
        return self.n_cand * per_slot + self.KERNELS_PER_BATCH + extra

    def enqueue(self, marks: Optional[list] = None, n_active: Optional[int] = None) -> None:
        """Enqueue the whole batch on the current stream (poses already on the device).

        ``marks``: when a list is given (eager runs only), a CUDA event is
        recorded after each stage and appended as (stage, event).
        ``n_active``: score only the first n_active slots (eager runs only)."""
        job = self.job
        n_act = self.n_cand if n_active is None else int(n_active)
        if not 0 < n_act <= self.n_cand:
            raise ValueError(f"n_active must be in 1..{self.n_cand}, got {n_active}")
        dev = job.device
        ctx = nat.Context.for_device(dev).handle
        st = nat.stream_of(dev)

        def mark(name):
            if marks is not None:
                ev = torch.cuda.Event(enable_timing=True)
                ev.record()
                marks.append((name, ev))

        mark("start")
        n_lanes = min(len(self.lanes), n_act)
        main = torch.cuda.current_stream(dev)
        if n_lanes > 1:
            fork = torch.cuda.Event()
            fork.record(main)
            for _, lane_stream, _ in self.lanes[1:n_lanes]:
                lane_stream.wait_event(fork)
        for c in range(n_act):
            lane_ctx, lane_stream, lane_vol = self.lanes[c % n_lanes]
            model = self.models[self.model_of[c]]
            if lane_ctx is None:
                job.enqueue_templates(job.model_density(model, self.poses_dev[c]), self.banks[c])
            else:
                with torch.cuda.stream(lane_stream), nat.Context.using(lane_ctx):
                    job.enqueue_templates(job.model_density(model, self.poses_dev[c], out=lane_vol),
                                          self.banks[c])
        for _, lane_stream, _ in self.lanes[1:n_lanes]:
            join = torch.cuda.Event()
            join.record(lane_stream)
            main.wait_event(join)
        mark("templates")
        np_ = len(job.records)
        if self.precision == "fp32":
            nat.call("gisapr_correlate_batch_subset", ctx, st, nat.ptr(self.banks), self.bank_stride, n_act,
                     nat.ptr(job.stack), nat.ptr(job.local_ptr), nat.ptr(job.local_idx), np_, job.nnz, job.n_psi,
                     job.cfg.new_box, job.cfg.crop, nat.ptr(self.subset), nat.ptr(self.score_buf),
                     nat.ptr(self.y_buf), nat.ptr(self.x_buf))
        else:
            m = max(1, job.nnz) * job.n_psi
            for c0, cc in self._chunks(n_act):
                work, n_work = self._tc_plan(cc)
                nat.call("gisapr_correlate_tc_batch_ex", ctx, st,
                         nat.c_ptr_offset(self.banks, c0 * self.bank_stride * 8), self.bank_stride, cc, self.n_slot,
                         nat.ptr(self.tbank), nat.ptr(job.stack), nat.ptr(job.local_ptr), nat.ptr(job.local_idx),
                         nat.ptr(work), n_work, job.nnz, job.n_psi, job.cfg.new_box, job.cfg.crop,
                         self.TC_CODES[self.precision], nat.ptr(self.t_scale), nat.ptr(self.p_scale),
                         int(self.tc_wait_limit), nat.c_ptr_offset(self.score_buf, c0 * m * 4),
                         nat.c_ptr_offset(self.y_buf, c0 * m * 4), nat.c_ptr_offset(self.x_buf, c0 * m * 4),
                         nat.ptr(self.tc_status))
        mark("correlate")
        nat.call("gisapr_particle_results_subset", st, nat.ptr(job.local_ptr), nat.ptr(self.score_buf),
                 nat.ptr(self.y_buf), nat.ptr(self.x_buf), np_, job.n_psi, n_act, nat.ptr(self.subset),
                 nat.ptr(self.best_entry),
                 nat.ptr(self.best_psi), nat.ptr(self.peak), nat.ptr(self.peak_y), nat.ptr(self.peak_x),
                 nat.ptr(self.zscore))
        nat.call("gisapr_score_sum_subset", st, nat.ptr(job.local_ptr), nat.ptr(self.peak), np_, n_act,
                 nat.ptr(self.subset), nat.ptr(self.totals))
        mark("records")

    def stage_ms(self, poses) -> Dict[str, float]:
        """Device time of each stage of one eager batch (CUDA events on the batch stream)."""
        self.set_poses(poses)
        marks: list = []
        self.stream.wait_stream(torch.cuda.current_stream(self.job.device))
        with torch.cuda.stream(self.stream):
            self.enqueue(marks)
        self.stream.synchronize()
        return {marks[i][0]: marks[i - 1][1].elapsed_time(marks[i][1]) for i in range(1, len(marks))}

    def _ensure_graph(self) -> None:
        if self.graph is not None or not self.use_graph:
            return
        # warm-up outside capture: plans, tables and scratch are created here
        with torch.cuda.stream(self.stream):
            self.enqueue()
        self.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self.enqueue()
        self.graph = g

    def run(self) -> None:
        """Score the poses already in poses_dev (enqueue only; graph replay if captured)."""
        self._ensure_graph()
        if self.graph is not None:
            self.graph.replay()
        else:
            self.enqueue()

    def set_subsets(self, subsets) -> None:
        """Particle subsets per slot (see ``subset_mask`` for the forms;
        None: every slot scores every particle). They stay until changed.
        The mask is copied synchronously, so it is in place for the next
        run or graph replay on any stream."""
        mask = subset_mask(subsets, self.n_cand, len(self.job.records))
        self.subset.copy_(torch.from_numpy(mask))

    def set_poses(self, poses) -> None:
        self.poses_host[:len(poses)].copy_(MovedChainDensity.pose_tensors(poses))
        self.poses_dev.copy_(self.poses_host, non_blocking=True)

    def score_active(self, poses, stream=None, subsets=None) -> np.ndarray:
        """Scores of up to n_cand poses in one eager launch sequence on
        ``stream`` (default: the batch stream); slots past len(poses) are not
        computed. ``subsets``: set_subsets first when given. Blocks until the
        scores are on the host."""
        k = len(poses)
        if not 0 < k <= self.n_cand:
            raise ValueError(f"expected 1..{self.n_cand} poses, got {k}")
        t = MovedChainDensity.pose_tensors(poses)
        # the batch shares the job's density buffer and spectra with the
        # job's own score(): calls on one job take turns
        with self.job._call_lock:
            if subsets is not None:
                self.set_subsets(subsets)
            st = stream if stream is not None else self.stream
            self.poses_host[:k].copy_(t)
            with torch.cuda.stream(st):
                self.poses_dev[:k].copy_(self.poses_host[:k], non_blocking=True)
                self.enqueue(n_active=k)
                self.totals_host[:k].copy_(self.totals[:k], non_blocking=True)
            st.synchronize()
            self.check_status()
            return self.totals_host[:k].numpy().copy()

    def slot_results(self, n_slots: Optional[int] = None) -> List[Dict[str, np.ndarray]]:
        """Per-particle arrays of each of the first n_slots slots of the last batch."""
        k = self.n_cand if n_slots is None else int(n_slots)
        cols = dict(best_entry=self.best_entry, best_psi=self.best_psi, peak=self.peak, peak_y=self.peak_y,
                    peak_x=self.peak_x, zscore=self.zscore)
        host = {name: t[:k].cpu().numpy() for name, t in cols.items()}
        return [{name: a[c] for name, a in host.items()} for c in range(k)]

    def search_texts(self, n_slots: Optional[int] = None) -> List[str]:
        """The search text of each of the first n_slots slots of the last batch."""
        return ["".join(str(row) + "\n" for row in self.job.format_results(r))
                for r in self.slot_results(n_slots)]

    def score_batch(self, poses, subsets=None) -> np.ndarray:
        """Scores of len(poses) == n_cand poses, in slot order
        (``subsets``: set_subsets first when given)."""
        if len(poses) != self.n_cand:
            raise ValueError(f"expected {self.n_cand} poses, got {len(poses)}")
        with self.job._call_lock:  # shared buffers with the job's score(), as in score_active
            if subsets is not None:
                self.set_subsets(subsets)
            self._ensure_graph()
            self.set_poses(poses)
            self.run()
            self.totals_host.copy_(self.totals, non_blocking=True)
            torch.cuda.current_stream(self.job.device).synchronize()
            self.check_status()
            return self.totals_host.numpy().copy()
