"""File-based search: the standalone v606 command (v606:1525-1836) on the GPU engine.

``run_search(args)`` takes the reference's argument namespace (same names,
defaults and meaning, ``create_search_parser``), reads the model angle STAR,
the particle STAR and its MRC stacks, the FSC file and the model MRC, and
writes the search text (three records per particle) to ``args.o``, exactly
the records make_result_records formats in the reference.

The reference loops over particles in Python: read one image, prepare its
psi stack, gather its local templates, correlate, format. Here the selected
particles are processed in chunks whose prepared spectra fit a device budget
(``--particleChunkMB``, default 16 GiB; usually one chunk): a reader thread
fills a pinned host stack for the next chunk from the memory-mapped MRC
files while the device works on the current one, and each chunk is one
ScoringJob (every particle's CTF*ISSPA-weighted psi spectra prepared in one
batched launch) scored against the model's density with one template
projection, one correlation launch over the chunk's CSR direction lists and
one records launch. Text is formatted on the host from the per-particle
maxima. Tuning switches of the reference that select its own batching
(``--ctfBatchSize``, ``--chunkSizeA/B``, ``--projectionBatchSize``,
``--psiGridBuildBatch``, ``--ctfBackend``, ``--torchThreads``) are accepted
and have no effect on the result. ``--orientations-out`` writes each
particle's Top-K directions (``--keep-orientations``) to a bank file and
``--orientations-in`` restricts every particle to its bank's directions, in
the Lite tree's bank format (see orientation_bank).
"""
from __future__ import annotations

import argparse
import os
import pickle
import sys
import threading
import time
from pathlib import Path
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from .engine import JobConfig, ScoringJob
from .mrc import read_mrc, read_mrc_volume
from .orientation_bank import bank_settings, pack_bank, ranked_row, read_bank, restricted_indices, write_bank
from .tables import (ModelAngles, ParticleRecord, build_local_orientation_entries, psi_sampling_for_record,
                     read_fsc_map, read_model_angles, read_particle_table, select_particle_records)

__all__ = ["create_search_parser", "choose_device", "run_search", "ParticleMRCReader",
           "load_or_build_local_orientation_map", "main"]


def create_search_parser() -> argparse.ArgumentParser:
    """Arguments of the standalone search (v606:1525-1567), plus
    ``--particleChunkMB`` (device budget of one particle chunk)."""
    p = argparse.ArgumentParser(description="GisAPR model/particle local search on a GB300")
    p.add_argument("--i", type=str, required=True, help="Compatibility argument; model angles are read from --ang")
    p.add_argument("--p", type=str, required=True, help="Input particle STAR")
    p.add_argument("--FSC", type=str, default="", help="Input FSC file")
    p.add_argument("--o", type=str, required=True, help="Output search text file")
    p.add_argument("--kk", type=float, default=0.0)
    p.add_argument("--gpuid", type=int, default=0)
    p.add_argument("--oriboxsize", type=int, default=256)
    p.add_argument("--newboxsize", type=int, default=256)
    p.add_argument("--apix", type=float, default=1.42, help="Original particle pixel size")
    p.add_argument("--transRange", type=int, default=0, help="Compatibility argument; CCG peak determines translation")
    p.add_argument("--voltage", type=float, default=300.0)
    p.add_argument("--cs", type=float, default=2.7)
    p.add_argument("--maskRadius", type=int, default=110)
    p.add_argument("--maskEdge", type=int, default=6)
    p.add_argument("--ignoreFSC", action="store_true")
    p.add_argument("--discardMask", action="store_true")
    p.add_argument("--psiStep", type=float, default=15.0)
    p.add_argument("--start", type=int, default=-1)
    p.add_argument("--end", type=int, default=-1)
    p.add_argument("--doLocalSearch", action="store_true")
    p.add_argument("--localRange", type=float, default=20.0)
    p.add_argument("--doContinue", action="store_true")
    p.add_argument("--ang", type=str, required=True,
                   help="RELION angle STAR used directly for projections and model orientations")
    p.add_argument("--mrc", type=str, required=True, help="Input 3-D model MRC; retained on disk")
    p.add_argument("--ctfBackend", choices=("torch", "numpy"), default="torch")
    p.add_argument("--ctfBatchSize", type=int, default=256)
    p.add_argument("--projectionBatchSize", type=int, default=8)
    p.add_argument("--psiGridBuildBatch", type=int, default=8)
    p.add_argument("--ccgCropSize", type=int, default=32)
    p.add_argument("--chunkSizeA", type=int, default=16)
    p.add_argument("--chunkSizeB", type=int, default=32)
    p.add_argument("--outputBufferParticles", type=int, default=96)
    p.add_argument("--torchThreads", type=int, default=4)
    p.add_argument("--profileStages", action="store_true")
    p.add_argument("--particleChunkMB", type=float, default=16384.0,
                   help="Device memory for one chunk of prepared particle spectra")
    p.add_argument("--keep-orientations", dest="keep_orientations", type=_positive_int, default=3,
                   help="K of the Top-K direction bank")
    bank = p.add_mutually_exclusive_group()
    bank.add_argument("--orientations-in", dest="orientations_in", metavar="JSON",
                      help="Score only the directions saved in this calibration bank")
    bank.add_argument("--orientations-out", dest="orientations_out", metavar="JSON",
                      help="Calibrate: write each particle's Top-K directions to this bank")
    return p


def _positive_int(text: str) -> int:
    v = int(text)
    if v < 1:
        raise argparse.ArgumentTypeError("must be >= 1")
    return v


def choose_device(gpuid) -> torch.device:
    """``cuda:<gpuid>``; the GB300 engine has no CPU path, so a missing
    device raises instead of falling back (v606:1570-1578 warns and uses the CPU)."""
    if gpuid == "cpu" or not torch.cuda.is_available():
        raise RuntimeError("GisAPR GB300 search needs a CUDA device")
    torch.cuda.set_device(int(gpuid))
    return torch.device(f"cuda:{int(gpuid)}")


class ParticleMRCReader:
    """Particle images named ``<serial>@<stack>`` (v606:1259-1318).

    ``read(name)`` returns one image on the device through a pinned staging
    image; ``read_stack(records, out)`` fills a pinned host stack with many
    images, keeping the last stack file memory-mapped."""

    def __init__(self, expected_size: int, device) -> None:
        self.expected_size = int(expected_size)
        self.device = torch.device(device)
        self.last_filename: Optional[str] = None
        self.last_data: Optional[np.ndarray] = None
        n = self.expected_size
        self.host_staging = torch.empty((n, n), dtype=torch.float32, pin_memory=self.device.type == "cuda")
        self.device_staging = torch.empty((n, n), dtype=torch.float32, device=self.device)

    @staticmethod
    def resolve_filename(filename: str) -> str:
        return os.path.realpath(filename) if os.path.islink(filename) else filename

    def _image(self, image_name: str) -> np.ndarray:
        serial, filename = image_name.split("@", 1)
        filename = self.resolve_filename(filename)
        if filename != self.last_filename:
            self.last_data = read_mrc(filename, mmap=True)
            self.last_filename = filename
        data = self.last_data
        image = data if data.ndim < 3 else data[int(serial) - 1]
        if image.shape != (self.expected_size, self.expected_size):
            raise ValueError(f"Particle image shape {image.shape} does not match --oriboxsize "
                             f"{self.expected_size} in {image_name}")
        return image

    def read(self, image_name: str) -> torch.Tensor:
        np.copyto(self.host_staging.numpy(), np.asarray(self._image(image_name), dtype=np.float32),
                  casting="unsafe")
        self.device_staging.copy_(self.host_staging)
        return self.device_staging

    def read_stack(self, records: Sequence[ParticleRecord], out: torch.Tensor) -> torch.Tensor:
        """Images of ``records`` into out[:len(records)] (host, float32)."""
        view = out.numpy()
        for i, rec in enumerate(records):
            np.copyto(view[i], self._image(rec.image_name), casting="unsafe")
        return out[:len(records)]

    def close(self) -> None:
        self.last_data = None
        self.last_filename = None


def _local_cache_valid(entries, records: Sequence[ParticleRecord], n_models: int) -> bool:
    """Shape of a cached local-direction table (v606:381-393)."""
    if not isinstance(entries, list) or len(entries) != len(records):
        return False
    for entry, rec in zip(entries, records):
        if not isinstance(entry, list) or not entry or entry[0] != rec.line_index:
            return False
        if any(not isinstance(k, (int, np.integer)) or k < 0 or k >= n_models for k in entry[1:]):
            return False
    return True


def load_or_build_local_orientation_map(particle_star: str, particle_records: Sequence[ParticleRecord],
                                        model_angles: ModelAngles, local_range: float,
                                        use_cache: bool = True) -> Dict[int, List[int]]:
    """Line index -> local direction indices, cached beside the particle STAR
    under the reference's file name (v606:396-438), so caches written by
    either implementation are reused by the other."""
    cache = particle_star + "_LocalSearch_Angle_" + str(int(local_range)) + "_data.pkl"
    entries = None
    if use_cache and os.path.exists(cache):
        try:
            with open(cache, "rb") as fh:
                loaded = pickle.load(fh)
            if _local_cache_valid(loaded, particle_records, len(model_angles.rot)):
                entries = loaded
        except Exception as exc:  # noqa: BLE001 - an unreadable cache is rebuilt
            print(f"Could not read local-search cache ({exc}); rebuilding: {cache}")
    if entries is None:
        entries = build_local_orientation_entries(particle_records, model_angles.rot, model_angles.tilt,
                                                  local_range)
        if use_cache:
            tmp = cache + f".tmp.{os.getpid()}"
            try:
                with open(tmp, "wb") as fh:
                    pickle.dump(entries, fh, protocol=pickle.HIGHEST_PROTOCOL)
                os.replace(tmp, cache)
            except OSError as exc:
                print(f"Could not write local-search cache ({exc}): {cache}")
            finally:
                if os.path.exists(tmp):
                    os.remove(tmp)
    return {int(e[0]): [int(k) for k in e[1:]] for e in entries}


def _validate(args) -> None:
    box, new = int(args.oriboxsize), int(args.newboxsize)
    if box % 2 or new % 2:
        raise ValueError("oriboxsize and newboxsize must be even")
    if new > box:
        raise ValueError("newboxsize cannot exceed oriboxsize")
    if args.psiStep <= 0:
        raise ValueError("psiStep must be positive")


def job_config(args) -> JobConfig:
    """The scoring configuration the search arguments describe."""
    return JobConfig(box=int(args.oriboxsize), apix=float(args.apix), crop=int(args.ccgCropSize),
                     psi_step=float(args.psiStep), local_range=float(args.localRange),
                     do_local_search=bool(args.doLocalSearch), newbox=int(args.newboxsize),
                     mask_radius=int(args.maskRadius), mask_edge=int(args.maskEdge),
                     discard_mask=bool(args.discardMask), kk=float(args.kk), voltage=float(args.voltage),
                     cs=float(args.cs))


def particle_chunks(records: Sequence[ParticleRecord], per_particle_bytes: int, budget_mb: float):
    """Consecutive record chunks whose prepared spectra fit the budget."""
    size = max(1, int(budget_mb * 2 ** 20 // max(1, per_particle_bytes)))
    return [list(records[i:i + size]) for i in range(0, len(records), size)]


class _StackPrefetch:
    """Reads the next chunk's images into one of two pinned stacks on a thread."""

    def __init__(self, reader: ParticleMRCReader, chunks, box: int, pin: bool):
        self.reader = reader
        self.chunks = chunks
        cap = max((len(c) for c in chunks), default=1)
        self.bufs = [torch.empty((cap, box, box), dtype=torch.float32, pin_memory=pin) for _ in range(2)]
        self.result = [None, None]
        self.error: List[BaseException] = []
        self.thread = None

    def _load(self, k: int) -> None:
        try:
            self.result[k % 2] = self.reader.read_stack(self.chunks[k], self.bufs[k % 2])
        except BaseException as exc:  # noqa: BLE001 - re-raised on the caller's thread
            self.error.append(exc)

    def start(self, k: int) -> None:
        if k < len(self.chunks):
            self.thread = threading.Thread(target=self._load, args=(k,), daemon=True)
            self.thread.start()

    def get(self, k: int) -> torch.Tensor:
        self.thread.join()
        if self.error:
            raise self.error[0]
        return self.result[k % 2]


def run_search(args, *, model_volume=None, verbose: bool = True) -> Dict[str, float]:
    """Search every selected particle against the model and write the search
    text to ``args.o`` (appended with ``--doContinue``). Returns the stage
    times in seconds and the score sum_i exp(rawCC_i / 1024) of the written
    records. ``model_volume`` (a [box]^3 array or device tensor) replaces
    reading ``args.mrc``."""
    t_total = time.perf_counter()
    say = print if verbose else (lambda *a, **k: None)
    _validate(args)
    device = choose_device(args.gpuid)
    box, new = int(args.oriboxsize), int(args.newboxsize)
    cfg = job_config(args)
    say(f"Device: {device}")
    say(f"--i retained for compatibility and not read: {args.i}")
    say(f"Model orientations read directly from: {args.ang}")
    angles = read_model_angles(args.ang)
    table = read_particle_table(args.p)
    selected = select_particle_records(table, args.start, args.end)
    say("Model orientation count:", len(angles.rot))
    say("Selected particle count:", len(selected))
    say("Particle STAR data start line:", table.loop.first_row)
    t_local = time.perf_counter()
    if args.doLocalSearch:
        local_map = load_or_build_local_orientation_map(args.p, table.records, angles, float(args.localRange))
        say("Local orientation table time =", round(time.perf_counter() - t_local, 4), "seconds")
    else:
        every = list(range(len(angles.rot)))
        local_map = {rec.line_index: every for rec in selected}
    bank_in, bank_out = getattr(args, "orientations_in", None), getattr(args, "orientations_out", None)
    keep = int(getattr(args, "keep_orientations", 3))
    settings = None
    if bank_in or bank_out:
        settings = bank_settings(args.p, args.ang, keep, bool(args.doLocalSearch), float(args.localRange),
                                 float(args.psiStep))
    if bank_in:
        rows = read_bank(bank_in, settings)
        local_map = {rec.line_index: restricted_indices(rows.get(str(rec.line_index)), rec,
                                                        local_map.get(rec.line_index, []), angles, keep)
                     for rec in selected}
    ranked: Dict[str, dict] = {}
    for rec in selected:
        if not local_map.get(rec.line_index):
            print(f"WARNING: no model orientations for particle STAR line {rec.line_index}; skipping",
                  file=sys.stderr)
    fsc_map = read_fsc_map(args.FSC, box, new, bool(args.ignoreFSC))
    if model_volume is None:
        model_volume = read_mrc_volume(args.mrc)
    volume = (model_volume if torch.is_tensor(model_volume)
              else torch.from_numpy(np.ascontiguousarray(model_volume, dtype=np.float32)))
    if tuple(volume.shape) != (box, box, box):
        raise ValueError(f"Model volume box {tuple(volume.shape)} does not match --oriboxsize {box}")
    volume = volume.to(device, torch.float32).contiguous()

    n_psi = len(psi_sampling_for_record(0.0, float(args.psiStep), bool(args.doLocalSearch),
                                        float(args.localRange))[1]) if selected else 1
    per_particle = n_psi * new * (new // 2 + 1) * 8 + box * box * 4
    chunks = particle_chunks(selected, per_particle, float(args.particleChunkMB)) if selected else []
    reader = ParticleMRCReader(box, device)
    prefetch = _StackPrefetch(reader, chunks, box, pin=True)
    times = dict(setup_s=0.0, read_wait_s=0.0, search_s=0.0, write_s=0.0)
    score = 0.0
    mode = "a" if args.doContinue else "w"
    t_search = time.perf_counter()
    try:
        with open(args.o, mode, encoding="utf-8") as out:
            prefetch.start(0)
            for k, recs in enumerate(chunks):
                t0 = time.perf_counter()
                images = prefetch.get(k)
                times["read_wait_s"] += time.perf_counter() - t0
                t0 = time.perf_counter()
                job = ScoringJob(cfg, None, angles, recs, images, fsc_map=fsc_map, has_ctf=table.has_ctf,
                                 device=device, local=[local_map.get(r.line_index, []) for r in recs])
                prefetch.start(k + 1)  # the job holds its own device copy of the images
                times["setup_s"] += time.perf_counter() - t0
                t0 = time.perf_counter()
                score += job.score_volume(volume)
                if bank_out:
                    ranked.update(_bank_rows(job, angles, keep))
                times["search_s"] += time.perf_counter() - t0
                t0 = time.perf_counter()
                out.write(job.search_text())
                out.flush()
                times["write_s"] += time.perf_counter() - t0
                del job
    finally:
        if prefetch.thread is not None:
            prefetch.thread.join()
        reader.close()
    torch.cuda.synchronize(device)
    if bank_out:
        if any(r.get("invalid_rawcc") for r in ranked.values()):
            raise ValueError("a calibration peak is NaN: no orientation bank is written")
        write_bank(bank_out, pack_bank(settings, ranked, mrc=str(Path(args.mrc).resolve())))
    times["total_search_s"] = time.perf_counter() - t_search
    times["total_s"] = time.perf_counter() - t_total
    times["particles"] = float(len(selected))
    times["chunks"] = float(len(chunks))
    times["score"] = float(score)
    say("Total search time =", round(times["total_search_s"], 4), "seconds")
    say("Total execution time =", round(times["total_s"], 4), "seconds")
    if args.profileStages:
        say("Particle preparation (setup) time =", round(times["setup_s"], 6), "seconds")
        say("Templates + correlation + records time =", round(times["search_s"], 6), "seconds")
    return times


def _bank_rows(job: ScoringJob, angles, keep: int) -> Dict[str, dict]:
    """Top-K bank rows of one chunk's particles from its per-map maxima
    (maximised over psi per direction)."""
    ptr = job.local_ptr.cpu().numpy()
    peaks = job.score_buf[:max(1, job.nnz) * job.n_psi].view(-1, job.n_psi).amax(dim=1).cpu().numpy()
    rows = {}
    for i, rec in enumerate(job.records):
        a, b = int(ptr[i]), int(ptr[i + 1])
        rows[str(rec.line_index)] = (ranked_row(rec, job.local[i], angles, peaks[a:b], keep) if b > a
                                     else {"image": rec.image_name, "directions": []})
    return rows


def main(argv=None) -> None:
    args = create_search_parser().parse_args(argv)
    with torch.inference_mode():
        run_search(args)


if __name__ == "__main__":
    main()
