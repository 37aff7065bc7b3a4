"""Round evaluation of many models against one particle set (Lite gisapr_batch_search.py:142-364).

``BatchSearchEngine(search_globals, device, options).run(args, models,
orientation_rows=None, calibrate=False)`` keeps the Lite tree's call and
result shape: one dict per model with the score sum_i exp(rawCC_i / 1024),
the search text, the ranked direction rows (``calibrate``) and timings.

The particle set of ``args`` (STAR selection, stacks, CTF, psi grids, mask,
FSC) is prepared once into a resident ScoringJob and reused while the
arguments and input files are unchanged. Models are the Lite tree's density
keyword dicts. Those that move one chain of a source PDB by a pose
(``source_pdb``, ``chain_id``, ``pose``) are scored in batches of
``options['batch_candidates']`` through BatchScoringJob: per slot the splat
of the moved chain on the cached fixed context, volume FFT and projection,
then one batched correlation over every slot (tensor-core form with
``options['precision']`` "fp16x3" or "fp16"), replayed as a CUDA graph when
the batch is full. Other models (a whole PDB, centred or y-flipped
densities) get their density from generate_volume and are scored one at a
time. Given ``orientation_rows`` (the rows of a bank written by a
calibration run; see orientation_bank), each particle searches only the
bank's directions (orientation_bank_v1.py:71-90);
the prepared particle spectra stay resident and only the direction lists
change.

``search_globals`` is the reference's module namespace its engine calls
into; here every step is a kernel of this package, so it is accepted and not
used.
"""
from __future__ import annotations

import math
import os
import time
from collections import OrderedDict
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from .engine import BatchScoringJob, ScoringJob
from .orientation_bank import ranked_row, restricted_indices
from .pdb2mrc import MovedChainDensity, generate_volume
from .standalone import ParticleMRCReader, job_config
from .tables import (build_local_orientation_entries, read_fsc_map, read_model_angles, read_particle_table,
                     select_particle_records)

__all__ = ["BatchSearchEngine", "restricted_indices", "ranked_row", "file_key"]

DEFAULT_OPTIONS = dict(batch_candidates=64, batch_template_mb=65536.0, precision="fp32", use_graph=True)


def file_key(path: str):
    """Identity of an input file: resolved path, size and modification time."""
    st = os.stat(path)
    return (os.path.realpath(path), st.st_size, st.st_mtime_ns)


class _Context:
    pass


class BatchSearchEngine:
    RUNTIME_ARGS = {"o", "mrc", "i", "gpuid", "verbose", "orientations_in", "orientations_out"}

    def __init__(self, search_globals=None, device="cuda", options: Optional[dict] = None):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("BatchSearchEngine needs a CUDA device")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.options = dict(DEFAULT_OPTIONS)
        self.options.update(options or {})
        if self.options["precision"] not in BatchScoringJob.PRECISIONS:
            raise ValueError(f"precision must be one of {BatchScoringJob.PRECISIONS}")
        self.context: Optional[_Context] = None
        self.densities: "OrderedDict[tuple, MovedChainDensity]" = OrderedDict()
        self.batches: "OrderedDict[tuple, BatchScoringJob]" = OrderedDict()

    def sync(self) -> None:
        torch.cuda.synchronize(self.device)

    # ------------------------------------------------------------ context
    def _context(self, args) -> _Context:
        key = (tuple(sorted((k, v) for k, v in vars(args).items() if k not in self.RUNTIME_ARGS)),
               file_key(args.ang), file_key(args.p), file_key(args.FSC) if args.FSC else None)
        ctx = self.context
        if ctx is not None and ctx.key == key and \
                tuple(file_key(p) for p in ctx.stack_paths) == ctx.stack_keys:
            return ctx
        self.context = None
        self.batches.clear()
        box, new = int(args.oriboxsize), int(args.newboxsize)
        if box <= 0 or box % 2 or new % 2 or new > box or args.psiStep <= 0:
            raise ValueError("Invalid original/new box or psiStep")
        angles = read_model_angles(args.ang)
        table = read_particle_table(args.p)
        records = select_particle_records(table, args.start, args.end)
        if not records:
            raise ValueError("No particles selected for batch evaluation")
        if args.doLocalSearch:
            local = {int(e[0]): [int(k) for k in e[1:]] for e in build_local_orientation_entries(
                table.records, angles.rot, angles.tilt, float(args.localRange))}
        else:
            local = {rec.line_index: list(range(len(angles.rot))) for rec in records}
        fsc_map = read_fsc_map(args.FSC, box, new, bool(args.ignoreFSC))
        reader = ParticleMRCReader(box, self.device)
        images = reader.read_stack(records, torch.empty((len(records), box, box), dtype=torch.float32,
                                                        pin_memory=True))
        reader.close()
        lists = [local.get(r.line_index, []) for r in records]
        job = ScoringJob(job_config(args), None, angles, records, images, fsc_map=fsc_map,
                         has_ctf=table.has_ctf, device=self.device, local=lists)
        ctx = _Context()
        ctx.key, ctx.args, ctx.angles, ctx.table, ctx.records = key, args, angles, table, records
        ctx.local, ctx.job, ctx.lists = local, job, lists
        ctx.stack_paths = sorted({r.image_name.split("@", 1)[1] for r in records})
        ctx.stack_keys = tuple(file_key(p) for p in ctx.stack_paths)
        self.context = ctx
        return ctx

    def _density(self, model: dict, args) -> MovedChainDensity:
        src = model["source_pdb"]
        key = (file_key(src), str(model["chain_id"]), int(model["boxsize"]), float(model["apix"]),
               float(model["res"]), bool(model.get("include_hetatm", False)))
        d = self.densities.get(key)
        if d is None:
            d = MovedChainDensity(src, str(model["chain_id"]), int(model["boxsize"]), float(model["apix"]),
                                  float(model["res"]), self.device,
                                  include_hetatm=bool(model.get("include_hetatm", False)))
            self.densities[key] = d
            while len(self.densities) > 8:
                self.densities.popitem(last=False)
        else:
            self.densities.move_to_end(key)
        return d

    def _batch(self, job: ScoringJob, capacity: int, models: List[MovedChainDensity], model_of: List[int]):
        key = (id(job), tuple(job.needed), job.nnz, capacity, tuple(id(m) for m in models), tuple(model_of))
        b = self.batches.get(key)
        if b is None:
            b = BatchScoringJob(job, capacity, models=models, model_of=model_of,
                                use_graph=bool(self.options["use_graph"]), precision=self.options["precision"])
            self.batches[key] = b
            while len(self.batches) > 2:
                self.batches.popitem(last=False)
        return b

    @staticmethod
    def _moving(model: dict) -> bool:
        return bool(model.get("source_pdb")) and not model.get("do_center", False) \
            and not model.get("do_yflip", False)

    # ---------------------------------------------------------------- run
    def run(self, args, models: Sequence[dict], orientation_rows=None, calibrate: bool = False) -> List[dict]:
        if calibrate and orientation_rows is not None:
            raise ValueError("Cannot calibrate from restricted directions")
        self.sync()
        started = time.perf_counter()
        ctx = self._context(args)
        job = ctx.job
        box = int(args.oriboxsize)
        for m in models:
            if int(m["boxsize"]) != box:
                raise ValueError(f"model box {m['boxsize']} does not match --oriboxsize {box}")
        if orientation_rows is not None:
            keep = int(args.keep_orientations)
            lists = [restricted_indices(orientation_rows.get(str(r.line_index)), r,
                                        ctx.local.get(r.line_index, []), ctx.angles, keep)
                     for r in ctx.records]
        else:
            lists = ctx.lists
        if lists != job.local:
            job.set_local(lists)
            self.batches.clear()
        keep = int(args.keep_orientations) if calibrate else 0
        nb = int(args.newboxsize)
        per_model = max(1, len(job.needed) * nb * (nb // 2 + 1) * 8)
        budget = float(self.options["batch_template_mb"]) * 2 ** 20
        capacity = max(1, min(int(self.options["batch_candidates"]), int(budget // per_model), len(models)))
        self.sync()
        setup_s = time.perf_counter() - started
        results: List[Optional[dict]] = [None] * len(models)
        moving = [i for i, m in enumerate(models) if self._moving(m)]
        others = [i for i, m in enumerate(models) if not self._moving(m)]
        for g0 in range(0, len(moving), capacity):
            group = moving[g0:g0 + capacity]
            t0 = time.perf_counter()
            dens = [self._density(models[i], args) for i in group]
            uniq: List[MovedChainDensity] = []
            for d in dens:
                if all(d is not u for u in uniq):
                    uniq.append(d)
            model_of = [next(k for k, u in enumerate(uniq) if u is d) for d in dens]
            model_of += [model_of[0]] * (capacity - len(model_of))
            batch = self._batch(job, capacity, uniq, model_of)
            poses = [list(map(float, models[i]["pose"])) for i in group]
            if len(poses) == capacity and batch.use_graph:
                scores = batch.score_batch(poses)
            else:
                scores = batch.score_active(poses)
            texts = batch.search_texts(len(group))
            rows = self._rank_batch(ctx, job, batch, len(group), keep) if calibrate else [None] * len(group)
            self.sync()
            search_s = (time.perf_counter() - t0) / len(group)
            for k, i in enumerate(group):
                results[i] = dict(score=float(scores[k]), orientation_rows=rows[k], search_text=texts[k],
                                  metrics=self._metrics(setup_s / len(models), search_s, len(group), job))
        for i in others:
            t0 = time.perf_counter()
            kwargs = {k: v for k, v in models[i].items() if k != "device"}
            volume = generate_volume(device=self.device, **kwargs)
            score = job.score_volume(volume)
            text = job.search_text()
            rows = self._rank_single(ctx, job, keep) if calibrate else None
            search_s = time.perf_counter() - t0
            results[i] = dict(score=float(score), orientation_rows=rows, search_text=text,
                              metrics=self._metrics(setup_s / len(models), search_s, 1, job))
        return results  # type: ignore[return-value]

    def _metrics(self, setup_s: float, search_s: float, batch: int, job: ScoringJob) -> dict:
        return dict(setup_s=setup_s, search_s=search_s, execution_s=setup_s + search_s, batch_candidates=batch,
                    template_directions=len(job.needed), particles=len(job.records),
                    precision=self.options["precision"] if batch > 1 else "fp32")

    @staticmethod
    def _rows(ctx, job: ScoringJob, dir_peaks: np.ndarray, keep: int) -> Dict[str, dict]:
        ptr = job.local_ptr.cpu().numpy()
        rows = {}
        for i, rec in enumerate(job.records):
            a, b = int(ptr[i]), int(ptr[i + 1])
            if b <= a:
                rows[str(rec.line_index)] = dict(image=rec.image_name, directions=[])
                continue
            rows[str(rec.line_index)] = ranked_row(rec, job.local[i], ctx.angles, dir_peaks[a:b], keep)
        return rows

    def _rank_batch(self, ctx, job, batch: BatchScoringJob, k: int, keep: int) -> List[Dict[str, dict]]:
        m = max(1, job.nnz)
        peaks = batch.score_buf[:k].view(k, m, job.n_psi).amax(dim=2).cpu().numpy()
        return [self._rows(ctx, job, peaks[c], keep) for c in range(k)]

    def _rank_single(self, ctx, job: ScoringJob, keep: int) -> Dict[str, dict]:
        m = max(1, job.nnz)
        peaks = job.score_buf.view(m, job.n_psi).amax(dim=1).cpu().numpy()
        return self._rows(ctx, job, peaks, keep)

