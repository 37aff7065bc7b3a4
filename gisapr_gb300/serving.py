"""Request loop for candidate evaluations from concurrent refinement drivers.

The reference serves candidates from a worker process per GPU that handles
one request at a time under a lock (R/gisapr_runtime.py:44,95;
ZL/gisapr_worker_v2.py:120-178) and re-reads or caches the particle stack
per job. Here one process keeps every admitted job's particle spectra, CTF
and whitening tables resident on the device and schedules requests
continuously:

* jobs are registered with a factory and an HBM footprint estimate and are
  admitted, in order, while the sum of admitted footprints stays under the
  cap (150 GB by default); a job that does not fit waits for retired jobs;
* requests (one job, 1..n poses) are queued per job; a worker thread that
  picks a job takes all its pending poses up to the batch size and scores
  them in one batched launch sequence, so requests that arrive while other
  work is on the device join the next batch of their job;
* several workers, each with its own CUDA stream and native context (FFT
  plans and scratch are per context), run different jobs at the same time,
  so their kernels overlap on the GPU; a job runs on one worker at a time;
* each request's latency (submission to scores on the host) is recorded;
* a batch that runs out of device memory fails its requests with a
  RuntimeError and releases the job's resident data (rebuilt by its next
  request), and the server keeps serving, as the Lite tree's worker turns
  a CUDA out-of-memory error into a recoverable request error
  (ZL/gisapr_worker_v2.py:131-139).

A candidate's score does not depend on which other candidates share its
batch (every kernel computes a slot from that slot's inputs only, with a
fixed reduction order), so a request's result is the same alone and in the
mix; tests/test_gpu_serving.py checks that bitwise.
"""
from __future__ import annotations

import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Callable, Deque, Dict, List, Optional

import numpy as np

__all__ = ["ScoringServer", "ServerStats", "job_footprint_bytes", "projector_scratch_bytes"]


# A library context grows a scratch buffer to at least twice its size when
# a call needs more, and keeps the buffers it replaced (CUDA graphs captured
# earlier may still name them): for the largest request R a context has
# seen, the live buffer is below 2 R and the replaced ones together below the
# live one, so the context holds less than 4 R of that kind of buffer.
CONTEXT_GROWTH_BOUND = 4


def projector_scratch_bytes(box: int, new_box: int, n_dirs: int, sm_count: int = 152) -> int:
    """Upper bound of the device memory a library context holds for
    projector calls of up to ``n_dirs`` templates at ``box``: the blocked
    spectrum copy and the pass-A planes (powers of two; at box 256 at most
    4,096 planes of 256 x 257), and the general projector's per-CTA scratch
    planes (boxes 96, 192, 256; 6, 3 and 2 CTAs per SM), each times
    CONTEXT_GROWTH_BOUND (buffers grown by later, larger calls keep their
    predecessors). Each host thread's context is shared by the jobs that
    thread runs."""
    n, h = int(box), new_box // 2 + 1
    pow2 = n & (n - 1) == 0
    out = 0
    if pow2:
        out += 4 * n * n * ((n + 2) // 2 * 2) * 8            # blocked spectrum
    if pow2 and n <= 128:
        ld = {32: 38, 64: 74, 128: 150}[n]
        out += n_dirs * n * ld * 8                            # pass-A planes
    else:
        if n == 256:
            out += min(n_dirs, 4096) * n * (n + 1) * 8        # pass-A planes
        per_sm = {96: 6, 192: 3}.get(n, 2)
        out += min(n_dirs, sm_count * per_sm) * (n * (n + 1) + new_box * h) * 8
    return int(CONTEXT_GROWTH_BOUND * out)


def job_footprint_bytes(box: int, new_box: int, n_particles: int, n_psi: int, n_dirs: int, max_batch: int,
                        precision: str = "fp32", local_dirs: int = 64, contexts: int = 2) -> int:
    """Upper bound of a job's device memory: resident particle spectra and
    tables, the per-candidate volume buffers, the padded FFT input and the
    volume spectrum of every native context that runs the job (``contexts``:
    the server's workers plus the extra template lanes of a batch; at boxes
    96 and 192 the projector keeps one spectrum per context), the batch's
    template banks (every model direction counted as needed), its per-map
    outputs (``local_dirs`` directions per particle at most) and the
    projector scratch of a library context (counted once for every job,
    although a context is per host thread and shared by that thread's jobs)."""
    h = new_box // 2 + 1
    spectra = n_particles * n_psi * new_box * h * 8
    tables = n_particles * (new_box * h * 4 + 64) + n_dirs * 64 + 8 * new_box * h * 4
    volume = max(1, int(contexts)) * ((2 * box) ** 3 * 4 + (2 * box) ** 2 * (box + 1) * 8) + box ** 3 * 4 * 2
    banks = max_batch * n_dirs * new_box * h * 8
    if precision != "fp32":
        banks += min(max_batch, 128) * n_dirs * new_box * h * 8
    maps = max_batch * n_particles * min(local_dirs, n_dirs) * n_psi * 12
    records = max_batch * n_particles * 24 + max_batch * 16
    return int(spectra + tables + volume + banks + maps + records + projector_scratch_bytes(box, new_box, n_dirs))


@dataclass
class _Request:
    poses: np.ndarray
    future: Future
    t_submit: float


@dataclass
class _Job:
    job_id: str
    factory: Callable
    footprint: int
    precision: str
    admitted: bool = False
    retiring: bool = False
    busy: bool = False
    job: object = None
    batch: object = None
    pending: Deque[_Request] = field(default_factory=deque)


@dataclass
class ServerStats:
    requests: int
    candidates: int
    wall_s: float
    latency_ms_p50: float
    latency_ms_p99: float
    batches: int
    mean_batch: float
    deferred_admissions: int = 0   # registrations that waited for memory to be freed
    peak_in_use: int = 0           # largest sum of admitted footprints (bytes)
    out_of_memory: int = 0         # batches that ran out of device memory (requests failed, job released)

    @property
    def candidates_per_s(self) -> float:
        return self.candidates / self.wall_s if self.wall_s > 0 else 0.0


class ScoringServer:
    """In-process continuous-batching server for candidate evaluations.

    ``register(job_id, factory, footprint)`` queues a job for admission;
    ``factory()`` (called on a worker thread once the job is admitted) must
    return a ``engine.ScoringJob``. ``submit(job_id, poses)`` returns a
    Future resolving to the scores (float64, one per pose) in pose order.
    """

    def __init__(self, device="cuda:0", hbm_cap_bytes: float = 150e9, max_batch: int = 64, n_workers: int = 2,
                 precision: str = "fp32"):
        import torch
        self.device = torch.device(device)
        if precision not in ("fp32", "fp16x3", "fp16", "bf16x3", "bf16"):
            raise ValueError(f"precision must be fp32, fp16x3, fp16, bf16x3 or bf16, got {precision!r}")
        self.cap = int(hbm_cap_bytes)
        self.max_batch = int(max_batch)
        self.precision = precision
        self._lock = threading.Condition()
        self._jobs: Dict[str, _Job] = {}
        self._order: List[str] = []
        self._in_use = 0
        self._closed = False
        self._latencies: List[float] = []
        self._candidates = 0
        self._batches = 0
        self._t0: Optional[float] = None
        self._t_last = 0.0
        self._errors: List[BaseException] = []
        self._deferred = 0
        self._peak_in_use = 0
        self._oom = 0
        self._workers = [threading.Thread(target=self._work, name=f"gisapr-serve-{i}", daemon=True)
                         for i in range(int(n_workers))]
        for w in self._workers:
            w.start()

    # ------------------------------------------------------------------ API
    def register(self, job_id: str, factory: Callable, footprint_bytes: int) -> None:
        with self._lock:
            if job_id in self._jobs:
                raise ValueError(f"job {job_id!r} is already registered")
            if footprint_bytes > self.cap:
                raise ValueError(f"job {job_id!r} needs {footprint_bytes / 1e9:.1f} GB, above the "
                                 f"{self.cap / 1e9:.1f} GB cap")
            self._jobs[job_id] = _Job(job_id, factory, int(footprint_bytes), self.precision)
            self._order.append(job_id)
            self._admit_locked()
            if not self._jobs[job_id].admitted:
                self._deferred += 1
            self._lock.notify_all()

    def retire(self, job_id: str) -> None:
        """Free the job's memory once its queued requests are done. A job
        not yet admitted keeps its place in the admission order while it
        has queued requests (they still run) and is dropped once it has
        none; new requests for a retiring job are refused."""
        with self._lock:
            j = self._jobs.get(job_id)
            if j is None:
                raise ValueError(f"job {job_id!r} is not registered")
            j.retiring = True
            self._maybe_free_locked(j)
            self._lock.notify_all()

    def submit(self, job_id: str, poses) -> Future:
        poses = np.asarray(poses, dtype=np.float64).reshape(-1, 6)
        if len(poses) == 0:
            raise ValueError("a request needs at least one pose")
        fut: Future = Future()
        with self._lock:
            if self._closed:
                raise RuntimeError("server is closed")
            j = self._jobs.get(job_id)
            if j is None or j.retiring:
                raise ValueError(f"job {job_id!r} is not registered")
            now = time.perf_counter()
            if self._t0 is None:
                self._t0 = now
            # requests larger than a batch are split into batch-sized parts
            parts = [poses[i:i + self.max_batch] for i in range(0, len(poses), self.max_batch)]
            if len(parts) == 1:
                j.pending.append(_Request(parts[0], fut, now))
            else:
                subs = [Future() for _ in parts]
                for p, f in zip(parts, subs):
                    j.pending.append(_Request(p, f, now))
                _join_futures(subs, fut)
            self._lock.notify_all()
        return fut

    def is_admitted(self, job_id: str) -> bool:
        with self._lock:
            return self._jobs[job_id].admitted

    def memory_in_use(self) -> int:
        with self._lock:
            return self._in_use

    def drain(self, timeout: Optional[float] = None) -> None:
        """Wait until every queued request is done."""
        end = None if timeout is None else time.perf_counter() + timeout
        with self._lock:
            while any(j.pending or j.busy for j in self._jobs.values()):
                left = None if end is None else end - time.perf_counter()
                if left is not None and left <= 0:
                    raise TimeoutError("requests still queued")
                self._lock.wait(left)
            if self._errors:
                raise self._errors[0]

    def stats(self) -> ServerStats:
        with self._lock:
            lat = np.asarray(self._latencies) * 1e3
            wall = (self._t_last - self._t0) if self._t0 is not None else 0.0
            return ServerStats(requests=len(lat), candidates=self._candidates, wall_s=wall,
                               latency_ms_p50=float(np.percentile(lat, 50)) if len(lat) else 0.0,
                               latency_ms_p99=float(np.percentile(lat, 99)) if len(lat) else 0.0,
                               batches=self._batches,
                               mean_batch=self._candidates / self._batches if self._batches else 0.0,
                               deferred_admissions=self._deferred, peak_in_use=self._peak_in_use,
                               out_of_memory=self._oom)

    def reset_stats(self) -> None:
        with self._lock:
            self._latencies.clear()
            self._candidates = 0
            self._batches = 0
            self._t0 = None

    def close(self) -> None:
        """Stop accepting requests, let the workers finish what admitted jobs
        have queued, then fail the requests of jobs never admitted."""
        with self._lock:
            self._closed = True
            self._lock.notify_all()
        for w in self._workers:
            w.join()
        with self._lock:
            for j in self._jobs.values():
                while j.pending:
                    r = j.pending.popleft()
                    if not r.future.done():
                        r.future.set_exception(RuntimeError(f"server closed before job {j.job_id!r} was admitted"))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ internals
    def _admit_locked(self) -> None:
        for jid in self._order:
            j = self._jobs[jid]
            if j.admitted:
                continue
            if self._in_use + j.footprint > self.cap:
                break  # admission in registration order
            j.admitted = True
            self._in_use += j.footprint
            self._peak_in_use = max(self._peak_in_use, self._in_use)

    def _maybe_free_locked(self, j: _Job) -> None:
        """Drop a retiring job with no queued or running work (releasing its
        memory if it was admitted) and admit the jobs waiting behind it."""
        if self._jobs.get(j.job_id) is not j or not j.retiring or j.pending or j.busy:
            return
        if j.admitted:
            j.job = None
            j.batch = None
            j.admitted = False
            self._in_use -= j.footprint
        self._order.remove(j.job_id)
        del self._jobs[j.job_id]
        self._admit_locked()

    def _next_locked(self) -> Optional[_Job]:
        best = None
        for jid in self._order:
            j = self._jobs[jid]
            if j.admitted and not j.busy and j.pending:
                if best is None or j.pending[0].t_submit < best.pending[0].t_submit:
                    best = j
        return best

    def _make_stream(self):
        import torch
        torch.cuda.set_device(self.device)
        return torch.cuda.Stream(self.device)

    def _work(self) -> None:
        stream = self._make_stream()
        while True:
            with self._lock:
                j = self._next_locked()
                while j is None and not self._closed:
                    self._lock.wait()
                    j = self._next_locked()
                if j is None:
                    return
                j.busy = True
                reqs: List[_Request] = []
                n = 0
                while j.pending and n + len(j.pending[0].poses) <= self.max_batch:
                    r = j.pending.popleft()
                    reqs.append(r)
                    n += len(r.poses)
            try:
                scores = self._run(j, np.concatenate([r.poses for r in reqs]), stream)
                done = time.perf_counter()
                off = 0
                for r in reqs:
                    k = len(r.poses)
                    r.future.set_result(scores[off:off + k])
                    off += k
                with self._lock:
                    for r in reqs:
                        self._latencies.append(done - r.t_submit)
                    self._candidates += n
                    self._batches += 1
                    self._t_last = max(self._t_last, done)
            except BaseException as e:  # noqa: BLE001 - reported through the futures
                if _is_out_of_memory(e):
                    # recoverable: release what the job holds on the device and
                    # fail only this batch; the job is rebuilt by its next request
                    err = RuntimeError(f"job {j.job_id!r}: the batch ran out of device memory; its requests "
                                       f"failed and the job's device data was released (it is rebuilt on the "
                                       f"next request). Lower max_batch or the HBM cap.")
                    err.__cause__ = e
                    j.job = None
                    j.batch = None
                    self._release_device_memory()
                    for r in reqs:
                        if not r.future.done():
                            r.future.set_exception(err)
                    with self._lock:
                        self._oom += 1
                else:
                    for r in reqs:
                        if not r.future.done():
                            r.future.set_exception(e)
                    with self._lock:
                        self._errors.append(e)
            finally:
                with self._lock:
                    j.busy = False
                    self._maybe_free_locked(j)
                    self._lock.notify_all()

    def _release_device_memory(self) -> None:
        import torch
        if torch.cuda.is_available():
            torch.cuda.empty_cache()

    def _run(self, j: _Job, poses: np.ndarray, stream) -> np.ndarray:
        import torch
        from .engine import BatchScoringJob
        with torch.cuda.stream(stream):
            if j.job is None:
                j.job = j.factory()
                j.batch = BatchScoringJob(j.job, self.max_batch, use_graph=False, precision=j.precision)
        return j.batch.score_active(list(poses), stream=stream)


def _is_out_of_memory(e: BaseException) -> bool:
    """A CUDA out-of-memory error from torch's allocator or from the
    library's own cudaMalloc (reported as RuntimeError naming it)."""
    try:
        import torch
        if isinstance(e, torch.cuda.OutOfMemoryError):
            return True
    except ImportError:  # pragma: no cover - torch is always present
        pass
    return isinstance(e, RuntimeError) and "out of memory" in str(e).lower()


def _join_futures(parts: List[Future], out: Future) -> None:
    """Resolve ``out`` with the concatenation of ``parts`` once all are done."""
    lock = threading.Lock()
    remaining = [len(parts)]

    def one_done(_):
        with lock:
            remaining[0] -= 1
            last = remaining[0] == 0
        if last and not out.done():
            errs = [p.exception() for p in parts if p.exception() is not None]
            if errs:
                out.set_exception(errs[0])
            else:
                out.set_result(np.concatenate([p.result() for p in parts]))

    for p in parts:
        p.add_done_callback(one_done)
