"""Scheduling and admission of the request loop, with a fake executor (CPU)."""
import threading
import time

import numpy as np
import pytest

from gisapr_gb300.serving import ScoringServer, job_footprint_bytes


class FakeServer(ScoringServer):
    """Scores are a pure function of (job, pose); each batch takes a few ms."""

    def __init__(self, *a, delay=0.003, **k):
        self.delay = delay
        self.ran = []  # (job_id, n) per batch
        self.built = []
        self.lock2 = threading.Lock()
        super().__init__(*a, device="cpu", **k)

    def _make_stream(self):
        return None

    def _run(self, j, poses, stream):
        if j.job is None:
            j.job = j.factory()
            with self.lock2:
                self.built.append(j.job_id)
        time.sleep(self.delay)
        with self.lock2:
            self.ran.append((j.job_id, len(poses)))
        return poses.sum(axis=1) * j.job


def poses_of(seed, n):
    return np.random.default_rng(seed).normal(size=(n, 6))


def test_results_follow_requests_and_batches_merge():
    with FakeServer(max_batch=16, n_workers=1, delay=0.02) as srv:
        srv.register("a", lambda: 2.0, 10)
        srv.register("b", lambda: 3.0, 10)
        reqs = [(("a", "b")[i % 2], poses_of(i, 1 + i % 5)) for i in range(24)]
        futs = [srv.submit(j, p) for j, p in reqs]
        srv.drain(timeout=30)
        for (j, p), f in zip(reqs, futs):
            np.testing.assert_array_equal(f.result(), p.sum(axis=1) * (2.0 if j == "a" else 3.0))
        st = srv.stats()
        assert st.requests == 24 and st.candidates == sum(len(p) for _, p in reqs)
        assert st.batches < 24  # requests queued behind a running batch share the next one
        assert all(n <= 16 for _, n in srv.ran)
        assert st.latency_ms_p99 >= st.latency_ms_p50 > 0


def test_large_request_is_split_and_joined():
    with FakeServer(max_batch=8, n_workers=2) as srv:
        srv.register("a", lambda: 1.5, 10)
        p = poses_of(3, 21)
        f = srv.submit("a", p)
        np.testing.assert_array_equal(f.result(timeout=30), p.sum(axis=1) * 1.5)
        assert sorted(n for _, n in srv.ran) == [5, 8, 8]


def test_admission_by_footprint_waits_for_retired_jobs():
    with FakeServer(hbm_cap_bytes=100, max_batch=8, n_workers=2) as srv:
        srv.register("a", lambda: 1.0, 60)
        srv.register("b", lambda: 2.0, 60)  # does not fit next to a
        srv.register("c", lambda: 3.0, 30)  # fits, but admission keeps registration order
        assert srv.is_admitted("a") and not srv.is_admitted("b") and not srv.is_admitted("c")
        assert srv.memory_in_use() == 60
        fa = srv.submit("a", poses_of(1, 3))
        fb = srv.submit("b", poses_of(2, 3))
        fa.result(timeout=30)
        time.sleep(0.05)
        assert not fb.done()  # b is queued until a retires
        srv.retire("a")
        np.testing.assert_array_equal(fb.result(timeout=30), poses_of(2, 3).sum(axis=1) * 2.0)
        assert srv.is_admitted("b") and srv.is_admitted("c")
        assert srv.memory_in_use() == 90
        assert srv.built == ["a", "b"]


def test_concurrent_drivers_and_errors():
    with FakeServer(max_batch=32, n_workers=3, delay=0.001) as srv:
        for k in range(4):
            srv.register(f"j{k}", (lambda k=k: float(k + 1)), 1)
        out = {}

        def driver(d):
            for i in range(15):
                jid = f"j{(d + i) % 4}"
                p = poses_of(100 * d + i, 1 + (i % 7))
                out[(d, i)] = (jid, p, srv.submit(jid, p))

        threads = [threading.Thread(target=driver, args=(d,)) for d in range(5)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        srv.drain(timeout=30)
        for jid, p, f in out.values():
            np.testing.assert_array_equal(f.result(), p.sum(axis=1) * float(int(jid[1:]) + 1))
        with pytest.raises(ValueError):
            srv.submit("missing", poses_of(0, 1))
        with pytest.raises(ValueError):
            srv.submit("j0", np.zeros((0, 6)))
        with pytest.raises(ValueError):
            srv.register("huge", lambda: 1.0, 10 ** 15)


def test_footprint_estimate_counts_spectra_and_banks():
    base = job_footprint_bytes(128, 128, 5000, 3, 768, 64)
    assert base > 5000 * 3 * 128 * 65 * 8 + 64 * 768 * 128 * 65 * 8
    assert job_footprint_bytes(128, 128, 5000, 3, 768, 64, precision="fp16x3") > base
    assert job_footprint_bytes(128, 128, 10000, 3, 768, 64) > base


def test_footprint_counts_one_spectrum_per_context():
    """Every native context that runs a job (the server's workers and a
    batch's extra template lanes) holds its own padded FFT input and volume
    spectrum of the job's box."""
    per_context = (2 * 96) ** 3 * 4 + (2 * 96) ** 2 * 97 * 8
    one = job_footprint_bytes(96, 96, 2000, 3, 768, 64, contexts=1)
    assert job_footprint_bytes(96, 96, 2000, 3, 768, 64, contexts=4) - one == 3 * per_context
    assert job_footprint_bytes(96, 96, 2000, 3, 768, 64) - one == per_context  # default: two template lanes


def test_footprint_counts_projector_scratch():
    from gisapr_gb300.serving import CONTEXT_GROWTH_BOUND as G, projector_scratch_bytes
    # a context's buffers grow by doubling and keep their predecessors: the
    # bound is four times the request
    assert G == 4
    # box 128: blocked spectrum (256 x 256 x 130 complex) + 768 planes of 128 x 150
    assert projector_scratch_bytes(128, 128, 768) == G * (4 * 128 * 128 * 130 * 8 + 768 * 128 * 150 * 8)
    # box 256: blocked spectrum, at most 4,096 flat planes, 304 CTA scratch planes
    small = projector_scratch_bytes(256, 256, 3072)
    assert small == G * (4 * 256 * 256 * 258 * 8 + 3072 * 256 * 257 * 8 + 304 * (256 * 257 + 256 * 129) * 8)
    assert projector_scratch_bytes(256, 256, 20000) == projector_scratch_bytes(256, 256, 4096)
    # boxes 96 and 192: general-kernel scratch only
    assert projector_scratch_bytes(96, 96, 10) == G * 10 * (96 * 97 + 96 * 49) * 8
    assert projector_scratch_bytes(192, 192, 10000) == G * 456 * (192 * 193 + 192 * 97) * 8
    assert job_footprint_bytes(256, 256, 4000, 3, 3072, 8) - small > 0


def test_out_of_memory_fails_the_batch_and_releases_the_job():
    """A batch that runs out of device memory fails its own requests with a
    recoverable error, the job's device data is dropped and rebuilt by the
    next request, and the server keeps serving (the Lite worker's OOM path)."""
    import torch

    class OomOnce(FakeServer):
        def __init__(self, *a, **k):
            self.boom = True
            self.released = 0
            super().__init__(*a, **k)

        def _release_device_memory(self):
            self.released += 1

        def _run(self, j, poses, stream):
            if j.job is None:
                j.job = j.factory()
                with self.lock2:
                    self.built.append(j.job_id)
            if self.boom:
                self.boom = False
                raise torch.cuda.OutOfMemoryError("CUDA out of memory. Tried to allocate 2.00 GiB")
            return poses.sum(axis=1) * j.job

    with OomOnce(max_batch=8, n_workers=1) as srv:
        srv.register("a", lambda: 2.0, 10)
        f1 = srv.submit("a", poses_of(1, 3))
        with pytest.raises(RuntimeError, match="ran out of device memory"):
            f1.result(timeout=30)
        p = poses_of(2, 4)
        np.testing.assert_array_equal(srv.submit("a", p).result(timeout=30), p.sum(axis=1) * 2.0)
        srv.drain(timeout=30)  # no unrecoverable error recorded
        st = srv.stats()
        assert st.out_of_memory == 1 and srv.released == 1
        assert srv.built == ["a", "a"]  # the job was rebuilt after the failure


def test_library_allocation_failure_counts_as_out_of_memory():
    from gisapr_gb300.serving import _is_out_of_memory
    assert _is_out_of_memory(RuntimeError("cudaMalloc(planes): out of memory"))
    assert not _is_out_of_memory(RuntimeError("tensor-core correlation: an on-chip barrier wait ran out"))
    assert not _is_out_of_memory(ValueError("out of memory"))


def test_deferred_admissions_and_peak_memory_are_counted():
    with FakeServer(hbm_cap_bytes=100, max_batch=8, n_workers=1) as srv:
        srv.register("a", lambda: 1.0, 70)
        srv.register("b", lambda: 2.0, 50)   # deferred
        srv.register("c", lambda: 3.0, 20)   # deferred behind b (registration order)
        st = srv.stats()
        assert st.deferred_admissions == 2 and st.peak_in_use == 70
        srv.submit("a", poses_of(1, 2)).result(timeout=30)
        srv.retire("a")
        srv.submit("b", poses_of(2, 2)).result(timeout=30)
        assert srv.stats().peak_in_use == 70


def test_retiring_a_deferred_job_still_serves_its_queued_requests():
    """A job retired before admission keeps its place while it has queued
    requests: they run once memory frees up, then the job is dropped and
    its id can be registered again; a deferred job retired with nothing
    queued is dropped at once."""
    with FakeServer(hbm_cap_bytes=100, max_batch=8, n_workers=1) as srv:
        srv.register("a", lambda: 1.0, 70)
        srv.register("b", lambda: 2.0, 50)   # deferred
        srv.register("c", lambda: 3.0, 40)   # deferred behind b
        fb = srv.submit("b", poses_of(5, 3))
        srv.retire("b")
        with pytest.raises(ValueError):
            srv.submit("b", poses_of(6, 1))  # retiring: no new requests
        srv.retire("c")                      # nothing queued: dropped now
        assert srv.memory_in_use() == 70
        srv.register("c", lambda: 4.0, 40)   # the id is free again
        srv.submit("a", poses_of(1, 2)).result(timeout=30)
        srv.retire("a")
        np.testing.assert_array_equal(fb.result(timeout=30), poses_of(5, 3).sum(axis=1) * 2.0)
        srv.drain(timeout=30)
        assert srv.is_admitted("c") and srv.memory_in_use() == 40
        assert srv.built == ["a", "b"]
        with pytest.raises(ValueError):
            srv.retire("b")                  # already gone


def test_close_fails_requests_of_jobs_never_admitted():
    srv = FakeServer(hbm_cap_bytes=100, max_batch=8, n_workers=1)
    srv.register("a", lambda: 1.0, 70)
    srv.register("b", lambda: 2.0, 50)   # never admitted: a is not retired
    fa = srv.submit("a", poses_of(1, 2))
    fb = srv.submit("b", poses_of(2, 2))
    srv.close()
    np.testing.assert_array_equal(fa.result(timeout=30), poses_of(1, 2).sum(axis=1))
    with pytest.raises(RuntimeError, match="closed"):
        fb.result(timeout=30)
