"""ctypes binding of libgisapr_gb300.so (the C ABI in include/gisapr_gb300.h).

The library is built in-tree by ``gisapr_gb300.build_native``. There is no
fallback: if the library cannot be loaded, every scoring call raises
RuntimeError naming the missing file.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_native" / "libgisapr_gb300.so"

OK, ERR_ARGUMENT, ERR_CUDA, ERR_CUFFT, ERR_UNSUPPORTED = 0, 1, 2, 3, 4

_p, _i, _d, _f = C.c_void_p, C.c_int, C.c_double, C.c_float

# name -> argtypes (every function returns int except gisapr_last_error)
SIGNATURES = {
    "gisapr_abi_version": [],
    "gisapr_context_create": [_i, C.POINTER(_p)],
    "gisapr_context_destroy": [_p],
    "gisapr_deposit": [_p, _p, _p, _p, _i, _p, _i, _i, _d, _d, _d],
    "gisapr_deposit_noalloc": [_p, _p, _p, _i, _p, _i, _i, _d, _d, _d],
    "gisapr_deposit_moved": [_p, _p, _p, _p, _i, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _d],
    "gisapr_volume_spectrum": [_p, _p, _p, _i, _p],
    "gisapr_volume_spectrum_blocked": [_p, _p, _p, _i],
    "gisapr_project_templates": [_p, _p, _p, _i, _p, _p, _i, _p, _p, _p, _i, _p],
    "gisapr_packed_ctf": [_p, _p, _p, _p, _i, _p, _p, _p, _p, _i, _f, _f, _f, _f, _f, _p],
    "gisapr_prepare_particles": [_p, _p, _p, _i, _i, _p, _p, _p, _p, _i, _i, _p],
    "gisapr_correlate": [_p, _p, _p, _p, _p, _p, _i, _i, _i, _i, _p, _p, _p],
    "gisapr_particle_results": [_p, _p, _p, _p, _p, _i, _i, _p, _p, _p, _p, _p, _p],
    "gisapr_score_sum": [_p, _p, _p, _i, _p],
    "gisapr_correlate_batch": [_p, _p, _p, C.c_longlong, _i, _p, _p, _p, _i, _i, _i, _i, _i, _p, _p, _p],
    "gisapr_particle_results_batch": [_p, _p, _p, _p, _p, _i, _i, _i, _p, _p, _p, _p, _p, _p],
    "gisapr_score_sum_batch": [_p, _p, _p, _i, _i, _p],
    "gisapr_correlate_batch_subset": [_p, _p, _p, C.c_longlong, _i, _p, _p, _p, _i, _i, _i, _i, _i, _p, _p, _p,
                                      _p],
    "gisapr_particle_results_subset": [_p, _p, _p, _p, _p, _i, _i, _i, _p, _p, _p, _p, _p, _p, _p],
    "gisapr_score_sum_subset": [_p, _p, _p, _i, _i, _p, _p],
    "gisapr_tc_bank_bytes": [_i, _i],
    "gisapr_project_launches": [_i, _i],
    "gisapr_projector_status": [_p, _p, _p],
    "gisapr_set_projector_wait": [_p, C.c_longlong],
    "gisapr_set_tuning": [_p, _i, _i, _i],
    "gisapr_get_tuning": [_p, _i, _i, _p],
    "gisapr_tc_plan_work": [_p, _p, _i, _i, _i, _i, _p, _i, _p],
    "gisapr_correlate_tc_batch": [_p, _p, _p, C.c_longlong, _i, _i, _p, _p, _p, _p, _p, _i, _i, _i, _i, _i, _i,
                                  _p, _p, _p, _p],
    "gisapr_correlate_tc_batch_ex": [_p, _p, _p, C.c_longlong, _i, _i, _p, _p, _p, _p, _p, _i, _i, _i, _i, _i, _i,
                                     _p, _p, C.c_uint, _p, _p, _p, _p],
    "gisapr_restraint_edt": [_p, _p, _p, _i, _f, _p, _p, _p],
    "gisapr_ingest_stack": [_p, _p, _p, _i, _i, _i, _p, _i, _i, _i, _p, _p, _p, _i, _p, _p, _p],
    "gisapr_restraint_init": [_p, _p, _i],
    "gisapr_restraint_eval": [_p, _p, _p, _p, _p, _i, _p, _f, _p],
}

# functions that return something other than an int status (gisapr_project_launches
# returns a count)
RESTYPES = {"gisapr_tc_bank_bytes": C.c_longlong}

_lib = None
_lock = threading.Lock()


def load():
    """Load the native library once; raise RuntimeError if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"GisAPR GB300 native library not built: {LIB_PATH} is missing "
                "(run `python -m gisapr_gb300.build_native`); there is no CPU fallback")
        lib = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | os.RTLD_GLOBAL)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = RESTYPES.get(name, C.c_int)
        lib.gisapr_last_error.argtypes = []
        lib.gisapr_last_error.restype = C.c_char_p
        _lib = lib
        return lib


def check(code: int, what: str) -> None:
    """Map an ABI status to the reference's exception types."""
    if code == OK:
        return
    msg = load().gisapr_last_error().decode(errors="replace")
    if code in (ERR_ARGUMENT, ERR_UNSUPPORTED):
        raise ValueError(f"{what}: {msg}")
    raise RuntimeError(f"{what}: {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def ptr(t) -> C.c_void_p:
    """Device (or host) address of a tensor, or NULL for None."""
    if t is None:
        return C.c_void_p(None)
    return C.c_void_p(t.data_ptr())


def stream_of(device) -> C.c_void_p:
    import torch
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


TUNE_CORR_CLUSTER = 1  # gisapr_set_tuning keys (include/gisapr_gb300.h)
TUNE_TC_A_STAGES = 2
TUNE_TC_B_STAGES = 3

# Process-wide launch-shape settings, (key, size) -> value, applied to every
# native context at creation (and to this thread's contexts when changed);
# set by the autotuner.
DEFAULT_TUNING: dict = {}


_TUNING_VERSION = [0]


def tuning_version() -> int:
    """Changes whenever set_default_tuning does (captured launch sequences
    taken before then use the old launch shapes and must be re-captured)."""
    return _TUNING_VERSION[0]


def set_default_tuning(key: int, size: int, value: int) -> None:
    DEFAULT_TUNING[(int(key), int(size))] = int(value)
    _TUNING_VERSION[0] += 1
    cache = getattr(Context._per_thread, "ctx", None) or {}
    for ctx in cache.values():
        call("gisapr_set_tuning", ctx.handle, int(key), int(size), int(value))


class Context:
    """Per-device native context (plans, tables, scratch). One per thread."""

    _per_thread = threading.local()

    def __init__(self, device_index: int):
        self.device_index = int(device_index)
        h = C.c_void_p()
        call("gisapr_context_create", self.device_index, C.byref(h))
        self.handle = h
        for (key, size), value in DEFAULT_TUNING.items():
            call("gisapr_set_tuning", h, key, size, value)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib is not None:
            try:
                _lib.gisapr_context_destroy(h)
            except Exception:
                pass
            self.handle = None

    @classmethod
    @contextlib.contextmanager
    def using(cls, ctx: "Context"):
        """Make ``ctx`` this thread's context for its device inside the block
        (a batch runs independent candidates on several contexts, each with
        its own scratch, on several streams)."""
        cls.for_device(f"cuda:{ctx.device_index}")  # the thread's own context exists
        cache = cls._per_thread.ctx
        prev = cache[ctx.device_index]
        cache[ctx.device_index] = ctx
        try:
            yield ctx
        finally:
            cache[ctx.device_index] = prev

    @classmethod
    def for_device(cls, device) -> "Context":
        import torch
        dev = torch.device(device)
        if dev.type != "cuda":
            raise ValueError(f"GisAPR GB300 kernels run on CUDA devices only, got {dev}")
        idx = dev.index if dev.index is not None else torch.cuda.current_device()
        cache = getattr(cls._per_thread, "ctx", None)
        if cache is None:
            cache = {}
            cls._per_thread.ctx = cache
        if idx not in cache:
            cache[idx] = cls(idx)
        return cache[idx]


def c_ptr_offset(t, nbytes: int) -> C.c_void_p:
    """Address ``nbytes`` past the start of tensor ``t``."""
    return C.c_void_p(t.data_ptr() + int(nbytes))
