"""The C ABI library builds for sm_103a, loads without a GPU and exports
every entry point include/gisapr_gb300.h declares."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "gisapr_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char\*)\s+(gisapr_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("gisapr_deposit", "gisapr_deposit_moved", "gisapr_volume_spectrum", "gisapr_project_templates",
                 "gisapr_packed_ctf", "gisapr_prepare_particles", "gisapr_correlate", "gisapr_particle_results",
                 "gisapr_score_sum", "gisapr_context_create", "gisapr_context_destroy", "gisapr_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(native_lib):
    for name in declared_functions():
        assert hasattr(native_lib, name), name


def test_binding_covers_declared_symbols(native_lib):
    from gisapr_gb300 import _native
    for name in declared_functions():
        assert name in _native.SIGNATURES or name == "gisapr_last_error", name


def test_version_and_argument_errors_without_gpu(native_lib):
    assert native_lib.gisapr_abi_version() == 100
    # argument checks return before any CUDA call
    rc = native_lib.gisapr_packed_ctf(None, None, None, None, -1, None, None, None, None, 10,
                                      C.c_float(1), C.c_float(1), C.c_float(1), C.c_float(0), C.c_float(3), None)
    assert rc == 1
    assert b"n < 0" in native_lib.gisapr_last_error()
    rc = native_lib.gisapr_correlate(None, None, None, None, None, None, 1, 3, 128, 12, None, None, None)
    assert rc == 1
    rc = native_lib.gisapr_score_sum(None, None, None, 4, None)
    assert rc == 1


def test_noalloc_deposit_rejects_non_positive_parameters_without_gpu(native_lib):
    """The no-allocation deposit checks apix, rp and kn (positive, finite)
    before it touches the device."""
    fake = C.c_void_p(16)
    for apix, rp, kn in ((0.0, 1.0, 1.0), (1.5, 0.0, 1.0), (1.5, 1.0, -2.0), (1.5, float("nan"), 1.0),
                         (1.5, 1.0, float("inf"))):
        rc = native_lib.gisapr_deposit_noalloc(None, fake, fake, 4, fake, 32, 6, C.c_double(apix), C.c_double(rp),
                                               C.c_double(kn))
        assert rc == 1
        assert b"positive and finite" in native_lib.gisapr_last_error()


def test_cpu_device_is_rejected():
    from gisapr_gb300.pdb2mrc import density_from_coords
    with pytest.raises(ValueError):
        density_from_coords([[0, 0, 0]], [6], 32, 3.0, 6.0, device="cpu")


def test_tensor_core_work_plan_on_host(native_lib):
    """gisapr_tc_plan_work is host code: every (particle, tile of 128 rows)
    appears once, tiles hold whole directions (row = direction * n_cand +
    candidate) and the list is sorted by the tile's directions
    (lexicographically), so tiles with the same directions are adjacent."""
    import numpy as np
    from gisapr_gb300 import _native
    lib = _native.load()
    rng = np.random.default_rng(3)
    counts = rng.integers(0, 9, size=40)
    ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    idx = np.concatenate([np.sort(rng.choice(50, size=c, replace=False)) for c in counts]).astype(np.int32)
    vp = lambda a: C.c_void_p(a.ctypes.data)
    for n_cand, n_psi, crop in ((1, 1, 12), (5, 3, 12), (64, 3, 12), (128, 5, 10), (48, 7, 8), (100, 2, 12),
                                (64, 3, 14), (7, 5, 14)):
        groups = -(-n_psi // (3 if crop <= 12 else 2))
        dpt = 128 // (-(-n_cand // 8) * 8)  # rows per direction rounded up to 8
        n = C.c_int(-1)
        assert lib.gisapr_tc_plan_work(vp(ptr), vp(idx), 40, n_cand, n_psi, crop, None, 0, C.byref(n)) == 0
        want = sum(-(-int(c) // dpt) for c in counts) * groups
        assert n.value == want
        work = np.zeros((max(1, want), 2), np.int32)
        assert lib.gisapr_tc_plan_work(vp(ptr), vp(idx), 40, n_cand, n_psi, crop, vp(work), want, C.byref(n)) == 0
        pairs = {(int(b), int(t)) for b, t in work[:want]}
        assert len(pairs) == want
        keys = []
        for b, t in work[:want]:
            e = int(ptr[b]) + (int(t) // groups) * dpt
            keys.append(tuple(int(v) for v in idx[e:min(e + dpt, int(ptr[b + 1]))]))
        assert keys == sorted(keys)
        if want > 1:
            assert lib.gisapr_tc_plan_work(vp(ptr), vp(idx), 40, n_cand, n_psi, crop, vp(work), want - 1,
                                           C.byref(n)) == 1
    n = C.c_int(0)
    assert lib.gisapr_tc_plan_work(vp(ptr), vp(idx), 40, 129, 3, 12, None, 0, C.byref(n)) == 1
    assert lib.gisapr_tc_plan_work(vp(ptr), vp(idx), 40, 8, 3, 16, None, 0, C.byref(n)) == 4
    assert lib.gisapr_tc_bank_bytes(760, 128) == 760 * 65 * 2 * 256 * 2


def test_projector_launch_counts_on_host(native_lib):
    """The launch count one projector call enqueues: three kernels on the
    shared-memory path, one on the general path at 96 and 192, and at 256 the
    blocked spectrum copy plus a gather and a general kernel per 4,096
    templates. The engine's gpu_launches figure is built from it."""
    lib = native_lib
    lib.gisapr_project_launches.argtypes = [C.c_int, C.c_int]
    for box in (32, 64, 128):
        assert lib.gisapr_project_launches(box, 3072) == 3
    for box in (96, 192):
        assert lib.gisapr_project_launches(box, 3072) == 1
    assert lib.gisapr_project_launches(256, 1) == 3
    assert lib.gisapr_project_launches(256, 4096) == 3
    assert lib.gisapr_project_launches(256, 4097) == 5
    assert lib.gisapr_project_launches(256, 3 * 4096 + 5) == 9
    assert lib.gisapr_project_launches(128, 0) == 0
    for bad in (16, 80, 512):
        assert lib.gisapr_project_launches(bad, 10) == -1
    from gisapr_gb300.engine import ScoringJob
    assert ScoringJob.projector_launches(256, 8192) == 5
    with pytest.raises(ValueError):
        ScoringJob.projector_launches(80, 1)


def test_projector_status_calls_check_their_arguments(native_lib):
    """The projector's status query and wait bound reject a NULL context or
    output pointer on the host."""
    from gisapr_gb300 import _native
    lib = _native.load()
    v = C.c_int(7)
    assert lib.gisapr_projector_status(None, None, C.byref(v)) == 1
    assert lib.gisapr_set_projector_wait(None, C.c_longlong(0)) == 1


def _native_signatures():
    from gisapr_gb300 import _native
    return _native.SIGNATURES


_NO_STATUS = ("gisapr_abi_version", "gisapr_tc_bank_bytes", "gisapr_project_launches", "gisapr_context_destroy")


@pytest.mark.parametrize("name", [n for n in _native_signatures() if n not in _NO_STATUS])
def test_every_entry_point_rejects_null_pointers_without_gpu(native_lib, name):
    """Every status-returning entry point, called with every pointer NULL
    (sizes 4, scalars 1), returns the argument error and a message before
    it touches the device."""
    from gisapr_gb300 import _native
    args = []
    for t in _native.SIGNATURES[name]:
        if t is C.c_void_p or (isinstance(t, type) and issubclass(t, C._Pointer)):
            args.append(None)
        elif t in (C.c_double, C.c_float):
            args.append(t(1.0))
        else:
            args.append(t(4))
    assert getattr(native_lib, name)(*args) == _native.ERR_ARGUMENT
    assert native_lib.gisapr_last_error()
