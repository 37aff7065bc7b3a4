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
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gisapr_\w+)\s*\(", text, flags=re.M)))


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


def test_cpu_device_is_rejected():
    from gisapr_gb300.pdb2mrc import density_from_coords
    with pytest.raises(ValueError):
        density_from_coords([[0, 0, 0]], [6], 32, 3.0, 6.0, device="cpu")
