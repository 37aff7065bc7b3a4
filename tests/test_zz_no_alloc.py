"""gisapr_deposit_noalloc: the deposit entry point that allocates nothing.

It serves callers that cannot allocate device memory (for example a host
whose device memory belongs to another framework's pool, or code running
during stream capture). Its atom scratch is a fixed static device array, so
it must give the same density as the allocating gisapr_deposit, call after
call, and refuse atom counts above the array's size. This file is collected
last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from tests.helpers import DENSITY_RRMS, rrms  # noqa: E402

MAX_ATOMS = 65536


def _atoms(seed, n, box, apix):
    rng = np.random.default_rng(seed)
    half = box * apix / 2.0
    xyz = rng.uniform(-0.95 * half, 0.95 * half, size=(n, 3)).astype(np.float32)
    z = rng.choice(np.asarray([1, 6, 7, 8, 15, 16, 0], np.float32), size=n)
    return xyz, z


def _deposit(lib, name, xyz, z, box, apix, res, ctx=None):
    from gisapr_gb300 import _native
    from gisapr_gb300.pdb2mrc import density_parameters
    width, rp, kn = density_parameters(apix, res)
    dev = torch.device("cuda", 0)
    x = torch.from_numpy(xyz).to(dev)
    zz = torch.from_numpy(z).to(dev)
    vol = torch.zeros((box,) * 3, dtype=torch.float32, device=dev)
    st = _native.stream_of(dev)
    if name == "gisapr_deposit":
        rc = lib.gisapr_deposit(ctx, st, _native.ptr(x), _native.ptr(zz), len(z), _native.ptr(vol), box, width,
                                apix, rp, kn)
    else:
        rc = lib.gisapr_deposit_noalloc(st, _native.ptr(x), _native.ptr(zz), len(z), _native.ptr(vol), box,
                                        width, apix, rp, kn)
    assert rc == 0, lib.gisapr_last_error()
    torch.cuda.synchronize(dev)
    return vol.cpu().numpy()


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    from gisapr_gb300 import _native
    return _native.load()


def test_noalloc_matches_allocating_deposit_on_two_calls(lib):
    from gisapr_gb300 import _native
    torch.cuda.set_device(0)
    ctx = _native.Context.for_device("cuda:0").handle
    # two calls in a row with different atom sets: the second must not see
    # anything the first left in the shared array
    for seed, n, box, apix in ((1, 5000, 64, 1.5), (2, 1200, 32, 3.0)):
        xyz, z = _atoms(seed, n, box, apix)
        ref = _deposit(lib, "gisapr_deposit", xyz, z, box, apix, 2 * apix, ctx)
        got = _deposit(lib, "gisapr_deposit_noalloc", xyz, z, box, apix, 2 * apix)
        assert rrms(got, ref) < DENSITY_RRMS
        np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_more_atoms_than_its_array(lib):
    from gisapr_gb300 import _native
    dev = torch.device("cuda", 0)
    vol = torch.zeros((32,) * 3, dtype=torch.float32, device=dev)
    x = torch.zeros((MAX_ATOMS + 1, 3), dtype=torch.float32, device=dev)
    z = torch.zeros(MAX_ATOMS + 1, dtype=torch.float32, device=dev)
    rc = lib.gisapr_deposit_noalloc(_native.stream_of(dev), _native.ptr(x), _native.ptr(z), MAX_ATOMS + 1,
                                    _native.ptr(vol), 32, 6, 3.0, 2.4674, 0.7)
    assert rc == 1
    assert b"at most 65536 atoms" in lib.gisapr_last_error()
    assert float(vol.abs().sum()) == 0.0
