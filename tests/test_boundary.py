"""CPU tests of the C-ABI boundary: the library builds for sm_103a, loads, and exports every symbol that
include/libkriging_gb300.h declares.  No compute call is made here (there is no GPU on this machine)."""
import ctypes
import subprocess

import pytest

import libkriging_gb300 as lk
from libkriging_gb300 import _lib
from libkriging_gb300.build import SO, build


@pytest.fixture(scope="module")
def so():
    build()
    return SO


def test_library_exports_every_header_symbol(so):
    names = lk.header_symbols()
    assert len(names) >= 40
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_ctypes_signatures_cover_header(so):
    assert set(lk.header_symbols()) == set(_lib._SIGS)


def test_constructor_errors_follow_reference(so):
    L = lk.load()
    assert L.lkg_kriging_new(b"nosuchkernel", b"none") is None
    assert "Unsupported covariance kernel: nosuchkernel" in lk._lib.last_error()  # Covariance.cpp:230
    assert L.lkg_kriging_new(b"gauss", b"heterogeneous") is None
    h = L.lkg_kriging_new(b"matern5_2", b"nugget")
    assert h
    assert L.lkg_kriging_kernel(h) == b"matern5_2"
    assert L.lkg_kriging_noise_model(h) == b"nugget"
    L.lkg_kriging_delete(h)


def test_settings_roundtrip(so):
    L = lk.load()
    old = L.lkg_get_num_nugget()
    assert old == 1e-10  # LinearAlgebra.cpp:33
    L.lkg_set_num_nugget(1e-8)
    assert L.lkg_get_num_nugget() == 1e-8
    L.lkg_set_num_nugget(old)


def test_call_on_unfitted_model_fails_loudly(so):
    L = lk.load()
    h = L.lkg_kriging_new(b"gauss", None)
    ll = ctypes.c_double()
    th = (ctypes.c_double * 2)(0.3, 0.3)
    rc = L.lkg_kriging_log_likelihood_fun(h, th, 2, 0, 0, ctypes.byref(ll), None, None)
    assert rc == -1
    assert "fit" in lk._lib.last_error()
    L.lkg_kriging_delete(h)


def test_load_errors_follow_reference(so, tmp_path):
    """Kriging::load (Kriging.cpp:2719-2731): version 2 and content "Kriging" required, with the reference's
    messages; the file is parsed before any device work, so these run without a GPU."""
    L = lk.load()
    f = tmp_path / "m.json"
    f.write_text('{"version": 3, "content": "Kriging"}')
    assert L.lkg_kriging_load(str(f).encode()) is None
    assert "Bad version to load from '%s'; found 3, requires 2" % f in lk._lib.last_error()
    f.write_text('{"version": 2, "content": "WarpKriging"}')
    assert L.lkg_kriging_load(str(f).encode()) is None
    assert "Bad content to load from '%s'; found 'WarpKriging', requires 'Kriging'" % f in lk._lib.last_error()
    f.write_text('{"version": 2, "content": "Kriging", ')
    assert L.lkg_kriging_load(str(f).encode()) is None
    assert "JSON parse error" in lk._lib.last_error()
    assert L.lkg_kriging_load(str(tmp_path / "missing.json").encode()) is None
    assert "cannot open" in lk._lib.last_error()


def test_update_rejects_noise_like_reference(so):
    """lk_kriging_update with a noise vector calls update(y, noise, X), which requires NoiseModel Heterogeneous
    (Kriging.cpp:2639-2640)."""
    L = lk.load()
    h = L.lkg_kriging_new(b"gauss", None)
    y = (ctypes.c_double * 1)(1.0)
    x = (ctypes.c_double * 2)(0.1, 0.2)
    rc = L.lkg_kriging_update(h, y, 1, y, 1, x, 1, 2, 0)
    assert rc == -1
    assert "requires NoiseModel::Heterogeneous" in lk._lib.last_error()
    L.lkg_kriging_delete(h)
