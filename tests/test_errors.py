"""Error behaviour of the data-file boundary: the reference exits with a
message on a missing or unreadable file (e.g. SimStoppingPower.cc:20-27); the
library returns a status code and a message instead. The files are parsed
before any CUDA call, so these run without a GPU."""
import ctypes as C
import os
import shutil

import pytest

from conftest import DATA_C3


def load(dpm, path):
    L = dpm.library()
    h = C.c_void_p()
    rc = L.dpmx_tables_load(str(path).encode(), C.byref(h))
    return rc, L.dpmx_last_error().decode()


def test_missing_directory(dpm):
    import importlib
    importlib.import_module("dpm-g4cpp_gb300.builder").build_library()
    rc, msg = load(dpm, "/nonexistent/dir")
    assert rc == dpm.ERR_FILE and "mat.dat" in msg


@pytest.mark.parametrize("victim", ["el_GSDtrData.dat", "imfp_total.dat", "brem_SBDtrData.dat", "eloss_rdedx.dat"])
def test_missing_file(dpm, tmp_path, victim):
    d = tmp_path / "data"
    shutil.copytree(DATA_C3, d)
    os.remove(d / victim)
    rc, msg = load(dpm, d)
    assert rc == dpm.ERR_FILE and victim in msg


@pytest.mark.parametrize("victim", ["compton_KNDtrData.dat", "imfp_brem.dat", "mat.dat"])
def test_truncated_file(dpm, tmp_path, victim):
    d = tmp_path / "data"
    shutil.copytree(DATA_C3, d)
    text = open(d / victim).read()
    open(d / victim, "w").write(text[: len(text) // 2])
    rc, msg = load(dpm, d)
    assert rc == dpm.ERR_PARSE and victim in msg


def test_ring_selftest_rejects_bad_arguments(dpm):
    """argument checks come before any CUDA call"""
    import importlib
    importlib.import_module("dpm-g4cpp_gb300.builder").build_library()
    for kw in ({"nslots": 0}, {"nslots": 513}, {"rounds": 0}, {"blocks": 0}, {"probe_cycles": -1}):
        with pytest.raises(dpm.DpmxError):
            dpm.ring_selftest(**kw)
