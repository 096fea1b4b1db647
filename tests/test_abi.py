"""The C-ABI library loads and exports every symbol include/dpmx.h declares
(no compute calls: runs without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "dpmx.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dpmx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ["dpmx_tables_load", "dpmx_phantom_slab", "dpmx_phantom_voxels", "dpmx_run", "dpmx_simulate",
              "dpmx_write_hist", "dpmx_sampler_eval", "dpmx_influence_build", "dpmx_csr_spmv", "dpmx_csr_spmv_t"]:
        assert s in syms


def test_library_exports_every_declared_symbol(dpm):
    import importlib
    builder = importlib.import_module("dpm-g4cpp_gb300.builder")
    lib = builder.build_library()
    L = ctypes.CDLL(lib)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert set(dpm.exported_symbols()) == set(declared_symbols())


def test_tools_built():
    import importlib
    builder = importlib.import_module("dpm-g4cpp_gb300.builder")
    builder.build()
    assert os.access(os.path.join(builder.BINDIR, "dpm_simulate"), os.X_OK)
    assert os.access(os.path.join(builder.BINDIR, "dpm_generate_data"), os.X_OK)


def test_torch_operators_build_and_register():
    """lib/libdpmx_torch.so builds against the installed PyTorch and registers
    the torch.ops.dpmx operators (no GPU needed to load it)"""
    import importlib
    builder = importlib.import_module("dpm-g4cpp_gb300.builder")
    builder.build()
    inf = importlib.import_module("dpm-g4cpp_gb300.influence")
    ops = inf.torch_ops()
    for name in ["influence_build", "csr_tensor", "csr_matvec", "csr_rmatvec", "csr_free"]:
        assert hasattr(ops, name), name
