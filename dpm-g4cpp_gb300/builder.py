"""Builds the native parts of the package in place (no CMake):

  lib/libdpmx.so          CUDA kernels (sm_103a) + host C++ behind include/dpmx.h
  lib/libdpmx_torch.so    torch.ops.dpmx operators over the influence matrix
  bin/dpm_simulate        drop-in for the reference `dpm_Simulate` CLI
  bin/dpm_generate_data   Geant4-free writer of the reference data files

Translation units are compiled in parallel; each nvcc call targets sm_103a only.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libdpmx.so")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE] + ARCH

# per-unit flags: the FP64 form keeps the reference's operation order (no FMA
# contraction); the FP32 form uses approximate division / square root and
# flushes denormals
CU_UNITS = {
    "transport_fp64.cu": ["-fmad=false"],
    "transport_fp32.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    "api.cu": [],
    "run.cu": [],
    "influence.cu": [],
    "noalloc.cu": [],
    "validation.cu": [],
}
CXX_UNITS = ["host_tables.cpp"]


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "dpmx.h")]


def build_library(verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src, extra in CU_UNITS.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([NVCC] + NVFLAGS + extra + ["-c", s, "-o", o])
    for src in CXX_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-I" + INCLUDE, "-I/usr/local/cuda/include",
                         "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_tools():
    os.makedirs(BINDIR, exist_ok=True)
    cli = os.path.join(BINDIR, "dpm_simulate")
    src = os.path.join(HERE, "cli", "dpm_simulate.cpp")
    if _stale(cli, [src, LIB]):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, src, "-o", cli, "-L" + LIBDIR, "-ldpmx",
              "-Wl,-rpath,$ORIGIN/../lib"])
    gen = os.path.join(BINDIR, "dpm_generate_data")
    gsrc = os.path.join(HERE, "datagen", "dpm_generate_data.cpp")
    if _stale(gen, [gsrc]):
        _run(["g++", "-O2", "-std=c++17", gsrc, "-o", gen])
    return cli, gen


TORCH_OPS = os.path.join(LIBDIR, "libdpmx_torch.so")


def build_torch_ops():
    """lib/libdpmx_torch.so: the torch.ops.dpmx operators (csrc/torch_ops.cpp),
    compiled against the installed PyTorch and linked to libdpmx.so."""
    src = os.path.join(CSRC, "torch_ops.cpp")
    if not _stale(TORCH_OPS, [src, LIB, os.path.join(INCLUDE, "dpmx.h")]):
        return TORCH_OPS
    import torch
    from torch.utils import cpp_extension as ce
    abi = int(torch.compiled_with_cxx11_abi())
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-D_GLIBCXX_USE_CXX11_ABI=%d" % abi, "-I" + INCLUDE,
           "-I/usr/local/cuda/include"]
    cmd += ["-I" + p for p in ce.include_paths()]
    cmd += [src, "-o", TORCH_OPS, "-L" + LIBDIR, "-ldpmx", "-Wl,-rpath,$ORIGIN"]
    cmd += ["-L" + p for p in ce.library_paths()] + ["-lc10", "-lc10_cuda", "-ltorch_cpu", "-ltorch_cuda"]
    _run(cmd)
    return TORCH_OPS


def build(verbose=False):
    lib = build_library(verbose)
    build_tools()
    build_torch_ops()
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
