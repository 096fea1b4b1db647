"""ctypes wrapper of the CPU oracle (dpm_oracle.cc). TEST INFRASTRUCTURE ONLY:
imported by the tests, the smoke check and the benchmark's CPU-baseline leg,
never by the product path.

Also wraps the reference's own code built by build_ref.sh (oracle/_ref), when
that build exists (it needs the reference sources, so only where they are).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libdpm_ref.so")
REF_CLI = os.path.join(HERE, "_ref", "dpm_Simulate")
_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(force=False):
    """Compiles the oracle restatement with g++ (IEEE arithmetic, no contraction)."""
    src = os.path.join(HERE, "dpm_oracle.cc")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        # compile beside the library and rename: a process that loads it
        # meanwhile sees the old file or the new one, never a partial one
        tmp = "%s.%d.tmp" % (LIB, os.getpid())
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", src, "-o", tmp],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


def reference_root():
    """The reference checkout the oracle recipes read: $DPM_REFERENCE_ROOT,
    else the path where the build container mounts it."""
    return os.environ.get("DPM_REFERENCE_ROOT", "/root/reference")


def build_ref(reference_root=None):
    """Builds oracle/_ref from the reference sources if they are present."""
    reference_root = reference_root or globals()["reference_root"]()
    if not os.path.isdir(os.path.join(reference_root, "Simulation", "src")):
        return None
    subprocess.run([os.path.join(HERE, "build_ref.sh"), reference_root], check=True, stdout=subprocess.DEVNULL)
    return REF_LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.oracle_load.restype = P
        L.oracle_load.argtypes = [C.c_char_p]
        L.oracle_free.argtypes = [P]
        L.oracle_num_materials.argtypes = [P]
        L.oracle_density.restype = C.c_double
        L.oracle_density.argtypes = [P, C.c_int]
        L.oracle_eval_table.argtypes = [P, C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.oracle_eval_sampler.argtypes = [P, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int]
        L.oracle_simulate_slab.argtypes = [P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_uint32, _dp, _dp,
                                           C.c_int, _dp]
        L.oracle_simulate_slab_philox.argtypes = [P, C.c_longlong, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int,
                                                  C.c_uint64, _dp, _dp, C.c_int, _dp, _dp]
        L.oracle_simulate_voxel.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                            np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS"), C.c_int, C.c_int,
                                            C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_double,
                                            C.c_double, C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_uint64, _dp,
                                            _dp, _dp, C.c_void_p, C.c_void_p]
        L.oracle_simulate_voxel_slabref.argtypes = [P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int,
                                                    C.c_uint32, _dp, _dp, C.c_int, _dp]
        u32 = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        L.oracle_philox.argtypes = [u32, u32, u32, C.c_int]
        _lib = L
    return _lib


def philox(counters, keys):
    """Philox-4x32-10 blocks of the oracle for counters (n, 4) and keys (n, 2)."""
    c = np.ascontiguousarray(counters, dtype=np.uint32).reshape(-1)
    k = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1)
    out = np.zeros_like(c)
    lib().oracle_philox(c, k, out, len(c) // 4)
    return out.reshape(-1, 4)


class Oracle:
    def __init__(self, data_dir):
        self._h = lib().oracle_load(str(data_dir).encode())
        if not self._h:
            raise RuntimeError("oracle could not load %s" % data_dir)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_free(self._h)
            self._h = None

    def table(self, q, energies, imat=0):
        e = np.ascontiguousarray(energies, dtype=np.float64)
        out = np.zeros_like(e)
        lib().oracle_eval_table(self._h, q, imat, e, out, len(e))
        return out

    def sampler(self, s, energies, uniforms, imat=0):
        e = np.ascontiguousarray(energies, dtype=np.float64)
        r = np.ascontiguousarray(uniforms, dtype=np.float64).reshape(-1)
        out = np.zeros_like(e)
        lib().oracle_eval_sampler(self._h, s, imat, e, r, out, len(e))
        return out

    def simulate_slab(self, n, e, iselectron=True, lbox=1.0, geom_index=3, seed=123, cap=4096):
        """Reference Simulate with the mt19937 stream; returns (edep, steps, stats)."""
        ed = np.zeros(cap)
        st = np.zeros(cap)
        stats = np.zeros(4)
        m = lib().oracle_simulate_slab(self._h, n, e, 1 if iselectron else 0, lbox, geom_index, seed, ed, st, cap, stats)
        return ed[:m], st[:m], stats

    def simulate_voxel_slabref(self, n, e, iselectron=True, lbox=1.0, geom_index=3, seed=123, cap=4096):
        """The reference Simulate workload (mt19937 stream) on a 3-D voxel
        phantom laid out as the reference's lattice; returns the depth tally
        (edep, steps) with the reference's histogram length, and stats."""
        ed = np.zeros(cap)
        st = np.zeros(cap)
        stats = np.zeros(4)
        m = lib().oracle_simulate_voxel_slabref(self._h, n, e, 1 if iselectron else 0, lbox, geom_index, seed, ed,
                                                st, cap, stats)
        return ed[:m], st[:m], stats

    def simulate_slab_philox(self, n, e, iselectron=True, lbox=1.0, geom_index=3, seed=12345, first=0, cap=4096):
        """Same workload with the per-history Philox streams of the FP64 GPU form;
        returns (edep, steps, per-history deposit, stats)."""
        ed = np.zeros(cap)
        st = np.zeros(cap)
        he = np.zeros(max(1, n))
        stats = np.zeros(4)
        m = lib().oracle_simulate_slab_philox(self._h, first, n, e, 1 if iselectron else 0, lbox, geom_index, seed,
                                              ed, st, cap, he, stats)
        return ed[:m], st[:m], he[:n], stats

    def simulate_voxel(self, mat, voxel_size, source, nhist, seed, first=0, density=None, tagged=False):
        """Voxel phantom (nz, ny, nx) uint8 (optionally with float32 densities
        per voxel) with a source (dict like the product's Source); returns
        (dose[nz,ny,nx], per-history deposited energy, stats), and with
        tagged=True (beamlet-grid sources) also the dose per beamlet
        [nbeamlets, nz, ny, nx]."""
        m = np.ascontiguousarray(mat, dtype=np.uint8)
        rho = None if density is None else np.ascontiguousarray(density, dtype=np.float32).reshape(-1)
        nz, ny, nx = m.shape
        v = np.broadcast_to(np.asarray(voxel_size, dtype=np.float64), (3,))
        dose = np.zeros(m.size)
        he = np.zeros(max(1, nhist))
        stats = np.zeros(4)
        s = source
        bt = None
        if tagged:
            nb = max(1, s["nbx"] * s["nby"]) if s["shape"] == 2 else 1
            bt = np.zeros((nb, nz, ny, nx))
        lib().oracle_simulate_voxel(self._h, nx, ny, nz, float(v[0]), float(v[1]), float(v[2]), m.reshape(-1),
                                    s["particle"], s["spectrum"], s["e0"], s["e1"], s["shape"], s["cx"], s["cy"],
                                    s["fx"], s["fy"], s["nbx"], s["nby"], first, nhist, seed, dose, he, stats,
                                    None if rho is None else rho.ctypes.data, None if bt is None else bt.ctypes.data)
        if tagged:
            return dose.reshape(nz, ny, nx), he[:nhist], stats, bt
        return dose.reshape(nz, ny, nx), he[:nhist], stats


class Reference:
    """The reference's own functions (oracle/_ref/libdpm_ref.so)."""

    def __init__(self, data_dir):
        if not os.path.exists(REF_LIB):
            raise RuntimeError("reference build missing (oracle/build_ref.sh)")
        L = C.CDLL(REF_LIB)
        P = C.c_void_p
        L.ref_load.restype = P
        L.ref_load.argtypes = [C.c_char_p]
        L.ref_seed.argtypes = [C.c_uint32]
        L.ref_eval_table.argtypes = [P, C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.ref_eval_sampler.argtypes = [P, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int]
        L.ref_simulate_full.argtypes = [P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, _dp, _dp, C.c_int]
        L.ref_simulate_cli.argtypes = [P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_char_p]
        L.ref_distance.argtypes = [C.c_double, C.c_int, P, _dp, _dp, np.ctypeslib.ndpointer(np.int32), _dp, C.c_int]
        self.L = L
        self._h = L.ref_load(str(data_dir).encode())

    def table(self, q, energies, imat=0):
        e = np.ascontiguousarray(energies, dtype=np.float64)
        out = np.zeros_like(e)
        self.L.ref_eval_table(self._h, q, imat, e, out, len(e))
        return out

    def sampler(self, s, energies, uniforms, imat=0):
        e = np.ascontiguousarray(energies, dtype=np.float64)
        r = np.ascontiguousarray(uniforms, dtype=np.float64).reshape(-1)
        out = np.zeros_like(e)
        self.L.ref_eval_sampler(self._h, s, imat, e, r, out, len(e))
        return out

    def simulate_full(self, n, e, iselectron=True, lbox=1.0, geom_index=3, seed=123, cap=4096):
        self.L.ref_seed(seed)
        ed = np.zeros(cap)
        st = np.zeros(cap)
        m = self.L.ref_simulate_full(self._h, n, e, 1 if iselectron else 0, lbox, geom_index, ed, st, cap)
        return ed[:m], st[:m]

    def simulate_cli(self, n, e, iselectron, lbox, geom_index, fname, seed=123):
        self.L.ref_seed(seed)
        self.L.ref_simulate_cli(self._h, n, e, 1 if iselectron else 0, lbox, geom_index, str(fname).encode())


# ---------------------------------------------------------------------------
# Parallel batches of the voxel transport (a spawned process pool, so that it
# is safe to start after the GPU has been used)
# ---------------------------------------------------------------------------
_worker_oracles = {}


def _voxel_batch(args):
    data_dir, mat, voxel, source, n, seed, first, density, tagged = args
    o = _worker_oracles.get(data_dir)
    if o is None:
        o = _worker_oracles[data_dir] = Oracle(data_dir)
    r = o.simulate_voxel(mat, voxel, source, n, seed, first=first, density=density, tagged=tagged)
    return (r[3] if tagged else r[0]), r[2]


def voxel_batches(data_dir, mat, voxel, source, per, batches, seed, first=0, density=None, processes=None,
                  tagged=False, keep=False):
    """Runs `batches` oracle batches of `per` histories each (batch k: history
    ids first + k*per ...) on the host cores. Returns the per-history mean
    dose, its standard error from the batch spread (both shaped like mat, or
    [nbeamlets, *mat.shape] per beamlet with tagged=True), and the summed
    stats [deposited, escaped, sub-steps, max stack depth]; with keep=True
    also every batch's per-history dose, stacked in batch order."""
    import multiprocessing as mp
    build()            # once, here: the workers then load the built library
    processes = processes or min(batches, os.cpu_count() or 1)
    tasks = [(str(data_dir), mat, voxel, source, per, seed, first + k * per, density, tagged)
             for k in range(batches)]
    s1 = s2 = None
    stats = np.zeros(4)
    kept = []
    with mp.get_context("spawn").Pool(processes) as pool:
        for dose, st in (pool.imap if keep else pool.imap_unordered)(_voxel_batch, tasks):
            if keep:
                kept.append(dose / per)
            if s1 is None:
                s1 = np.zeros(dose.shape)
                s2 = np.zeros(dose.shape)
            d = dose / per
            s1 += d
            s2 += d * d
            stats[:3] += st[:3]
            stats[3] = max(stats[3], st[3])
    mean = s1 / batches
    var = np.maximum(s2 / batches - mean * mean, 0.0) * batches / max(batches - 1, 1)
    if keep:
        return mean, np.sqrt(var / batches), stats, np.stack(kept)
    return mean, np.sqrt(var / batches), stats
