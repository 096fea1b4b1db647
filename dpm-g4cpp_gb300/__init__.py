"""GB300-native dpm_Simulate: Python host layer over libdpmx.so (include/dpmx.h).

The names mirror the reference's simulation-phase interface:

  Tables(data_dir)            SimElectronData/SimPhotonData/SimMaterialData::Load
                              (dpm_Simulate.cc:71-78): the 14 data files
  Phantom.slab(t, geom, lbox) Geom(lbox, matData, geomIndex) (Geom.cc:9-17)
  Phantom.voxels(t, mat, v)   a 3-D voxel phantom behind the same Geom interface
  simulate(...)               Simulate(nprimary, eprimary, isElectron, lbox, ...,
                              geomIndex, filename) (SimDPMLike.cc:40-251)
  write_hist(...)             Geom::Write (Geom.cc:167-192), hist.sim
  run(t, jobs, ...)           many Simulate-like jobs batched in one run

Errors raise DpmxError carrying the library's status code and message, the
counterpart of the reference's `exit(EXIT_FAILURE)` with a stderr message. All
transport runs on the GPU; importing the package without the built library
raises at the first call.
"""
import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# the in-tree build (builder.py), or another build of the same library named by $DPMX_LIBRARY
LIB_PATH = os.environ.get("DPMX_LIBRARY") or os.path.join(_HERE, "lib", "libdpmx.so")

FP64_PLAIN = 0
FP32_EVENT = 1
DOSE_RAW = 0      # 3-D dose [Gy per history] + relative uncertainty (voxel phantoms)
DOSE_DEPTH = 1    # hist.sim-format depth profile (any phantom)
MODEL_BREM, MODEL_MOLLER, MODEL_MSC = 0, 1, 2

OK, ERR_FILE, ERR_PARSE, ERR_CUDA, ERR_ARG, ERR_OVERFLOW, ERR_NOMEM = 0, -1, -2, -3, -4, -5, -6


class DpmxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("dpmx error %d: %s" % (code, msg))
        self.code = code


class _Source(C.Structure):
    _fields_ = [("particle", C.c_int), ("spectrum", C.c_int), ("e0", C.c_double), ("e1", C.c_double),
                ("shape", C.c_int), ("cx", C.c_double), ("cy", C.c_double), ("fx", C.c_double),
                ("fy", C.c_double), ("nbx", C.c_int), ("nby", C.c_int)]


class _Job(C.Structure):
    _fields_ = [("phantom", C.c_void_p), ("source", _Source), ("histories", C.c_longlong), ("seed", C.c_uint64),
                ("first_history", C.c_longlong)]


class _Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("batches", C.c_int), ("block_size", C.c_int), ("blocks_per_sm", C.c_int),
                ("chunk_histories", C.c_longlong), ("tally_aggregate", C.c_int), ("use_graph", C.c_int),
                ("tag_beamlets", C.c_int), ("autotune", C.c_int), ("profile_phases", C.c_int),
                ("electron_kernel", C.c_int), ("photon_kernel", C.c_int), ("stream", C.c_void_p),
                ("electron_slots", C.c_int)]


class _Stats(C.Structure):
    _fields_ = [("edep", C.c_double), ("escaped", C.c_double), ("primary_energy", C.c_double),
                ("max_residual", C.c_double), ("residual_violations", C.c_longlong), ("lost", C.c_longlong),
                ("steps", C.c_longlong), ("histories", C.c_longlong)]


_lib = None
_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


def library():
    """Loads libdpmx.so (built in place by build.py); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise DpmxError(ERR_FILE, "native library %s not built (run build())" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sig = {
        "dpmx_last_error": (C.c_char_p, []),
        "dpmx_version": (C.c_char_p, []),
        "dpmx_tables_load": (C.c_int, [C.c_char_p, C.POINTER(P)]),
        "dpmx_tables_free": (None, [P]),
        "dpmx_tables_num_materials": (C.c_int, [P]),
        "dpmx_tables_param": (C.c_double, [P, C.c_int]),
        "dpmx_tables_density": (C.c_double, [P, C.c_int]),
        "dpmx_tables_material_name": (C.c_int, [P, C.c_int, C.c_char_p, C.c_int]),
        "dpmx_phantom_slab": (C.c_int, [P, C.c_int, C.c_double, C.POINTER(P)]),
        "dpmx_phantom_voxels": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                          np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS"), C.POINTER(P)]),
        "dpmx_phantom_voxels_density": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                                  np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS"),
                                                  np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS"),
                                                  C.POINTER(P)]),
        "dpmx_phantom_free": (None, [P]),
        "dpmx_phantom_tally_size": (C.c_longlong, [P]),
        "dpmx_run_options_default": (None, [C.POINTER(_Opts)]),
        "dpmx_run": (C.c_int, [P, C.POINTER(_Job), C.c_int, C.POINTER(_Opts), C.POINTER(P)]),
        "dpmx_result_tally": (C.c_int, [P, C.c_int, P, P, P]),
        "dpmx_result_tally_device": (C.c_void_p, [P, C.c_int]),
        "dpmx_result_stats": (C.c_int, [P, C.c_int, C.POINTER(_Stats)]),
        "dpmx_result_elapsed_ms": (C.c_double, [P]),
        "dpmx_result_launches": (C.c_longlong, [P]),
        "dpmx_result_config": (C.c_int, [P, C.POINTER(C.c_longlong)]),
        "dpmx_result_profile": (C.c_int, [P, C.POINTER(C.c_double)]),
        "dpmx_result_free": (None, [P]),
        "dpmx_scratch_release": (None, []),
        "dpmx_result_write": (C.c_int, [P, C.c_int, C.c_char_p, C.c_int]),
        "dpmx_model_histogram": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_longlong, C.c_uint64,
                                           C.c_int, _dp, _dp]),
        "dpmx_simulate": (C.c_int, [P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_uint64, C.c_int,
                                    _dp, _dp, C.c_int, C.POINTER(C.c_int)]),
        "dpmx_write_hist": (C.c_int, [P, C.c_char_p, C.c_int, C.c_double, C.c_int, _dp, _dp, C.c_int]),
        "dpmx_simulate_noalloc": (C.c_int, [P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_uint64,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                            C.c_void_p]),
        "dpmx_sampler_eval": (C.c_int, [P, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int]),
        "dpmx_table_eval": (C.c_int, [P, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_int]),
        "dpmx_simulate_histories": (C.c_int, [P, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_uint64,
                                              _dp, _dp, C.c_int]),
        "dpmx_influence_build": (C.c_int, [P, C.c_int, C.c_double, C.POINTER(P)]),
        "dpmx_csr_shape": (C.c_int, [P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "dpmx_csr_device": (C.c_int, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
        "dpmx_csr_spmv": (C.c_int, [P, C.c_void_p, C.c_void_p, C.c_void_p]),
        "dpmx_csr_spmv_t": (C.c_int, [P, C.c_void_p, C.c_void_p, C.c_void_p]),
        "dpmx_csr_download": (C.c_int, [P, C.c_void_p, C.c_void_p, C.c_void_p]),
        "dpmx_csr_free": (None, [P]),
        "dpmx_ring_selftest": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_longlong,
                                         C.POINTER(C.c_longlong)]),
        "dpmx_rng_eval": (C.c_int, [_u32p, _u32p, C.c_int, _u32p,
                                    np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS"), _dp]),
        "dpmx_atomic_roof": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
        "dpmx_job_histories": (C.c_int, [P, C.POINTER(_Job), _dp, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != OK:
        raise DpmxError(rc, library().dpmx_last_error().decode())


def exported_symbols():
    """Names the C ABI exports (declared in include/dpmx.h)."""
    return ["dpmx_last_error", "dpmx_version", "dpmx_tables_load", "dpmx_tables_free", "dpmx_tables_num_materials",
            "dpmx_tables_param", "dpmx_tables_density", "dpmx_tables_material_name", "dpmx_phantom_slab",
            "dpmx_phantom_voxels", "dpmx_phantom_voxels_density", "dpmx_phantom_free", "dpmx_phantom_tally_size", "dpmx_run_options_default",
            "dpmx_run", "dpmx_result_tally", "dpmx_result_tally_device", "dpmx_result_stats",
            "dpmx_result_elapsed_ms", "dpmx_result_launches", "dpmx_result_config", "dpmx_result_profile",
            "dpmx_result_free", "dpmx_scratch_release", "dpmx_result_write", "dpmx_model_histogram",
            "dpmx_simulate", "dpmx_simulate_noalloc", "dpmx_write_hist", "dpmx_sampler_eval", "dpmx_table_eval", "dpmx_simulate_histories",
            "dpmx_influence_build", "dpmx_csr_shape", "dpmx_csr_device", "dpmx_csr_spmv", "dpmx_csr_spmv_t",
            "dpmx_csr_download", "dpmx_csr_free", "dpmx_ring_selftest", "dpmx_rng_eval",
            "dpmx_atomic_roof", "dpmx_job_histories"]


class Tables:
    """The simulation data of one data directory, uploaded to the GPU."""

    def __init__(self, data_dir):
        L = library()
        h = C.c_void_p()
        _check(L.dpmx_tables_load(str(data_dir).encode(), C.byref(h)))
        self._h = h
        self.data_dir = str(data_dir)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            library().dpmx_tables_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_materials(self):
        return library().dpmx_tables_num_materials(self._h)

    def density(self, imat):
        return library().dpmx_tables_density(self._h, imat)

    def material_name(self, imat):
        buf = C.create_string_buffer(128)
        _check(library().dpmx_tables_material_name(self._h, imat, buf, 128))
        return buf.value.decode()

    @property
    def electron_cut(self):
        return library().dpmx_tables_param(self._h, 0)

    @property
    def gamma_cut(self):
        return library().dpmx_tables_param(self._h, 1)

    def eval_sampler(self, sampler, energies, uniforms, imat=0, precision=FP64_PLAIN):
        """Runs sampler 0 KN, 1 Moller, 2 SB, 3 GS on the GPU with given uniforms (n x 3)."""
        e = np.ascontiguousarray(energies, dtype=np.float64)
        r = np.ascontiguousarray(uniforms, dtype=np.float64).reshape(-1)
        out = np.zeros_like(e)
        _check(library().dpmx_sampler_eval(self._h, precision, sampler, imat, e, r, out, len(e)))
        return out

    def model_histogram(self, model, e0, n, imat=0, seed=1, hbins=101, precision=FP64_PLAIN):
        """(x, hist_x, cos, hist_cos): the reference's model-validation histograms
        (testAPI) of n interactions sampled on the GPU; counts, not normalised."""
        hx = np.zeros(hbins)
        hc = np.zeros(hbins)
        _check(library().dpmx_model_histogram(self._h, precision, model, imat, float(e0), int(n), int(seed), hbins,
                                              hx, hc))
        xmin = math.log10(self.gamma_cut / e0)
        hdel = (0.1 - xmin) / (hbins - 1)
        return xmin + (np.arange(hbins) + 0.5) * hdel, hx, -1.0 + np.arange(hbins) * 2.0 / (hbins - 1), hc

    def eval_table(self, quantity, energies, imat=0, precision=FP64_PLAIN):
        e = np.ascontiguousarray(energies, dtype=np.float64)
        out = np.zeros_like(e)
        _check(library().dpmx_table_eval(self._h, precision, quantity, imat, e, out, len(e)))
        return out


class Phantom:
    def __init__(self, tables, handle, shape):
        self.tables = tables
        self._h = handle
        self.shape = shape

    @classmethod
    def slab(cls, tables, geom_index, lbox):
        h = C.c_void_p()
        _check(library().dpmx_phantom_slab(tables.handle, geom_index, lbox, C.byref(h)))
        return cls(tables, h, (library().dpmx_phantom_tally_size(h),))

    @classmethod
    def voxels(cls, tables, mat, voxel_size, density=None):
        """mat: uint8 array of shape (nz, ny, nx) (x fastest), 255 = vacuum; voxel_size mm (scalar or 3);
        density: optional float32 array like mat [g/cm3] (per-voxel density; the material id keeps
        the composition)."""
        m = np.ascontiguousarray(mat, dtype=np.uint8)
        nz, ny, nx = m.shape
        v = np.broadcast_to(np.asarray(voxel_size, dtype=np.float64), (3,))
        h = C.c_void_p()
        if density is None:
            _check(library().dpmx_phantom_voxels(tables.handle, nx, ny, nz, float(v[0]), float(v[1]), float(v[2]),
                                                  m.reshape(-1), C.byref(h)))
        else:
            r = np.ascontiguousarray(density, dtype=np.float32)
            if r.shape != m.shape:
                raise DpmxError(ERR_ARG, "density must have the shape of mat")
            _check(library().dpmx_phantom_voxels_density(tables.handle, nx, ny, nz, float(v[0]), float(v[1]),
                                                          float(v[2]), m.reshape(-1), r.reshape(-1), C.byref(h)))
        return cls(tables, h, (nz, ny, nx))

    @property
    def handle(self):
        return self._h

    @property
    def tally_size(self):
        return library().dpmx_phantom_tally_size(self._h)

    def close(self):
        if self._h:
            library().dpmx_phantom_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Source:
    particle: int = -1          # -1 electron, 0 photon
    spectrum: int = 0           # 0 mono, 1 uniform [e0,e1], 2 p(E) ~ (e1-E)
    e0: float = 15.0
    e1: float = 15.0
    shape: int = 0              # 0 pencil, 1 rectangle, 2 beamlet grid
    cx: float = 0.0
    cy: float = 0.0
    fx: float = 0.0
    fy: float = 0.0
    nbx: int = 0
    nby: int = 0

    def _c(self):
        return _Source(self.particle, self.spectrum, self.e0, self.e1, self.shape, self.cx, self.cy, self.fx,
                       self.fy, self.nbx, self.nby)


@dataclass
class Job:
    phantom: Phantom
    source: Source = field(default_factory=Source)
    histories: int = 1000
    seed: int = 12345
    first_history: int = 0


@dataclass
class JobStats:
    edep: float
    escaped: float
    primary_energy: float
    max_residual: float
    residual_violations: int
    lost: int
    steps: int
    histories: int


class Result:
    def __init__(self, handle, jobs):
        self._h = handle
        self._jobs = jobs

    def tally(self, j=0, out=None):
        """(dose, dose2, steps) of job j as numpy arrays shaped like the phantom tally.

        out: optional (dose, dose2, steps) float64 arrays of tally_size elements
        to copy into (for instance views of pinned host memory, which copy
        faster); steps may be None."""
        ph = self._jobs[j].phantom
        n = ph.tally_size
        if out is None:
            d, d2, s = np.zeros(n), np.zeros(n), np.zeros(n)
        else:
            d, d2, s = out
            for x in (d, d2) + ((s,) if s is not None else ()):
                if x.dtype != np.float64 or x.size != n or not x.flags["C_CONTIGUOUS"]:
                    raise DpmxError(ERR_ARG, "tally output arrays must be contiguous float64 of tally_size")
        _check(library().dpmx_result_tally(self._h, j, d.ctypes.data, d2.ctypes.data,
                                           s.ctypes.data if s is not None else None))
        if s is None:
            s = np.zeros(0)
        shp = ph.shape
        if len(shp) == 3:
            return d.reshape(shp), d2.reshape(shp), (s.reshape(shp) if s.size else s)
        return d, d2, s

    def write(self, path, j=0, fmt=DOSE_DEPTH):
        """Writes job j's dose: DOSE_RAW (binary, see read_dose_raw) or DOSE_DEPTH (hist.sim text)."""
        _check(library().dpmx_result_write(self._h, j, str(path).encode(), fmt))

    def tally_device_ptr(self, j=0):
        return library().dpmx_result_tally_device(self._h, j)

    def stats(self, j=0):
        s = _Stats()
        _check(library().dpmx_result_stats(self._h, j, C.byref(s)))
        return JobStats(s.edep, s.escaped, s.primary_energy, s.max_residual, s.residual_violations, s.lost,
                        s.steps, s.histories)

    @property
    def elapsed_ms(self):
        return library().dpmx_result_elapsed_ms(self._h)

    @property
    def launches(self):
        return library().dpmx_result_launches(self._h)

    @property
    def config(self):
        a = (C.c_longlong * 4)()
        _check(library().dpmx_result_config(self._h, a))
        return dict(block_size=a[0], blocks_per_sm=a[1], chunk_histories=a[2], tally_aggregate=a[3] & 1,
                    electron_kernel=(a[3] >> 1) & 1, photon_kernel=(a[3] >> 2) & 1, electron_slots=a[3] >> 3)

    @property
    def profile(self):
        """Phase profile of a run made with profile_phases=True."""
        a = (C.c_double * 10)()
        _check(library().dpmx_result_profile(self._h, a))
        keys = ["electron_ms", "photon_ms", "electron_launches", "photon_launches", "electron_steps",
                "photon_steps", "electrons", "photons", "histories", "total_ms"]
        return dict(zip(keys, list(a)))

    def influence(self, j=0, threshold=0.0):
        from .influence import InfluenceMatrix
        h = C.c_void_p()
        _check(library().dpmx_influence_build(self._h, j, threshold, C.byref(h)))
        return InfluenceMatrix(h)

    def close(self):
        if self._h:
            library().dpmx_result_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_dose_raw(path):
    """Reads a DOSE_RAW file: (dose [Gy per history], relative 1-sigma
    uncertainty, header dict), arrays shaped (nz, ny, nx)."""
    with open(path, "rb") as f:
        if f.read(8) != b"DPMXDOSE":
            raise DpmxError(ERR_PARSE, "%s is not a raw dose file" % path)
        version, nx, ny, nz = np.frombuffer(f.read(16), dtype="<i4")
        if version != 1:
            raise DpmxError(ERR_PARSE, "raw dose version %d not supported" % version)
        vx, vy, vz, x0, y0, z0 = np.frombuffer(f.read(48), dtype="<f8")
        hist, batches = np.frombuffer(f.read(16), dtype="<i8")
        n = int(nx) * int(ny) * int(nz)
        dose = np.frombuffer(f.read(8 * n), dtype="<f8").reshape(nz, ny, nx)
        rel = np.frombuffer(f.read(8 * n), dtype="<f8").reshape(nz, ny, nx)
    head = dict(nx=int(nx), ny=int(ny), nz=int(nz), voxel_mm=(vx, vy, vz), origin_mm=(x0, y0, z0),
                histories=int(hist), batches=int(batches))
    return dose, rel, head


def ring_selftest(blocks=152, nslots=416, rounds=1000, seed=1, probe_cycles=1 << 20):
    """Runs the slot-ring self-test on the GPU (dpmx_ring_selftest): returns
    (slots taken, slots taken a wrong number of times, warps that gave up a
    wait, blocks whose probe wait on a never-filled cell ran out)."""
    out = (C.c_longlong * 4)()
    _check(library().dpmx_ring_selftest(int(blocks), int(nslots), int(rounds), int(seed), int(probe_cycles), out))
    return tuple(int(v) for v in out)


def rng_eval(counters, keys):
    """Philox-4x32-10 on the GPU (dpmx_rng_eval): for counters (n, 4) and keys
    (n, 2) uint32, returns the blocks (n, 4) uint32, the FP32 transport's
    uniforms of each word (n, 4) float32 and the FP64 form's uniforms of each
    word pair (n, 2) float64."""
    c = np.ascontiguousarray(counters, dtype=np.uint32).reshape(-1, 4)
    k = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 2)
    n = len(c)
    if len(k) != n:
        raise DpmxError(ERR_ARG, "one key per counter")
    w = np.zeros((n, 4), dtype=np.uint32)
    f = np.zeros((n, 4), dtype=np.float32)
    d = np.zeros((n, 2), dtype=np.float64)
    _check(library().dpmx_rng_eval(c.reshape(-1), k.reshape(-1), n, w.reshape(-1), f.reshape(-1), d.reshape(-1)))
    return w, f, d


def atomic_roof(nbins=1 << 22, per_thread=256):
    """FP64 atomicAdd operations per second into an L2-resident array (the
    dose tally's roof), measured on the current GPU."""
    v = C.c_double(0.0)
    _check(library().dpmx_atomic_roof(int(nbins), int(per_thread), C.byref(v)))
    return v.value


def scratch_release():
    """Frees the device scratch that finished runs keep for later runs."""
    library().dpmx_scratch_release()


def run(tables, jobs, precision=FP32_EVENT, batches=10, block_size=0, blocks_per_sm=0, chunk_histories=0,
        tally_aggregate=-1, use_graph=True, tag_beamlets=False, autotune=False, profile_phases=False,
        electron_kernel=-1, photon_kernel=-1, stream=None, electron_slots=0):
    """Runs the jobs (one run, one stream) and returns a Result."""
    L = library()
    arr = (_Job * len(jobs))()
    for i, j in enumerate(jobs):
        arr[i] = _Job(j.phantom.handle.value if hasattr(j.phantom.handle, "value") else j.phantom.handle,
                      j.source._c(), int(j.histories), int(j.seed), int(j.first_history))
    o = _Opts()
    L.dpmx_run_options_default(C.byref(o))
    o.precision = precision
    o.batches = batches
    o.block_size = block_size
    o.blocks_per_sm = blocks_per_sm
    o.chunk_histories = chunk_histories
    o.tally_aggregate = tally_aggregate
    o.use_graph = 1 if use_graph else 0
    o.tag_beamlets = 1 if tag_beamlets else 0
    o.autotune = 1 if autotune else 0
    o.profile_phases = 1 if profile_phases else 0
    o.electron_kernel = electron_kernel
    o.photon_kernel = photon_kernel
    o.stream = stream
    o.electron_slots = electron_slots
    h = C.c_void_p()
    rc = L.dpmx_run(tables.handle, arr, len(jobs), C.byref(o), C.byref(h))
    if rc != OK:
        msg = L.dpmx_last_error().decode()
        if h:
            L.dpmx_result_free(h)
        raise DpmxError(rc, msg)
    return Result(h, list(jobs))


def simulate(tables, nprimary, eprimary=15.0, iselectron=True, lbox=1.0, geom_index=0, seed=123,
             precision=FP64_PLAIN, cap=4096):
    """The reference Simulate workload: returns (edep_hist, step_hist) with the
    reference's histogram length."""
    e = np.zeros(cap)
    s = np.zeros(cap)
    n = C.c_int(0)
    _check(library().dpmx_simulate(tables.handle, int(nprimary), float(eprimary), 1 if iselectron else 0,
                                   float(lbox), int(geom_index), int(seed), precision, e, s, cap, C.byref(n)))
    return e[:n.value].copy(), s[:n.value].copy()


def simulate_histories(tables, nprimary, eprimary=15.0, iselectron=True, lbox=1.0, geom_index=0, seed=123,
                       cap=4096):
    """FP64 form, also returning each history's deposited energy."""
    he = np.zeros(max(1, nprimary))
    e = np.zeros(cap)
    _check(library().dpmx_simulate_histories(tables.handle, int(nprimary), float(eprimary), 1 if iselectron else 0,
                                             float(lbox), int(geom_index), int(seed), he, e, cap))
    return he[:nprimary], e


def job_histories(tables, job, with_dose=False):
    """FP64 form of one job on any phantom: each history's deposited energy
    (and the job's dose tally when with_dose)."""
    h = job.phantom.handle
    j = _Job(h.value if hasattr(h, "value") else h, job.source._c(), int(job.histories), int(job.seed),
             int(job.first_history))
    he = np.zeros(max(1, int(job.histories)))
    dose = np.zeros(job.phantom.tally_size) if with_dose else None
    _check(library().dpmx_job_histories(tables.handle, C.byref(j), he,
                                        None if dose is None else dose.ctypes.data))
    he = he[:int(job.histories)]
    return (he, dose) if with_dose else he


def write_hist(tables, fname, geom_index, lbox, nprimary, edep_hist, step_hist):
    e = np.ascontiguousarray(edep_hist, dtype=np.float64)
    s = np.ascontiguousarray(step_hist, dtype=np.float64)
    _check(library().dpmx_write_hist(tables.handle, str(fname).encode(), geom_index, lbox, nprimary, e, s, len(e)))


def build(verbose=False):
    from . import builder
    return builder.build(verbose)
