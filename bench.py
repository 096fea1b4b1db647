#!/usr/bin/env python
"""Benchmark: histories/s of the FP32 event-based transport (FP64 tallies) on
the precision-form workload: a 128x128x256 phantom of 2 mm voxels (water body,
G4_LUNG_ICRP slab z = 60-120 mm, G4_BONE_COMPACT_ICRU cylinder r = 15 mm along
y at x = 0, z = 180 mm), a 10x10 cm2 photon beam with energy uniform in
1-20 MeV, seed 7. A step is one run of `--hist` histories (default 1e7; 10
steps = the workload's 1e8 histories) with 10 statistical batches.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU oracle (the restatement of the reference's
double-precision transport) on the host cores on a bounded sample of the same
workload. Under torchrun each rank runs its own history range (weak scaling).

Besides the timed steps the line carries, measured outside the timed region:
the plain FP64 GPU form on the same workload (`fp64_gpu`, and `vs_fp64_gpu` =
value / its histories/s), a voxel-by-voxel dose check of the FP32 form
against it (`dose_check`), Gy-voxels/s, and the roofline of the dominant
kernel against four roofs (instruction issue, L2 FP64 atomics, FP32 pipe,
DRAM), `bound` naming the one it is closest to.
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
DATA = os.path.join(ROOT, "data", "water_lung_bone")
METRIC = "histories/s"
WORKLOAD = "precision form: 128x128x256 x 2 mm water/lung-slab/bone-cylinder phantom, 10x10 cm2 photon beam U[1,20] MeV"

# nominal FP32 rate: 152 SMs x 128 lanes x 2 (FMA) x 2.07 GHz
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
# instruction issue: 4 schedulers per SM, one warp instruction per cycle each
ISSUE_PER_SM_CYCLE = 4
SMS = 152


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--hist", type=float, default=1e7, help="histories per step and GPU")
    ap.add_argument("--cpu-hist", type=int, default=200000, help="oracle histories per CPU worker and step")
    ap.add_argument("--batches", type=int, default=10, help="statistical batches per step")
    ap.add_argument("--fp64-hist", type=float, default=1e7, help="histories of the FP64 GPU arm")
    ap.add_argument("--check-hist", type=float, default=4e7, help="FP32 histories of the dose check")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# CPU oracle (reference arm and cpu_baseline): one process per core
# ---------------------------------------------------------------------------
def _oracle_worker(args):
    first, n, seed = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, ROOT)
    import numpy as np  # noqa: F401
    orc = importlib.import_module("cpu_oracle")
    wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
    o = orc.Oracle(DATA)
    m = wl.precision_phantom()
    s = wl.precision_source()
    src = dict(particle=s.particle, spectrum=s.spectrum, e0=s.e0, e1=s.e1, shape=s.shape, cx=s.cx, cy=s.cy,
               fx=s.fx, fy=s.fy, nbx=s.nbx, nby=s.nby)
    t0 = time.perf_counter()
    if n > 0:
        o.simulate_voxel(m, 2.0, src, n, seed, first=first)
    return time.perf_counter() - t0


def oracle_pool():
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(cores)
    pool.map(_oracle_worker, [(0, 0, 7)] * cores)   # load oracle + phantom in every worker
    return pool, cores


def oracle_step(pool, cores, per, step):
    t0 = time.perf_counter()
    pool.map(_oracle_worker, [((step * cores + k) * per, per, 7) for k in range(cores)])
    dt = time.perf_counter() - t0
    return cores * per / dt, dt


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []          # (arrival time, fields)
        self.proc = None
        self.t0 = self.t1 = None

    def start(self):
        """Starts sampling every 50 ms and returns once the first sample has
        arrived, so that the timed region that follows is covered."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
            return
        t = time.time()
        while not self.rows and time.time() - t < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        # the samples taken between begin() and end() (a line arrives a few ms
        # after its sample); all of them when the region was shorter than one period
        rows = [r for t, r in self.rows if self.t0 is not None and self.t1 is not None and self.t0 <= t <= self.t1 + 0.02]
        if not rows:
            rows = [r for _, r in self.rows]
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def roofline_of(dpm, pr, eblock, pblock, clk):
    """The dominant phase kernel against four roofs, from a profiled run's
    per-phase times and unit counts and the per-unit counters that ncu
    measured for that kernel (profiles/counters.json):
      issue      warp instructions / s against 4 per SM and cycle at the SM
                 clock measured during the timed region
      l2_atomic  tally atomics / s (one FP64 atomicAdd per electron sub-step
                 at most) against dpmx_atomic_roof on this GPU
      fp32       FP32 flops / s against the nominal FP32 rate
      dram       DRAM bytes / s (ncu traffic per unit) against MEASURED_PEAKS
    `bound` is the roof with the largest fraction."""
    with open(os.path.join(ROOT, "profiles", "counters.json")) as f:
        counters = json.load(f)
    if pr["electron_ms"] >= pr["photon_ms"]:
        kname = "ElectronPhaseB" if eblock else "ElectronPhase"
        kms, nl, units = pr["electron_ms"], pr["electron_launches"], pr["electron_steps"]
        atomics = pr["electron_steps"]
    else:
        kname = "PhotonPhaseB" if pblock else "PhotonPhase"
        kms, nl, units = pr["photon_ms"], pr["photon_launches"], pr["photon_steps"]
        atomics = None
    c = counters.get(kname, {})
    secs = kms * 1e-3
    sm_mhz = clk.get("sm_mhz") or 2070.0
    roofs = {}
    if c.get("warp_inst_per_unit"):
        ach = c["warp_inst_per_unit"] * units / secs / 1e9
        peak = SMS * ISSUE_PER_SM_CYCLE * sm_mhz * 1e6 / 1e9
        roofs["issue"] = {"achieved": ach, "peak": peak, "unit": "Gwarp-inst/s", "frac": ach / peak,
                          "peak_source": "4 warp instructions per SM per cycle at the measured SM clock"}
    if atomics:
        peak = dpm.atomic_roof() / 1e9
        ach = atomics / secs / 1e9
        roofs["l2_atomic"] = {"achieved": ach, "peak": peak, "unit": "G FP64 atomics/s", "frac": ach / peak,
                              "peak_source": "measured (dpmx_atomic_roof, 32 MB array)"}
    if c.get("fp32_flops_per_unit"):
        ach = c["fp32_flops_per_unit"] * units / secs / 1e12
        roofs["fp32"] = {"achieved": ach, "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                         "frac": ach / FP32_NOMINAL_TFLOPS, "peak_source": "nominal"}
    traffic = None
    if c.get("dram_bytes_per_unit"):
        peak, kind = measured_peaks()
        traffic = c["dram_bytes_per_unit"] * units / max(1.0, nl)
        ach = c["dram_bytes_per_unit"] * units / secs / 1e9
        roofs["dram"] = {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "peak_source": kind}
    bound = max(roofs, key=lambda k: roofs[k]["frac"]) if roofs else None
    top = roofs.get(bound, {})
    return {"bound": bound, "kernel": kname, "achieved": top.get("achieved"), "peak": top.get("peak"),
            "unit": top.get("unit"), "frac": top.get("frac"), "traffic": traffic, "roofs": roofs,
            "avg_launch_ms": kms / max(1.0, nl), "units_per_launch": units / max(1.0, nl),
            "unit_name": c.get("unit"),
            "electron_phase_share": pr["electron_ms"] / max(1e-9, pr["total_ms"]),
            "photon_phase_share": pr["photon_ms"] / max(1e-9, pr["total_ms"]),
            "electron_steps_per_s": pr["electron_steps"] / max(1e-9, pr["electron_ms"] * 1e-3),
            "photon_steps_per_s": pr["photon_steps"] / max(1e-9, pr["photon_ms"] * 1e-3)}


# ---------------------------------------------------------------------------
def main():
    a = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if a.impl == "reference":
        if rank != 0:
            return 0
        pool, cores = oracle_pool()
        for w in range(a.warmup):
            oracle_step(pool, cores, max(1, a.cpu_hist // 4), w)
        tot_h, tot_t = 0.0, 0.0
        for k in range(a.steps):
            rate, dt = oracle_step(pool, cores, a.cpu_hist, a.warmup + k)
            tot_h += cores * a.cpu_hist
            tot_t += dt
        pool.close()
        value = tot_h / tot_t
        sample = "%d histories per core per step on %d cores" % (a.cpu_hist, cores)
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * tot_t / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "histories_per_step": cores * a.cpu_hist, "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": "histories/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return 0

    # CPU baseline workers start before the first GPU call (spawned processes)
    pool = cores = None
    if rank == 0:
        pool, cores = oracle_pool()

    import numpy as np
    import torch
    torch.cuda.set_device(local)   # before the process group: each rank's communicator on its own GPU
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dpm = importlib.import_module("dpm-g4cpp_gb300")
    wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
    tables = dpm.Tables(DATA)
    mat = wl.precision_phantom()
    src = wl.precision_source()
    ph = dpm.Phantom.voxels(tables, mat, 2.0)
    H = int(a.hist)
    # a non-default stream: the library captures each run into a CUDA graph on it,
    # and the timing events are recorded on the same stream
    stream = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > L2 (129 MB)

    def seed_of(step):
        return 7 + 1000003 * rank + step

    def one(step, profile=False):
        return dpm.run(tables, [dpm.Job(ph, src, H, seed_of(step))], batches=a.batches, stream=stream.cuda_stream,
                       profile_phases=profile)

    for w in range(a.warmup):
        one(-1 - w).close()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    launches = 0
    stats = []
    torch.cuda.synchronize()
    clocks.begin()
    for k in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))      # L2 flush between timed steps, on the timed stream, before its events
        ev[k][0].record(stream)
        r = one(k)
        ev[k][1].record(stream)
        launches += r.launches
        stats.append(r.stats(0))
        r.close()
    torch.cuda.synchronize()
    clocks.end()
    clk = clocks.stop()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
    ms_max = float(t.item())
    value = world * H * a.steps / (ms_max * 1e-3)

    # e2e through the public API with host buffers: per step the phantom goes
    # host->device from pinned memory and the dose + dose^2 come back into
    # pinned host arrays
    pinned = torch.from_numpy(mat.reshape(-1)).pin_memory().numpy().reshape(mat.shape)
    nbins = int(mat.size)
    out_d = torch.empty(nbins, dtype=torch.float64).pin_memory().numpy()
    out_d2 = torch.empty(nbins, dtype=torch.float64).pin_memory().numpy()
    e2e_steps = max(1, a.steps)   # as many steps as the device-timed loop
    p2 = dpm.Phantom.voxels(tables, pinned, 2.0)   # one untimed step: the first run on the library's own stream
    dpm.run(tables, [dpm.Job(p2, src, H, seed_of(99))], batches=a.batches).close()
    p2.close()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        p2 = dpm.Phantom.voxels(tables, pinned, 2.0)
        r = dpm.run(tables, [dpm.Job(p2, src, H, seed_of(100 + k))], batches=a.batches)
        d, d2, _ = r.tally(0, out=(out_d, out_d2, None))
        r.close()
        p2.close()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * H * e2e_steps / e2e_s, "unit": "histories/s",
           "h2d_bytes_per_step": int(mat.nbytes), "d2h_bytes_per_step": int(2 * d.nbytes)}

    # live roofline of the dominant kernel from a profiled run (every phase launch timed)
    r = one(10**6, profile=True)
    pr = r.profile
    eblock = r.config["electron_kernel"] == 1
    pblock = r.config["photon_kernel"] == 1
    r.close()
    roofline = roofline_of(dpm, pr, eblock, pblock, clk)

    # the plain FP64 GPU form on the same workload and a voxel-by-voxel dose
    # check of the FP32 form against it (both outside the timed region)
    dc = importlib.import_module("dpm-g4cpp_gb300.dosecheck")
    # 10 batches: each FP64 launch carries 1e6 histories and fills the GPU, so
    # the FP64 rate is the form's own (the check's coverage is t-corrected)
    H64, B = int(a.fp64_hist), 10
    r64 = dpm.run(tables, [dpm.Job(ph, src, H64, seed_of(200))], precision=dpm.FP64_PLAIN, batches=B,
                  stream=stream.cuda_stream)
    fp64_rate = world * H64 / (r64.elapsed_ms * 1e-3)
    d64, d64b, _ = r64.tally(0)
    r64.close()
    Hc = int(a.check_hist)
    rc_ = dpm.run(tables, [dpm.Job(ph, src, Hc, seed_of(300))], batches=B, stream=stream.cuda_stream)
    d32, d32b, _ = rc_.tally(0)
    rc_.close()
    m32, s32 = dc.batch_estimate(d32, d32b, B, Hc)
    m64, s64 = dc.batch_estimate(d64, d64b, B, H64)
    check = dc.compare(m32, s32, B, m64, s64, B)
    check.update(fp32_histories=Hc, fp64_histories=H64, batches=B, against="fp64_gpu")
    # Gy-voxels/s: the dose summed over voxels per history [Gy], times histories/s
    rho = np.array([tables.density(int(i)) for i in range(tables.num_materials)], dtype=np.float64)
    mass_kg = rho[mat.reshape(-1)] * (2.0 ** 3) * 1e-3 * 1e-3     # g/cm3 x mm3 -> kg
    gy_per_hist = float((m32.reshape(-1) * 1.602176634e-13 / mass_kg).sum())

    cpu = None
    if rank == 0:
        rate, dt = oracle_step(pool, cores, 5 * a.cpu_hist, 0)
        pool.close()
        cpu = {"value": rate, "unit": "histories/s", "cores": cores, "kind": "port",
               "sample": "%d histories per core on %d cores (%.1f s wall)" % (5 * a.cpu_hist, cores, dt)}
    st = stats[-1]
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64-tally", "data": "synthetic",
            "config": {"workload": WORKLOAD, "histories_per_step": H, "batches": a.batches, "phantom": [256, 128, 128],
                       "voxel_mm": 2.0, "seed": 7, "l2": "flushed between steps (256 MB write)"},
            "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "fp64_gpu": {"value": fp64_rate, "unit": "histories/s", "histories": H64,
                         "form": "plain FP64, one thread per history (dpmx FP64_PLAIN)"},
            "vs_fp64_gpu": value / fp64_rate, "dose_check": check,
            "gy_voxels_per_s": {"value": gy_per_hist * value, "unit": "Gy-voxels/s",
                                "definition": "sum over voxels of the dose per history [Gy] x histories/s"},
            "energy_check": {"max_residual_mev": st.max_residual, "violations": st.residual_violations,
                             "lost": st.lost},
        }))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
