"""Measurements of the five workloads beyond the headline benchmark.

    python dpm-g4cpp_gb300/measure.py [precision|slab|batching|differentiation|full|phases] ... [--quick]

Each prints one JSON line. The workloads are synthetic, with the shapes of the
reference's configurations:

  slab            15 MeV e- pencil beam on the Water/Ti/Bone/Water slab (1 mm
                  depth bins), FP64 plain form vs FP32 event form
  precision       128x128x256 x 2 mm heterogeneous phantom, 10x10 cm2 photon
                  beam U[1,20] MeV: FP32 event form vs FP64 plain form, dose
                  agreement in voxels above 10 % of the maximum
  batching        64 independent jobs in one graph-captured run, against the
                  same jobs run one at a time
  differentiation 128^3 phantom, 20x20 grid of 6 MeV beamlets: beamlet-tagged
                  run, CSR influence matrix, A w and A^T g, a few gradient steps
  full            512x512x256 x 1 mm CT-like phantom, 16 jobs, 1e9 histories
  phases          the precision workload at --hist histories with every phase
                  launch timed: the unit counts behind a profiler capture
  deposit         deposited energy per history, FP32 against FP64, for photon
                  and electron sources (ten runs of each form, --seed)
"""
import argparse
import importlib
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
dpm = importlib.import_module("dpm-g4cpp_gb300")
wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
DATA_WLB = os.path.join(ROOT, "data", "water_lung_bone")
DATA_WTB = os.path.join(ROOT, "data", "water_ti_bone")
DATA_WLBA = os.path.join(ROOT, "data", "water_lung_bone_air")


def emit(d):
    print(json.dumps(d), flush=True)


dc = importlib.import_module("dpm-g4cpp_gb300.dosecheck")


def compare(d1, q1, n1, d2, q2, n2, batches=10):
    """Agreement of two runs' dose estimates (tallies of `batches` batches) in
    the voxels above 10 % of the maximum (dosecheck.compare)."""
    a, sa = dc.batch_estimate(d1, q1, batches, n1)
    b, sb = dc.batch_estimate(d2, q2, batches, n2)
    return dc.compare(a, sa, batches, b, sb, batches)


def run_timed(tables, jobs, **kw):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = dpm.run(tables, jobs, **kw)
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def slab(quick):
    t = dpm.Tables(DATA_WTB)
    ph = dpm.Phantom.slab(t, 3, 1.0)
    src = dpm.Source(particle=-1, e0=15.0, e1=15.0)
    n64 = 10**5 if quick else 10**6
    n32 = 10**6 if quick else 10**7
    r64, w64 = run_timed(t, [dpm.Job(ph, src, n64, 12345)], precision=dpm.FP64_PLAIN, batches=10)
    r32, w32 = run_timed(t, [dpm.Job(ph, src, n32, 12345)], batches=10)
    a64, q64, _ = r64.tally(0)
    a32, q32, _ = r32.tally(0)
    emit({"workload": "slab: 15 MeV e- pencil, Water/Ti/Bone/Water, 1 mm bins",
          "fp64_hist_per_s": n64 / (r64.elapsed_ms * 1e-3), "fp32_hist_per_s": n32 / (r32.elapsed_ms * 1e-3),
          "speedup_fp32_over_fp64": (n32 / r32.elapsed_ms) / (n64 / r64.elapsed_ms),
          "fp64_histories": n64, "fp32_histories": n32,
          "edep_per_history_fp64": r64.stats(0).edep / n64, "edep_per_history_fp32": r32.stats(0).edep / n32,
          "dose_fp32_vs_fp64": compare(a32, q32, n32, a64, q64, n64)})


def precision(quick):
    t = dpm.Tables(DATA_WLB)
    mat = wl.precision_phantom()
    ph = dpm.Phantom.voxels(t, mat, 2.0)
    src = wl.precision_source()
    n64 = 10**6 if quick else 2 * 10**7
    n32 = 10**7 if quick else 10**8
    r64, _ = run_timed(t, [dpm.Job(ph, src, n64, 7)], precision=dpm.FP64_PLAIN, batches=10)
    r32, _ = run_timed(t, [dpm.Job(ph, src, n32, 7)], batches=10)
    a64, q64, _ = r64.tally(0)
    a32, q32, _ = r32.tally(0)
    st = r32.stats(0)
    emit({"workload": "precision: 128x128x256 x 2 mm, 10x10 cm2 photons U[1,20] MeV",
          "fp64_hist_per_s": n64 / (r64.elapsed_ms * 1e-3), "fp32_hist_per_s": n32 / (r32.elapsed_ms * 1e-3),
          "speedup_fp32_over_fp64": (n32 / r32.elapsed_ms) / (n64 / r64.elapsed_ms),
          "fp64_histories": n64, "fp32_histories": n32,
          "energy_check": {"max_residual_mev": st.max_residual, "violations": st.residual_violations, "lost": st.lost},
          "dose_fp32_vs_fp64": compare(a32, q32, n32, a64, q64, n64)})


def phases(quick, hist=1e6):
    """The precision workload at `hist` histories, run twice (the first warms
    up); the second run launches every phase kernel outside a graph and
    prints its phase profile: the electron sub-steps and photon steps of
    exactly the launches a profiler captures from that run."""
    t = dpm.Tables(DATA_WLB)
    ph = dpm.Phantom.voxels(t, wl.precision_phantom(), 2.0)
    src = wl.precision_source()
    for k in range(2):
        r = dpm.run(t, [dpm.Job(ph, src, int(hist), 7 + k)], batches=10, profile_phases=True)
    emit({"workload": "precision phases", "histories": int(hist), "profile": r.profile, "config": r.config})


def deposit(quick, seed0=11):
    """Deposited energy per history, FP32 event form against the plain FP64
    form, per source, on a 128x128x256 x 2 mm water box: ten independent runs
    of each form (4e6 FP32 and 1e6 FP64 histories each, a tenth with --quick),
    the mean and its standard error from their spread."""
    t = dpm.Tables(DATA_WLB)
    water = np.zeros((256, 128, 128), dtype=np.uint8)
    ph = dpm.Phantom.voxels(t, water, 2.0)
    broad = dict(particle=0, spectrum=0, shape=1, fx=100.0, fy=100.0)
    cases = [("photons 1-20 MeV", wl.precision_source())]
    cases += [("photons %g MeV" % e, dpm.Source(e0=e, e1=e, **broad)) for e in (2.0, 6.0, 10.0, 15.0, 19.0)]
    cases += [("electrons %g MeV" % e, dpm.Source(particle=-1, e0=e, e1=e)) for e in (15.0, 19.0)]
    K = 10
    n32, n64 = (400_000, 100_000) if quick else (4_000_000, 1_000_000)
    for name, src in cases:
        out = {}
        for prec, n in ((dpm.FP32_EVENT, n32), (dpm.FP64_PLAIN, n64)):
            v = []
            for k in range(K):
                r = dpm.run(t, [dpm.Job(ph, src, n, seed0 + k, first_history=k * n)], precision=prec, batches=1)
                v.append(r.stats(0).edep / n)
                r.close()
            out[prec] = (float(np.mean(v)), float(np.std(v, ddof=1) / math.sqrt(K)))
        (a, sa), (b, sb) = out[dpm.FP32_EVENT], out[dpm.FP64_PLAIN]
        emit({"workload": "deposited energy per history, water box", "source": name, "fp32_mev": a, "fp64_mev": b,
              "diff_pct": 100.0 * (a - b) / b, "z": (a - b) / math.hypot(sa, sb)})


def batching(quick):
    t = dpm.Tables(DATA_WLB)
    jobs, phantoms = wl.batching_jobs(t, scale=0.1 if quick else 1.0)
    total = sum(j.histories for j in jobs)
    r, wall = run_timed(t, jobs, batches=10)
    batched_ms = r.elapsed_ms
    lost = sum(r.stats(j).lost for j in range(len(jobs)))
    r.close()
    ra, wall_a = run_timed(t, jobs, batches=10, autotune=True)
    tuned_ms, tuned_cfg = ra.elapsed_ms, ra.config
    ra.close()
    seq_ms, seq_wall = 0.0, 0.0
    for j in jobs:
        rj, wj = run_timed(t, [j], batches=10)
        seq_ms += rj.elapsed_ms
        seq_wall += wj
        rj.close()
    emit({"workload": "batching: 64 jobs (edges 32-192 x 2 mm, e-/photon, 4-20 MeV)", "histories": total,
          "batched_hist_per_s": total / (batched_ms * 1e-3), "batched_wall_s": wall,
          "autotuned_hist_per_s": total / (tuned_ms * 1e-3), "autotuned_config": tuned_cfg,
          "autotuned_wall_s": wall_a,
          "sequential_hist_per_s": total / (seq_ms * 1e-3), "sequential_wall_s": seq_wall,
          "speedup_batched_over_sequential": seq_ms / batched_ms, "lost": lost})


def differentiation(quick):
    import torch
    infl = importlib.import_module("dpm-g4cpp_gb300.influence")
    t = dpm.Tables(DATA_WLB)
    n = 64 if quick else 128
    mat, src, target = wl.differentiation_setup(n=n)
    ph = dpm.Phantom.voxels(t, mat, 2.0)
    per = 10**4 if quick else 2 * 10**5
    nb = src.nbx * src.nby
    r, wall = run_timed(t, [dpm.Job(ph, src, per * nb, 4)], batches=1, tag_beamlets=True)
    t0 = time.perf_counter()
    A = r.influence(0)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    w = torch.ones(nb, dtype=torch.float64, device="cuda", requires_grad=True)
    # dose in Gy per unit beamlet weight: energy per beamlet history -> Gy
    scale = torch.tensor(wl.dose_gy(np.ones(mat.shape), mat, [t.density(k) for k in range(t.num_materials)], 8.0,
                                    per).reshape(-1), device="cuda")
    T = torch.tensor(target.reshape(-1), device="cuda")
    reps = 20
    for _ in range(3):     # warm-up (the first backward starts autograd's worker thread)
        D = infl.dose(A, w)
        (D.sum()).backward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        D = infl.dose(A, w)
        (D.sum()).backward()
    torch.cuda.synchronize()
    fb_ms = 1e3 * (time.perf_counter() - t0) / reps
    # finite-difference check of A^T g on a random direction
    g = torch.randn(A.rows, dtype=torch.float64, device="cuda")
    w0 = torch.rand(nb, dtype=torch.float64, device="cuda")
    v = torch.randn(nb, dtype=torch.float64, device="cuda")
    eps = 1e-3
    fd = ((A.matvec(w0 + eps * v) - A.matvec(w0 - eps * v)) @ g) / (2 * eps)
    an = A.rmatvec(g) @ v
    fd_rel = float(abs(fd - an) / abs(an))
    # projected gradient steps on 1/2 |s A w - T|^2, with s chosen so that unit
    # weights give the target's 2 Gy at the hottest target voxel
    with torch.no_grad():
        d1 = A.matvec(torch.ones(nb, dtype=torch.float64, device="cuda")) * scale
        s = 2.0 / float(d1[T > 0].max())
    wopt = torch.ones(nb, dtype=torch.float64, device="cuda", requires_grad=True)
    opt = torch.optim.Adam([wopt], lr=0.05)
    losses = []
    for _ in range(50):
        opt.zero_grad()
        D = infl.dose(A, wopt) * (scale * s)
        loss = 0.5 * ((D - T) ** 2).sum()
        loss.backward()
        opt.step()
        with torch.no_grad():
            wopt.clamp_(min=0.0)
        losses.append(float(loss.detach()))
    emit({"workload": "differentiation: %d^3 x 2 mm, 20x20 beamlets of 6 MeV photons" % n,
          "histories": per * nb, "tagged_hist_per_s": per * nb / (r.elapsed_ms * 1e-3), "tagged_wall_s": wall,
          "csr": {"rows": A.rows, "cols": A.cols, "nnz": A.nnz, "build_s": build_s},
          "forward_backward_ms": fb_ms, "fd_vs_backward_rel": fd_rel,
          "objective_first_last": [losses[0], losses[-1]]})


def full(quick):
    t = dpm.Tables(DATA_WLBA)
    nx, nz = (128, 64) if quick else (512, 256)
    mat = wl.full_scale_phantom(nx=nx, ny=nx, nz=nz, v=512.0 / nx)
    ph = dpm.Phantom.voxels(t, mat, 512.0 / nx)
    src = wl.full_scale_source()
    total = 10**7 if quick else 10**9
    jobs = [dpm.Job(ph, src, total // 16, 99 + k) for k in range(16)]
    r, wall = run_timed(t, jobs, batches=10)
    lost = sum(r.stats(j).lost for j in range(16))
    emit({"workload": "full: %dx%dx%d CT-like phantom, 10x10 cm2 photons p(E)~(20-E), 16 jobs" % (nx, nx, nz),
          "histories": total, "hist_per_s": total / (r.elapsed_ms * 1e-3), "graph_ms": r.elapsed_ms,
          "wall_s": wall, "launches": r.launches, "lost": lost})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", nargs="*", default=["slab", "precision", "batching", "differentiation", "full"])
    ap.add_argument("--quick", action="store_true", help="reduced sizes")
    ap.add_argument("--hist", type=float, default=1e6, help="histories of the phases run")
    ap.add_argument("--seed", type=int, default=11, help="first seed of the deposit runs")
    a = ap.parse_args()
    fns = {"slab": slab, "precision": precision, "batching": batching, "differentiation": differentiation,
           "full": full, "phases": lambda q: phases(q, a.hist), "deposit": lambda q: deposit(q, a.seed)}
    for w in a.what:
        fns[w](a.quick)
        dpm.scratch_release()


if __name__ == "__main__":
    main()
