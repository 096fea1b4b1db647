"""Times the unmodified reference dpm_Simulate (oracle/_ref/dpm_Simulate, built
from the reference sources by build_ref.sh) on the reference's CLI workload,
and the oracle restatement (the CPU port that bench.py times on machines
without the reference sources) on the same workload and the same cores.
TEST INFRASTRUCTURE: a measurement recipe, not part of the library.

Workload (the reference's own default case): data set water_ti_bone (the
generated -c 3 data), 15 MeV e- pencil beam, 1 mm voxels, slab geometry 3
(Water/Ti/Bone/Water), seed 123 (the reference's fixed seed).

  python oracle/time_reference.py [--hist 100000] [--procs N]

Prints one JSON line: histories/s of (i) the unmodified CLI in one process on
one core, (ii) N concurrent CLI processes, each running hist/N histories (the
reference has one global RNG and no seed flag, so every process replays the
same stream: a timing of throughput, not N independent estimates), (iii) the
oracle port in one process, (iv) the port in N processes on disjoint history
shares (spawned workers, timed around the work alone), and the CPU model. On a
machine without the reference sources only (iii) and (iv) are timed.
"""
import argparse
import json
import multiprocessing as mp
import os
import platform
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DATA = os.path.join(ROOT, "data", "water_ti_bone")
sys.path.insert(0, HERE)


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def time_cli(n, procs):
    cli = os.path.join(HERE, "_ref", "dpm_Simulate")
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        ps = [subprocess.Popen([cli, "-p", "e-", "-e", "15", "-n", str(n // procs), "-d", DATA, "-b", "1", "-c",
                                "3", "-o", os.path.join(d, "h%d.sim" % k)],
                               stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL) for k in range(procs)]
        rcs = [p.wait() for p in ps]
        dt = time.perf_counter() - t0
    if any(rcs):
        raise RuntimeError("reference CLI failed: %s" % rcs)
    return procs * (n // procs) / dt


def _port(args):
    n, seed = args
    import cpu_oracle
    o = cpu_oracle.Oracle(DATA)
    if n == 0:
        return 0.0
    t0 = time.perf_counter()
    o.simulate_slab(n, 15.0, True, 1.0, 3, seed)
    return time.perf_counter() - t0


def time_port(n, procs):
    import cpu_oracle
    cpu_oracle.build()
    with mp.get_context("spawn").Pool(procs) as pool:
        pool.map(_port, [(0, 0)] * procs)             # start the workers and load the tables
        t0 = time.perf_counter()
        pool.map(_port, [(n // procs, 123 + k) for k in range(procs)])
        dt = time.perf_counter() - t0
    return procs * (n // procs) / dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--hist", type=int, default=100000)
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    have_ref = os.path.exists(os.path.join(HERE, "_ref", "dpm_Simulate"))
    if not have_ref:
        import cpu_oracle
        have_ref = bool(cpu_oracle.build_ref()) and os.path.exists(os.path.join(HERE, "_ref", "dpm_Simulate"))
    res = {
        "workload": "dpm_Simulate -p e- -e 15 -n %d -b 1 -c 3 (water_ti_bone data, seed 123)" % a.hist,
        "cpu": cpu_model(), "cores": os.cpu_count(), "procs": a.procs, "unit": "histories/s",
        "port_1proc": time_port(a.hist, 1),
        "port_nproc": time_port(a.hist, a.procs),
    }
    if have_ref:
        res["reference_cli_1proc"] = time_cli(a.hist, 1)
        res["reference_cli_nproc"] = time_cli(a.hist, a.procs)
        res["port_over_reference_1proc"] = res["port_1proc"] / res["reference_cli_1proc"]
        res["port_over_reference_nproc"] = res["port_nproc"] / res["reference_cli_nproc"]
    else:
        res["reference_cli"] = "unavailable: the reference sources are not on this machine (build_ref.sh cannot build the CLI)"
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
