"""Generates the golden vectors in this directory from the reference's own
simulation code (oracle/_ref/libdpm_ref.so, built from the reference sources by
oracle/build_ref.sh) on the committed data set data/water_ti_bone.

    python tests/golden/make_golden.py [reference-root]

Contents of golden_water_ti_bone.npz:
  tab_E, tab_<q>_<imat>         interpolated tables (quantity codes of dpmx_table_eval)
  smp_<s>_<imat>_{E,R,out}      samplers fed with the uniforms R (codes of dpmx_sampler_eval)
  slab_<name>_{edep,steps}      full-precision depth histograms of the reference
                                history loop (mt19937 with the given seed)
  cli_hist                      hist.sim text of the unmodified Simulate (100 e-)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import cpu_oracle  # noqa: E402

DATA = os.path.join(ROOT, "data", "water_ti_bone")
OUT = os.path.join(HERE, "golden_water_ti_bone.npz")

# (name, particle e-?, energy, lbox, geometry, histories, seed)
SLAB_RUNS = [
    ("e15_c3", True, 15.0, 1.0, 3, 1000, 12345),
    ("g15_c3", False, 15.0, 1.0, 3, 1500, 777),
    ("e6_c0_b2", True, 6.0, 2.0, 0, 500, 5),
    ("e20_c1", True, 20.0, 1.0, 1, 300, 99),
]


def main(ref_root=None):
    ref_root = ref_root or cpu_oracle.reference_root()
    cpu_oracle.build_ref(ref_root)
    ref = cpu_oracle.Reference(DATA)
    rng = np.random.default_rng(2024)
    out = {}
    E = np.exp(np.linspace(np.log(0.01), np.log(25.0), 1200))
    E = np.concatenate([E, [0.198, 0.2, 0.0495, 0.05, 20.999999, 21.0, 0.4, 1.022]])
    out["tab_E"] = E
    for q in range(9):
        for im in range(3):
            out["tab_%d_%d" % (q, im)] = ref.table(q, E, im)
    # sampler energy ranges where the reference samplers are defined
    ranges = {0: (0.0501, 20.99), 1: (0.4001, 20.99), 2: (0.0501, 20.99), 3: (0.2001, 20.99)}
    for s, (lo, hi) in ranges.items():
        for im in range(3):
            Es = np.exp(rng.uniform(np.log(lo), np.log(hi), 1500))
            R = rng.random((1500, 3))
            out["smp_%d_%d_E" % (s, im)] = Es
            out["smp_%d_%d_R" % (s, im)] = R
            out["smp_%d_%d_out" % (s, im)] = ref.sampler(s, Es, R, im)
    for name, ise, e, lbox, geom, n, seed in SLAB_RUNS:
        ed, st = ref.simulate_full(n, e, ise, lbox, geom, seed)
        out["slab_%s_edep" % name] = ed
        out["slab_%s_steps" % name] = st
    # the unmodified Simulate writes hist.sim (5 significant digits); it must
    # agree with the restated history loop above
    tmp = os.path.join(HERE, "_hist_tmp.sim")
    ref.simulate_cli(100, 15.0, True, 1.0, 3, tmp, seed=4242)
    with open(tmp) as f:
        out["cli_hist"] = np.array(f.read())
    os.remove(tmp)
    ed, st = ref.simulate_full(100, 15.0, True, 1.0, 3, 4242)
    out["cli_full_edep"] = ed
    out["cli_full_steps"] = st
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(*sys.argv[1:])
