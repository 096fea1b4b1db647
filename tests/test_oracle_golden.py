"""The CPU oracle against the reference's own outputs (golden vectors made by
tests/golden/make_golden.py from the reference sources): bit-for-bit."""
import numpy as np
import pytest

from conftest import GOLDEN

SLAB_RUNS = [
    ("e15_c3", True, 15.0, 1.0, 3, 1000, 12345),
    ("g15_c3", False, 15.0, 1.0, 3, 1500, 777),
    ("e6_c0_b2", True, 6.0, 2.0, 0, 500, 5),
    ("e20_c1", True, 20.0, 1.0, 1, 300, 99),
]


@pytest.mark.parametrize("q", range(9))
@pytest.mark.parametrize("imat", range(3))
def test_tables_bit_exact(golden, oracle_c3, q, imat):
    E = golden["tab_E"]
    np.testing.assert_array_equal(oracle_c3.table(q, E, imat), golden["tab_%d_%d" % (q, imat)])


@pytest.mark.parametrize("s", range(4))
@pytest.mark.parametrize("imat", range(3))
def test_samplers_bit_exact(golden, oracle_c3, s, imat):
    k = "smp_%d_%d_" % (s, imat)
    out = oracle_c3.sampler(s, golden[k + "E"], golden[k + "R"], imat)
    np.testing.assert_array_equal(out, golden[k + "out"])


@pytest.mark.parametrize("run", SLAB_RUNS, ids=[r[0] for r in SLAB_RUNS])
def test_slab_transport_bit_exact(golden, oracle_c3, run):
    name, ise, e, lbox, geom, n, seed = run
    ed, st, stats = oracle_c3.simulate_slab(n, e, ise, lbox, geom, seed)
    np.testing.assert_array_equal(ed, golden["slab_%s_edep" % name])
    np.testing.assert_array_equal(st, golden["slab_%s_steps" % name])


@pytest.mark.parametrize("run", SLAB_RUNS, ids=[r[0] for r in SLAB_RUNS])
def test_voxel_geometry_reproduces_reference_geom(golden, oracle_c3, run):
    """The oracle's 3-D voxel geometry, laid out as the reference's own lattice
    (voxels of lbox centred on integer multiples of lbox, world |x|,|y| <= 100
    mm and -lbox <= z <= 100 mm, Geom.cc:20-28, each voxel holding the slab
    material of its depth, Geom.cc:133-164), reproduces the unmodified
    reference's depth histograms bit for bit: the voxel boundary arithmetic,
    3-D material lookup and 3-D scoring are Geom's."""
    name, ise, e, lbox, geom, n, seed = run
    ed, st, stats = oracle_c3.simulate_voxel_slabref(n, e, ise, lbox, geom, seed)
    np.testing.assert_array_equal(ed, golden["slab_%s_edep" % name])
    np.testing.assert_array_equal(st, golden["slab_%s_steps" % name])


def test_restated_loop_matches_unmodified_simulate(golden):
    """The full-precision history loop used for the goldens reproduces the
    unmodified Simulate's hist.sim (5 significant digits)."""
    text = str(golden["cli_hist"])
    rows = [l.split() for l in text.splitlines() if not l.startswith("#")]
    ed = golden["cli_full_edep"]
    st = golden["cli_full_steps"]
    assert len(rows) == len(ed)
    norm = 1.0 / (100 * 1.0 * 0.1)
    dens = {0: 1.0, 1: 4.54, 2: 1.85}
    for i, r in enumerate(rows):
        iz = int(r[0])
        m = 0 if iz < 10 else (1 if iz < 15 else (2 if iz < 25 else 0))
        assert float(r[2]) == pytest.approx(ed[i] * norm / dens[m], rel=6e-5, abs=1e-30)
        assert float(r[3]) == pytest.approx(st[i] / 100, rel=6e-5, abs=1e-30)


def test_golden_physics_sanity(golden):
    """The generated data reproduce the reference fixture's scale: ~13.7 MeV of
    15 MeV deposited per e- history and ~130 scoring steps per history
    (tests/WaterTiBoneWater_15MeV/hist.sim of the reference: 13.661, 129.99)."""
    ed = golden["slab_e15_c3_edep"]
    st = golden["slab_e15_c3_steps"]
    assert ed.sum() / 1000 == pytest.approx(13.661, rel=0.03)
    assert st.sum() / 1000 == pytest.approx(129.99, rel=0.05)
