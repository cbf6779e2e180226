"""The mixed-precision forms against the FP64 exact form on the same inputs:
"mixed" (SL_MODE_MIXED: FP32 force and torque arithmetic, FP64 pair
subtraction, close-pair overlaps and per-sphere accumulation) and
"mixed_df" (SL_MODE_MIXED_DF: the double-float variant).  The exact form is bit-identical to the reference step
(tests/test_gpu_parity.py), so these bound the mixed form's error against
the reference.  Bars (stated per quantity):
  * step-0 contact set identical;
  * step-0 accelerations within 2e-5 of the largest |acc| (FP32 pair math,
    relative error ~1e-6 per term);
  * smooth (vdW-dominated) dynamics -- the polydisperse cluster: total
    energy E = PE + KE tracks the FP64 run within 1e-6 relative;
  * stiff contact-rich dynamics: the reference's loading/unloading switch
    (k = kin or kout by the sign of the distance change) is discontinuous, so
    a 1e-7 force difference can flip k for a pair at its turning point; the
    runs then separate like two FP64 runs in different summation orders
    would.  Bars there: E within 1e-2 of |E0|, positions within 1e-2 radii
    after 100 steps, and no worse than an FP64 run whose initial positions
    differ from the reference run's in the last bit (measured alongside).
"""
import numpy as np
import pytest

from cases import contact_case, material, two_sphere_case
from spacelab_gb300 import BallGroup, GpuStep, configs

pytestmark = pytest.mark.gpu

MIXED_MODES = ("mixed", "mixed_df")


def _sim(c, mode):
    g = BallGroup.from_arrays(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"])
    s = GpuStep(g, material(), mode)
    s.set_scalars(c["dt"], c["kin"], c["kout"])
    return s


# 6500 and 7000 spheres: 20,910 and 24,090 block tiles, enough for the pair
# kernel to take two column blocks per work item on a GB300
# (mixed_pair_double); 204 row blocks (the last of 4 spheres) and 219 (an odd
# count, with empty items)
@pytest.mark.parametrize("mode", MIXED_MODES)
@pytest.mark.parametrize("n,seed", [(2, 1), (65, 2), (300, 3), (6500, 5), (7000, 4)])
def test_mixed_step0_forces_and_contacts(n, seed, mode):
    c = contact_case(n, seed)
    ex, mx = _sim(c, "exact"), _sim(c, mode)
    assert ex.pair_kernel() == "pair_tile_kernel"
    if mode == "mixed":
        assert mx.pair_kernel() == "mixed64_pair_kernel"
    else:
        assert mx.pair_kernel() == ("mixed_pair2_kernel" if n >= 6500 else "mixed_pair_kernel")
    ee, em = ex.init_conditions(), mx.init_conditions()
    assert np.array_equal(ex.contacts(), mx.contacts())
    ge, gm = ex.download(), mx.download()
    scale = np.abs(ge.acc).max()
    assert np.abs(gm.acc - ge.acc).max() <= 2e-5 * scale
    ascale = np.abs(ge.aacc).max() + 1e-300
    assert np.abs(gm.aacc - ge.aacc).max() <= 2e-5 * ascale
    assert abs(em.PE - ee.PE) <= 1e-5 * abs(ee.PE)
    assert abs(em.KE - ee.KE) <= 1e-12 * ee.KE


@pytest.mark.parametrize("mode", MIXED_MODES)
def test_mixed_trajectory_and_energy_track_fp64(mode):
    # contact-rich: the loading/unloading spring switch amplifies any
    # difference, so the bars are on energy (1% of |E0|) and position (1% of
    # a radius) over 100 steps, not on single-step round-off
    c = contact_case(400, 7, vel_sigma=30.0)
    ex, mx = _sim(c, "exact"), _sim(c, mode)
    e0 = ex.init_conditions()
    mx.init_conditions()
    E0 = e0.PE + e0.KE
    dev_mixed = 0.0
    for step in range(1, 101):
        write = step % 10 == 0
        a = ex.sim_one_step(write)
        b = mx.sim_one_step(write)
        if write:
            dev_mixed = max(dev_mixed, abs((b.PE + b.KE) - (a.PE + a.KE)))
    assert dev_mixed <= 1e-2 * abs(E0)
    ge, gm = ex.download(), mx.download()
    assert np.abs(gm.pos - ge.pos).max() <= 1e-2 * c["R"].max()


@pytest.mark.parametrize("mode", MIXED_MODES)
@pytest.mark.parametrize("n", [256, 7000])
def test_mixed_looper_is_deterministic(n, mode):
    c = contact_case(n, 9)
    a, b = _sim(c, mode), _sim(c, mode)
    a.init_conditions(); b.init_conditions()
    ra = a.sim_looper(steps=41, skip=10)
    rb = b.sim_looper(steps=41, skip=10)
    assert [r.E for r in ra] == [r.E for r in rb]
    ga, gb = a.download(), b.download()
    assert np.array_equal(ga.pos, gb.pos) and np.array_equal(ga.vel, gb.vel)


@pytest.mark.parametrize("mode", MIXED_MODES)
def test_mixed_polydisperse_cluster_energy_tracks_fp64(mode):
    """The polydisperse workload's radius spread (0.5-2 x median) at a
    smaller N: 200 steps, energy within 1e-6 of the FP64 run."""
    g = configs.build_cluster(3000, 11, sigma_v=1e-2, sigma_ln=0.2)
    kin, kout, dt = configs.spring_and_dt(float(g.R.max()), float(g.m.min()), 1.0)
    c = dict(pos=g.pos, vel=g.vel, w=g.w, R=g.R, m=g.m, moi=g.moi, dt=dt, kin=kin, kout=kout)
    ex, mx = _sim(c, "exact"), _sim(c, mode)
    e0 = ex.init_conditions()
    mx.init_conditions()
    ra = ex.sim_looper(steps=201, skip=50)
    rb = mx.sim_looper(steps=201, skip=50)
    E0 = abs(e0.PE + e0.KE)
    for x, y in zip(ra, rb):
        assert abs(x.E - y.E) <= 1e-6 * E0


@pytest.mark.parametrize("mode", MIXED_MODES)
@pytest.mark.parametrize("spacing", [2.9, 4.6, 9.0])
def test_mixed_separated_lattice_forces_and_potential(spacing, mode):
    """Jittered lattices whose nearest pairs sit at about 1.3-1.6, 2.1-2.5
    and 4.1-5 radii sums, out of contact: every pair takes the FP32 far-pair
    force path (no square root), and at the two wider spacings every pair's
    write-step potential comes from the FP32 series of the vdW bracket.
    Bars: accelerations within 1e-5 of the largest, PE within 5e-6
    relative."""
    c = contact_case(343, 21, spacing=spacing, r_spread=0.1)
    ex, mx = _sim(c, "exact"), _sim(c, mode)
    ee, em = ex.init_conditions(), mx.init_conditions()
    assert len(ex.contacts()) == 0 and len(mx.contacts()) == 0
    ge, gm = ex.download(), mx.download()
    scale = np.abs(ge.acc).max()
    assert np.abs(gm.acc - ge.acc).max() <= 1e-5 * scale
    assert abs(em.PE - ee.PE) <= 5e-6 * abs(ee.PE)


@pytest.mark.parametrize("mode", MIXED_MODES)
@pytest.mark.parametrize("gap", [0.2, 0.25 * (1 - 1e-6), 0.25, 0.25 * (1 + 1e-6), 0.3])
def test_mixed_far_pair_threshold_is_seamless(gap, mode):
    """Two spheres at |r| = (1 + gap) (R_A + R_B) around the far-pair
    threshold, 1.25 radii sums for these radii and h_min: below it the pair
    takes the double-float close path and its potential is FP64, above it the
    FP32 force without a square root and the FP32 series of the vdW bracket.
    Both sides must agree with the FP64 exact form to the far-pair bars:
    accelerations within 1e-5, PE within 5e-6 relative."""
    c = two_sphere_case(gap)
    ex, mx = _sim(c, "exact"), _sim(c, mode)
    ee, em = ex.init_conditions(), mx.init_conditions()
    assert len(ex.contacts()) == 0 and len(mx.contacts()) == 0
    ge, gm = ex.download(), mx.download()
    scale = np.abs(ge.acc).max()
    assert scale > 0
    assert np.abs(gm.acc - ge.acc).max() <= 1e-5 * scale
    assert abs(em.PE - ee.PE) <= 5e-6 * abs(ee.PE)


@pytest.mark.parametrize("mode", MIXED_MODES)
def test_mixed_polydisperse_n20000_energy_and_trajectory_track_fp64(mode):
    """The polydisperse workload itself (N = 20000, lognormal radii) over the
    first 1000 of its 10000 steps, energy every 100 steps: E = PE + KE of
    the mixed run within 1e-6 of |E0| of the FP64 run at every write step,
    positions within 1e-6 of a radius after 1000 steps.  The full 10000
    steps are bench.py --drift-steps 10000."""
    w = configs.polydisperse_cluster_20000()
    g = w.group
    c = dict(pos=g.pos, vel=g.vel, w=g.w, R=g.R, m=g.m, moi=g.moi, dt=w.dt, kin=w.kin, kout=w.kout)
    ex, mx = _sim(c, "exact"), _sim(c, mode)
    e0 = ex.init_conditions()
    mx.init_conditions()
    ra = ex.sim_looper(steps=1001, skip=w.skip)
    rb = mx.sim_looper(steps=1001, skip=w.skip)
    assert len(ra) == len(rb) == 10
    E0 = abs(e0.PE + e0.KE)
    worst = max(abs(x.E - y.E) for x, y in zip(ra, rb)) / E0
    assert worst <= 1e-6, worst
    ge, gm = ex.download(), mx.download()
    assert np.abs(gm.pos - ge.pos).max() <= 1e-6 * float(g.R.max())
