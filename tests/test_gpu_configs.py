"""The two FP64 workloads at their stated lengths, GPU against the oracle.

  dust cluster, N = 1000: 2000 steps, energy every 100 steps (20 rows);
  aggregate collision, N = 5000 (4000-sphere target, 1000-sphere projectile
  at 100 cm/s): 5000 steps, energy every 100 steps (50 rows).

The aggregate collision is the case the workload exists for: the clusters
meet after about 1500 steps, so the later checkpoints compare the impact
itself -- contacts between target and projectile, the loading/unloading
spring switch (ColliderSingleCore.cpp:119-126), sliding and rolling friction
(:160-178) -- bit for bit.  The oracle runs row-parallel on all host cores
(its state is bit-identical to its sequential form and to the reference's
own step, tests/test_oracle_pin.py).

Bars: pos/vel/w/acc/aacc bit-identical at every checkpoint; the contact
set identical at every checkpoint; energy rows as in test_gpu_parity.py
(KE 1e-12 relative, PE 1e-10 relative, momentum and angular momentum 1e-12
of the sum of their terms' magnitudes)."""
import numpy as np
import pytest

from oracle.oracle import CpuOracle
from spacelab_gb300 import GpuStep, configs
from test_gpu_parity import STATE_KEYS, _assert_energy, _state

pytestmark = pytest.mark.gpu


def _run_both(w, checkpoints):
    """Advance the GPU and the oracle over the workload's whole schedule in
    blocks of w.skip steps, the last step of each block a write step; yield
    (step, gpu energy, oracle energy, gpu state or None, oracle state or
    None, sim) at every write step."""
    g = w.group
    sim = GpuStep(g.copy(), w.material, "exact")
    sim.set_scalars(w.dt, w.kin, w.kout)
    o = CpuOracle(g.pos, g.vel, g.w, g.R, g.m, g.moi, w.material, w.dt, w.kin, w.kout)
    e0 = sim.init_conditions()
    eo0 = o.init()
    _assert_energy(e0, eo0, o.state(), g.m, g.moi)
    assert np.array_equal(sim.contacts(), o.contacts())
    step = 0
    try:
        while step < w.steps:
            nblock = min(w.skip, w.steps - step)
            e = sim.step(nblock, write_last=True)
            eo = None
            for k in range(nblock):
                eo = o.step(k == nblock - 1, threads=0)
            step += nblock
            if step in checkpoints:
                yield step, e, eo, _state(sim), o.state(), sim, o
            else:
                yield step, e, eo, None, o.state() if step % w.skip == 0 else None, sim, o
    finally:
        sim.close()
        o.close()


def _check_workload(w, checkpoints, inter_cluster=None):
    rows = 0
    contacts_seen = {}
    for step, e, eo, st, so, sim, o in _run_both(w, checkpoints):
        _assert_energy(e, eo, so, w.group.m, w.group.moi)
        rows += 1
        if st is not None:
            for key in STATE_KEYS:
                assert np.array_equal(st[key], so[key]), (w.name, step, key)
            cg, co = sim.contacts(), o.contacts()
            assert np.array_equal(cg, co), (w.name, step, "contact set")
            if inter_cluster is not None:
                contacts_seen[step] = int(((co[:, 0] >= inter_cluster) & (co[:, 1] < inter_cluster)).sum())
    assert rows == w.steps // w.skip
    return contacts_seen


def test_dust_cluster_n1000_2000_steps_20_energy_rows():
    w = configs.dust_cluster_1000()
    assert (w.n, w.steps, w.skip) == (1000, 2000, 100)
    _check_workload(w, checkpoints=(500, 1000, 1500, 2000))


def test_aggregate_collision_n5000_5000_steps_through_impact():
    w = configs.aggregate_collision_5000()
    assert (w.n, w.steps, w.skip) == (5000, 5000, 100)
    seen = _check_workload(w, checkpoints=(100, 1000, 2000, 3000, 4000, 5000), inter_cluster=4000)
    # the projectile (spheres 4000..4999) touches the target (0..3999):
    # the impact is inside the compared window
    assert seen[100] == 0
    assert max(seen.values()) > 0, seen


def test_polydisperse_cluster_n20000_exact_matches_oracle():
    """The 20000-sphere polydisperse workload (lognormal radii, so every tile
    takes the general, unequal-radius form) in the exact mode: 30 steps with
    a write step every 10, bit-identical to the oracle at steps 10 and 30,
    the contact set identical, energy rows to the usual bars.  (The workload's
    10,000 steps are the mixed forms' drift runs, bench.py --drift-steps.)"""
    w = configs.polydisperse_cluster_20000()
    assert w.n == 20000
    g = w.group
    sim = GpuStep(g.copy(), w.material, "exact")
    sim.set_scalars(w.dt, w.kin, w.kout)
    o = CpuOracle(g.pos, g.vel, g.w, g.R, g.m, g.moi, w.material, w.dt, w.kin, w.kout)
    try:
        _assert_energy(sim.init_conditions(), o.init(), o.state(), g.m, g.moi)
        assert np.array_equal(sim.contacts(), o.contacts())
        for step in range(1, 31):
            write = step % 10 == 0
            e = sim.sim_one_step(write)
            eo = o.step(write, threads=0)
            if write:
                _assert_energy(e, eo, o.state(), g.m, g.moi)
            if step in (10, 30):
                st, so = _state(sim), o.state()
                for key in STATE_KEYS:
                    assert np.array_equal(st[key], so[key]), (step, key)
                assert np.array_equal(sim.contacts(), o.contacts())
    finally:
        sim.close()
        o.close()
