"""Batched solver: one persistent launch for many independent collisions.

SL_MODE_EXACT: every instance's state after the run must be bit-identical
to running that instance alone through the single-system exact step (which
is bit-identical to the reference), and its energy records must agree with
the single-system ones within the parity tests' bar.  SL_MODE_MIXED: within
the mixed-precision bars against the exact batch.
"""
import numpy as np
import pytest

from cases import contact_case
from spacelab_gb300 import BallGroup, GpuStep
from spacelab_gb300 import batch as B

pytestmark = pytest.mark.gpu

STATE = ("pos", "vel", "w", "acc", "aacc")


def _contact_instance(n, seed, mu):
    c = contact_case(n, seed)
    col = B.Collision(n, 0, 0.0, 0.0, np.sqrt(c["kout"] / c["kin"]), mu, seed)
    col.group = BallGroup.from_arrays(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"])
    col.dt, col.kin, col.kout = c["dt"], c["kin"], c["kout"]
    return col


def _instances():
    cols = [_contact_instance(n, 100 + n, mu) for n, mu in ((1, 0.3), (2, 0.1), (33, 0.5), (150, 0.2), (257, 0.4))]
    cols += B.sample_collisions(6, seed=7, nt_range=(20, 180))
    return cols


@pytest.mark.parametrize("shape", [(64, 128), (0, 128)])
def test_exact_batch_matches_single_system_runs(shape):
    """Both exact pair passes -- the per-sphere loop and the pair-tile pass
    (each pair once into per-CTA buffers, then ordered row sums) -- are bit
    for bit the single-system step, hence the reference's."""
    cols = _instances()
    steps, skip = 40, 10
    run = B.BatchRun(cols, "exact", steps=steps, skip=skip)
    run.set_shape(*shape)
    run.run(1, steps, do_init=True)
    assert not run.status().any()
    st = run.state()
    en = run.energy()
    for i, c in enumerate(cols):
        with GpuStep(c.group.copy(), B.instance_material(c), "exact") as s:
            s.set_scalars(c.dt, c.kin, c.kout)
            e0 = s.init_conditions()
            rows = []
            for step in range(1, steps + 1):
                e = s.sim_one_step(step % skip == 0)
                if e is not None:
                    rows.append(e.as_array())
            g = s.download()
        mine = run.instance_state(st, i)
        for k in STATE:
            assert np.array_equal(mine[k], getattr(g, k)), (i, c.n, k)
        ref = np.vstack([e0.as_array()] + rows)
        np.testing.assert_allclose(en[i][:, 1], ref[:, 1], rtol=1e-12)          # KE
        np.testing.assert_allclose(en[i][:, 0], ref[:, 0], rtol=1e-10, atol=1e-300)  # PE
        scale = np.abs(ref[:, 2:]).max() + 1e-300
        assert np.abs(en[i][:, 2:] - ref[:, 2:]).max() <= 1e-10 * scale


def test_batch_shapes_agree_and_autotuner_picks_one():
    cols = _instances()
    results = []
    for tile, threads in ((32, 64), (128, 256), (0, 128), (0, 256)):
        run = B.BatchRun(cols, "exact", steps=10, skip=5)
        run.set_shape(tile, threads)
        run.run(1, 10, do_init=True)
        results.append(run.state())
    for r in results[1:]:  # the pair-tile pass (tile 0) too: bit for bit
        for k in STATE:
            assert np.array_equal(results[0][k], r[k])
    run = B.BatchRun(cols, "exact", steps=10, skip=5)
    tuned = run.autotune(sample_steps=2)
    assert tuned["tile"] in (0, 32, 64, 128) and tuned["threads"] in (64, 128, 256)
    assert len(tuned["times_ms"]) == 12
    assert all(t > 0 for t in tuned["times_ms"].values())
    run.run(1, 10, do_init=True)   # the autotuner restored the initial state
    st = run.state()
    for k in STATE:
        assert np.array_equal(st[k], results[0][k])


@pytest.mark.parametrize("shape", [(64, 128), (0, 256), (0, 64), (0, 128), (0, 512)])
def test_mixed_batch_tracks_exact_batch(shape):
    """Both mixed pair passes: the per-sphere partner loop (j-tiles of 64)
    and the pair-tile pass (tile 0: each pair once, Z-ordered 32-sphere
    blocks, contacts in the reference's orientation)."""
    cols = _instances()
    ex = B.BatchRun(cols, "exact", steps=40, skip=10)
    mx = B.BatchRun(cols, "mixed_df", steps=40, skip=10)
    mx.set_shape(*shape)
    ex.run(1, 40, True)
    mx.run(1, 40, True)
    se, sm = ex.state(), mx.state()
    ee, em = ex.energy(), mx.energy()
    for i, c in enumerate(cols):
        a, b = ex.instance_state(se, i), mx.instance_state(sm, i)
        # contact-rich instances separate through the kin/kout switch
        # (tests/test_gpu_mixed.py); the sampled collisions are smooth here
        contact_rich = c.n_p == 0
        tol_pos, tol_E = (1e-3, 1e-3) if contact_rich else (1e-6, 1e-6)
        assert np.abs(b["pos"] - a["pos"]).max() <= tol_pos * c.group.R.max(), i
        E = ee[i][:, 0] + ee[i][:, 1]
        Em = em[i][:, 0] + em[i][:, 1]
        assert np.abs(Em - E).max() <= tol_E * np.abs(E).max(), i


def test_mixed_batch_autotuner_includes_pair_tiles():
    cols = _instances()
    run = B.BatchRun(cols, "mixed_df", steps=10, skip=5)
    tuned = run.autotune(sample_steps=2)
    assert len(tuned["times_ms"]) == 12 and all(t > 0 for t in tuned["times_ms"].values())
    assert tuned["tile"] in (0, 32, 64, 128)
    run.run(1, 10, do_init=True)
    assert not run.status().any()
