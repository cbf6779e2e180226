"""Parity of the GPU exact step with the oracle (which is pinned to the
reference's own sim_one_step, tests/test_oracle_pin.py).

Bar: positions, velocities, spins, acc and aacc bit-identical (the exact
mode reproduces the reference's operation order and IEEE rounding).
Energy totals are sums the GPU forms in another order (a reduction tree
instead of the reference's running sum), so they are compared against the
magnitude of their terms: |dKE| <= 1e-12 KE; each momentum and angular-
momentum component within 1e-12 x sum_i |term_i| (the totals themselves
cancel to ~0 for a system at rest); PE (10^7 mixed-sign pair terms, and the
GPU's log) within 1e-10 relative.
The headline tolerance of the hot path -- 1e-10 relative on positions and
velocities after 100 steps at N=5000 -- is asserted too, as a floor."""
import numpy as np
import pytest

from cases import DENSITY, GOLDEN_CASES, GOLDEN_CHECKPOINTS, OracleMaterial, contact_case, material, two_sphere_case
from oracle.oracle import CpuOracle
from spacelab_gb300 import BallGroup, GpuStep, SpaceLabError, configs
from spacelab_gb300 import _lib

pytestmark = pytest.mark.gpu

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"
STATE_KEYS = ("pos", "vel", "w", "acc", "aacc")
E_RTOL = 1e-12
PE_RTOL = 1e-10


def _gpu(c, mode="exact"):
    g = BallGroup.from_arrays(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"])
    s = GpuStep(g, material(), mode)
    s.set_scalars(c["dt"], c["kin"], c["kout"])
    return s


def _oracle(c):
    return CpuOracle(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"], OracleMaterial(), c["dt"], c["kin"],
                     c["kout"])


def _state(s):
    g = s.download()
    return {k: getattr(g, k).copy() for k in STATE_KEYS}


def _term_scales(st, m, moi):
    """sum_i |m v_i|, sum_i |m (r x v)_i + moi w_i| per component."""
    pos, vel, w = st["pos"], st["vel"], st["w"]
    mom = (m[:, None] * np.abs(vel)).sum(0)
    L = (m[:, None] * np.abs(np.cross(pos, vel)) + moi[:, None] * np.abs(w)).sum(0)
    return mom, L


def _assert_energy(e_gpu, e_ref, st=None, m=None, moi=None):
    e_gpu = e_gpu.as_array() if hasattr(e_gpu, "as_array") else np.asarray(e_gpu)
    np.testing.assert_allclose(e_gpu[1], e_ref[1], rtol=E_RTOL, atol=0)
    np.testing.assert_allclose(e_gpu[0], e_ref[0], rtol=PE_RTOL, atol=0)
    if st is None:
        scale_mom = np.abs(e_ref[2:5]).max() * np.ones(3)
        scale_L = np.abs(e_ref[5:8]).max() * np.ones(3)
    else:
        scale_mom, scale_L = _term_scales(st, m, moi)
    assert np.all(np.abs(e_gpu[2:5] - e_ref[2:5]) <= 1e-12 * scale_mom + 1e-300), (e_gpu[2:5], e_ref[2:5])
    assert np.all(np.abs(e_gpu[5:8] - e_ref[5:8]) <= 1e-12 * scale_L + 1e-300), (e_gpu[5:8], e_ref[5:8])


@pytest.mark.parametrize("name", [c[0] for c in GOLDEN_CASES])
def test_exact_matches_reference_golden(name):
    g = np.load(GOLDEN / f"{name}.npz")
    c = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    for k in ("dt", "kin", "kout"):
        c[k] = float(c[k])
    s = _gpu(c)
    e0 = s.init_conditions()
    st = _state(s)
    assert np.array_equal(st["acc"], g["init_acc"])
    assert np.array_equal(st["aacc"], g["init_aacc"])
    _assert_energy(e0, g["init_energy"])
    assert np.array_equal(s.contacts(), g["contacts0"])
    every = int(g["write_every"])
    k = 0
    for step in range(1, max(GOLDEN_CHECKPOINTS) + 1):
        write = step % every == 0
        e = s.sim_one_step(write)
        if write:
            _assert_energy(e, g["energies"][k])
            k += 1
        if step in GOLDEN_CHECKPOINTS:
            st = _state(s)
            for key in STATE_KEYS:
                assert np.array_equal(st[key], g[f"step{step}_{key}"]), (name, step, key)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 31, 32, 33, 63, 64, 65, 100, 200])
def test_exact_matches_oracle_ragged_sizes(n):
    c = contact_case(n, 1000 + n)
    s, o = _gpu(c), _oracle(c)
    e0 = o.init()
    _assert_energy(s.init_conditions(), e0, o.state(), c["m"], c["moi"])
    assert np.array_equal(s.contacts(), o.contacts())
    for step in range(1, 41):
        write = step % 8 == 0
        e = s.sim_one_step(write)
        eo = o.step(write)
        if write:
            _assert_energy(e, eo, o.state(), c["m"], c["moi"])
        if step % 10 == 0:
            a, b = _state(s), o.state()
            for key in STATE_KEYS:
                assert np.array_equal(a[key], b[key]), (n, step, key)


@pytest.mark.parametrize("n,odd_every", [(300, 0), (300, 7), (1000, 64)])
def test_equal_radius_tiles_match_oracle(n, odd_every):
    """Monodisperse systems take the equal-radius tile form (radius sums and
    vdW radius products formed once per tile); with a few odd radii some
    tiles take the general form.  Contacts included; bit-identical."""
    c = contact_case(n, 2000 + n + odd_every, r_spread=0.0)
    if odd_every:
        R = c["R"].copy()
        R[::odd_every] *= 1.05
        c["R"] = R
        c["m"] = DENSITY * 4.0 / 3.0 * np.pi * R ** 3
        c["moi"] = 0.4 * c["m"] * R * R
    s, o = _gpu(c), _oracle(c)
    e0 = o.init()
    _assert_energy(s.init_conditions(), e0, o.state(), c["m"], c["moi"])
    assert len(o.contacts()) > 0
    assert np.array_equal(s.contacts(), o.contacts())
    for step in range(1, 31):
        write = step % 10 == 0
        e = s.sim_one_step(write)
        eo = o.step(write)
        if write:
            _assert_energy(e, eo, o.state(), c["m"], c["moi"])
    a, b = _state(s), o.state()
    for key in STATE_KEYS:
        assert np.array_equal(a[key], b[key]), key


def test_two_spheres_touching_and_separated():
    for gap in (-0.05, -1e-9, 0.0, 0.02, 5.0):
        c = two_sphere_case(gap)
        s, o = _gpu(c), _oracle(c)
        _assert_energy(s.init_conditions(), o.init())
        for step in range(1, 31):
            s.sim_one_step(step % 5 == 0)
            o.step(step % 5 == 0)
        a, b = _state(s), o.state()
        for key in STATE_KEYS:
            assert np.array_equal(a[key], b[key]), (gap, key)


def test_dense_contacts_n5000_step0_and_100_steps():
    """Contact-rich N=5000 system: step-0 contact set identical, then 100
    steps bit-identical to the oracle (row-parallel, all host cores)."""
    c = contact_case(5000, 5000, vel_sigma=20.0)
    s, o = _gpu(c), _oracle(c)
    e0 = o.init()
    _assert_energy(s.init_conditions(), e0, o.state(), c["m"], c["moi"])
    cg, co = s.contacts(), o.contacts()
    assert len(co) > 5000
    assert np.array_equal(cg, co)
    for step in range(1, 101):
        write = step % 50 == 0
        e = s.sim_one_step(write)
        eo = o.step(write, threads=0)
        if write:
            _assert_energy(e, eo, o.state(), c["m"], c["moi"])
    a, b = _state(s), o.state()
    for key in ("pos", "vel"):
        rel = np.abs(a[key] - b[key]).max() / np.abs(b[key]).max()
        assert rel <= 1e-10
    for key in STATE_KEYS:
        assert np.array_equal(a[key], b[key]), key


def test_aggregate_collision_n5000_100_steps():
    """The N=5000 benchmark workload: step-0 contact set, then 100 steps
    within 1e-10 relative (and in fact bit-identical) to the oracle."""
    w = configs.aggregate_collision_5000()
    c = dict(pos=w.group.pos, vel=w.group.vel, w=w.group.w, R=w.group.R, m=w.group.m, moi=w.group.moi, dt=w.dt,
             kin=w.kin, kout=w.kout)
    s, o = _gpu(c), _oracle(c)
    e0 = o.init()
    _assert_energy(s.init_conditions(), e0, o.state(), c["m"], c["moi"])
    assert np.array_equal(s.contacts(), o.contacts())
    for step in range(1, 101):
        write = step % w.skip == 0
        e = s.sim_one_step(write)
        eo = o.step(write, threads=0)
        if write:
            _assert_energy(e, eo, o.state(), c["m"], c["moi"])
    a, b = _state(s), o.state()
    for key in ("pos", "vel"):
        assert np.abs(a[key] - b[key]).max() <= 1e-10 * np.abs(b[key]).max()
    for key in STATE_KEYS:
        assert np.array_equal(a[key], b[key]), key


def test_looper_graph_matches_single_steps():
    c = contact_case(300, 77)
    a, b = _gpu(c), _gpu(c)
    a.init_conditions(); b.init_conditions()
    rows = a.sim_looper(steps=61, skip=10)
    ebs = []
    for step in range(1, 61):
        e = b.sim_one_step(step % 10 == 0)
        if e is not None:
            ebs.append(e)
    assert len(rows) == len(ebs) == 6
    for r, e in zip(rows, ebs):
        assert r.PE == e.PE and r.KE == e.KE
    sa, sb = _state(a), _state(b)
    for key in STATE_KEYS:
        assert np.array_equal(sa[key], sb[key])


@pytest.mark.parametrize("n", [20, 40, 300, 1000])
def test_pipelined_step_matches_sequential(n):
    """Row sums run per block-column phase beside the later pair phases
    (1 phase at n=20, 2 at n=40, 5 at n>=300); the sums keep their order, so
    single steps and the graph-captured looper equal the one-launch step
    bit for bit and the oracle stays bit-identical."""
    c = contact_case(n, 300 + n)
    a, b = _gpu(c), _gpu(c)
    a.set_overlap(True)
    b.set_overlap(False)
    o = _oracle(c)
    a.init_conditions(); b.init_conditions(); o.init()
    for step in range(1, 21):
        ea = a.sim_one_step(step % 5 == 0)
        eb = b.sim_one_step(step % 5 == 0)
        o.step(step % 5 == 0)
        if ea is not None:
            assert ea.as_array().tolist() == eb.as_array().tolist()
    sa, sb, so = _state(a), _state(b), o.state()
    for key in STATE_KEYS:
        assert np.array_equal(sa[key], sb[key]), key
        assert np.array_equal(sa[key], so[key]), key
    ra = a.sim_looper(steps=41, skip=10, first_step=21)
    rb = b.sim_looper(steps=41, skip=10, first_step=21)
    assert [r.PE for r in ra] == [r.PE for r in rb] and [r.KE for r in ra] == [r.KE for r in rb]
    sa, sb = _state(a), _state(b)
    for key in STATE_KEYS:
        assert np.array_equal(sa[key], sb[key]), key


@pytest.mark.parametrize("case", ["dense1000", "poly3000", "pipelined300"])
def test_rowsum_methods_bit_identical(case):
    """The row sums' FP64 additions on the integer pipe (the default) and on
    the FP64 unit give the same state bit for bit, over single steps and the
    graph-captured looper, with contacts, unequal radii and the pipelined
    step; and both equal the oracle."""
    if case == "dense1000":
        c = contact_case(1000, 77)
    elif case == "poly3000":
        g = configs.build_cluster(3000, 3000, sigma_v=1e-2, sigma_ln=0.2)
        kin, kout, dt = configs.spring_and_dt(float(g.R.max()), float(g.m.min()), 1.0)
        c = {"pos": g.pos, "vel": g.vel, "w": g.w, "R": g.R, "m": g.m, "moi": g.moi, "dt": dt, "kin": kin,
             "kout": kout}
    else:
        c = contact_case(300, 9)
    a, b = _gpu(c), _gpu(c)
    a.set_rowsum("int")
    b.set_rowsum("fp64")
    if case == "pipelined300":
        a.set_overlap(True)
        b.set_overlap(True)
    o = _oracle(c)
    a.init_conditions(); b.init_conditions(); o.init()
    for step in range(1, 11):
        a.sim_one_step(step % 5 == 0)
        b.sim_one_step(step % 5 == 0)
        o.step(step % 5 == 0)
    sa, sb, so = _state(a), _state(b), o.state()
    for key in STATE_KEYS:
        assert np.array_equal(sa[key], sb[key]), key
        assert np.array_equal(sa[key], so[key]), key
    a.sim_looper(steps=30, skip=10, first_step=11)
    b.sim_looper(steps=30, skip=10, first_step=11)
    sa, sb = _state(a), _state(b)
    for key in STATE_KEYS:
        assert np.array_equal(sa[key], sb[key]), key


def test_rowsum_method_is_exact_mode_only():
    c = contact_case(64, 5)
    s = _gpu(c, "mixed_df")
    with pytest.raises(SpaceLabError):
        s.set_rowsum("fp64")


@pytest.mark.parametrize("mode", ["mixed", "mixed_df"])
def test_mixed_mode_has_no_pipelined_step(mode):
    c = contact_case(64, 5)
    s = _gpu(c, mode)
    s.set_overlap(False)
    with pytest.raises(SpaceLabError):
        s.set_overlap(True)


def test_resume_matches_continuous_run():
    c = contact_case(128, 31)
    a = _gpu(c)
    a.init_conditions()
    for step in range(1, 21):
        a.sim_one_step(False)
    mid = _state(a)
    o = _oracle(c)
    o.init()
    for step in range(1, 20):
        o.step(False)
    prev = o.state()["pos"]  # positions one step before `mid`
    b = _gpu(c)
    b.group.pos[:] = mid["pos"]; b.group.vel[:] = mid["vel"]; b.group.w[:] = mid["w"]
    b.group.acc[:] = mid["acc"]; b.group.aacc[:] = mid["aacc"]
    b.upload_resume(pos_prev=prev)
    for step in range(21, 41):
        a.sim_one_step(False)
        b.sim_one_step(False)
    sa, sb = _state(a), _state(b)
    for key in STATE_KEYS:
        assert np.array_equal(sa[key], sb[key]), key


def test_step_host_matches_resident_steps_and_oracle():
    """sl_step_host (state on the host, read and overwritten every step)
    gives the device-resident run's states and totals bit for bit, step after
    step, and the oracle's; an array it cannot read fails cleanly."""
    c = contact_case(300, 41)
    a, b = _gpu(c), _gpu(c)
    o = _oracle(c)
    a.init_conditions(); b.init_conditions(); o.init()
    b.download()  # the host copy b's steps work on
    for step in range(1, 21):
        write = step % 5 == 0
        ea = a.sim_one_step(write)
        eb = b.sim_one_step_host(write)
        o.step(write)
        if write:
            assert ea.as_array().tolist() == eb.as_array().tolist()
        sa = _state(a)
        for key in STATE_KEYS:
            assert np.array_equal(sa[key], getattr(b.group, key)), (step, key)
    so = o.state()
    for key in STATE_KEYS:
        assert np.array_equal(getattr(b.group, key), so[key]), key
    g = b.group
    rc = _lib.lib().sl_step_host(b.handle, _lib.dptr(g.pos), _lib.dptr(g.vel), _lib.dptr(g.w), None,
                                 _lib.dptr(g.aacc), 0, None)
    assert rc == _lib.SL_ERR_ARG
    # a NaN or Inf input is rejected and the arrays are left as they were;
    # the next valid call steps as before
    before = {k: getattr(g, k).copy() for k in STATE_KEYS}
    for key, bad in (("pos", np.nan), ("vel", np.inf), ("w", -np.inf)):
        getattr(g, key)[7, 1] = bad
        with pytest.raises(SpaceLabError):
            b.sim_one_step_host(False)
        getattr(g, key)[7, 1] = before[key][7, 1]
        for k in STATE_KEYS:
            assert np.array_equal(getattr(g, k), before[k]), (key, k)
    b.sim_one_step_host(False)
    a.sim_one_step(False)
    sa = _state(a)
    for key in STATE_KEYS:
        assert np.array_equal(sa[key], getattr(b.group, key)), key


def test_reciprocal_division_is_ieee_exact():
    lib = _lib.lib()
    rng = np.random.default_rng(0)
    n = 1 << 20
    a = rng.normal(0, 1, n) * 10.0 ** rng.uniform(-20, 20, n)
    b = 10.0 ** rng.uniform(-15, 15, n)
    # divisors with all-ones / all-zero significands and near-midpoint cases
    b[:4096] = np.nextafter(2.0 ** rng.integers(-40, 40, 4096), 0)
    b[4096:8192] = 2.0 ** rng.integers(-40, 40, 4096) * (1 + 2.0 ** -52)
    a[8192:12288] = b[8192:12288] * (1 + rng.integers(1, 1 << 20, 4096) * 2.0 ** -53)
    qr, qi = np.zeros(n), np.zeros(n)
    assert lib.sl_diag_division(n, _lib.dptr(a), _lib.dptr(b), _lib.dptr(qr), _lib.dptr(qi)) == 0
    assert np.array_equal(qi, a / b)  # the GPU's IEEE division agrees with numpy
    assert np.array_equal(qr.view(np.int64), qi.view(np.int64))


def test_nonfinite_state_is_reported_not_trapped():
    c = contact_case(40, 3)
    s = _gpu(c)
    s.init_conditions()
    s.set_scalars(1e300, c["kin"], c["kout"])
    with pytest.raises(SpaceLabError) as ei:
        s.step(3, write_last=True)
    assert ei.value.code == _lib.SL_ERR_NONFINITE


def test_bad_inputs_rejected():
    c = contact_case(10, 4)
    c["R"] = c["R"].copy()
    c["R"][3] = 0.0
    with pytest.raises(SpaceLabError):
        _gpu(c)
    c = contact_case(10, 4)
    c["pos"] = c["pos"].copy()
    c["pos"][2, 1] = np.nan
    with pytest.raises(SpaceLabError):
        _gpu(c)


def test_integer_rounded_quotient_and_sqrt_are_ieee_exact():
    """The step kernels' quotients and square roots (FP64 estimate + exact
    integer rounding, with hardware fallback) equal the IEEE results bit for
    bit: random operands over wide exponent ranges, quotients next to
    midpoints and binade edges, signed zeros and the physics' own ranges."""
    lib = _lib.lib()
    rng = np.random.default_rng(7)
    n = 1 << 21
    a = rng.normal(0, 1, n) * 10.0 ** rng.uniform(-30, 30, n)
    b = rng.normal(0, 1, n) * 10.0 ** rng.uniform(-18, 18, n)
    k = n // 8
    b[:k] = np.nextafter(2.0 ** rng.integers(-60, 60, k), 0)               # all-ones significands
    b[k:2 * k] = 2.0 ** rng.integers(-60, 60, k) * (1 + 2.0 ** -52)        # 1 + ulp
    a[2 * k:3 * k] = b[2 * k:3 * k] * (1 + rng.integers(1, 1 << 20, k) * 2.0 ** -53)  # near midpoints
    a[3 * k:4 * k] = rng.uniform(1e-6, 3e-3, k)                              # displacements (cm)
    b[3 * k:4 * k] = rng.uniform(1e-4, 3e-3, k)                              # distances
    a[4 * k:5 * k] = rng.normal(0, 1e-8, k)                                  # forces (dyn)
    b[4 * k:5 * k] = rng.uniform(1e-12, 6e-11, k)                            # masses (g)
    a[5 * k:5 * k + 8] = [0.0, -0.0, 1.0, -1.0, 2.0 ** -1022, 1e308, 4.0, 9.0]
    out = np.zeros(4 * n)
    assert lib.sl_diag_exact_ops(n, _lib.dptr(a), _lib.dptr(b), _lib.dptr(out)) == 0
    fast_q, hw_q, fast_s, hw_s = out.reshape(4, n)
    assert np.array_equal(hw_q, a / b, equal_nan=True)
    assert np.array_equal(fast_q.view(np.int64), hw_q.view(np.int64))
    assert np.array_equal(hw_s, np.sqrt(np.abs(a)))
    assert np.array_equal(fast_s.view(np.int64), hw_s.view(np.int64))


def test_integer_pipe_estimates_round_to_ieee():
    """The exact step's integer-pipe arithmetic (fixed-point mass
    reciprocals, Newton reciprocals, fixed-point 1/sqrt, products) equals
    the IEEE quotient, square root and product bit for bit."""
    lib = _lib.lib()
    rng = np.random.default_rng(11)
    n = 1 << 21
    a = rng.normal(0, 1, n) * 10.0 ** rng.uniform(-30, 30, n)
    b = rng.normal(0, 1, n) * 10.0 ** rng.uniform(-18, 18, n)
    k = n // 8
    b[:k] = np.nextafter(2.0 ** rng.integers(-60, 60, k), 0)               # all-ones significands
    b[k:2 * k] = 2.0 ** rng.integers(-60, 60, k) * (1 + 2.0 ** -52)        # 1 + ulp
    a[2 * k:3 * k] = b[2 * k:3 * k] * (1 + rng.integers(1, 1 << 20, k) * 2.0 ** -53)  # near midpoints
    a[3 * k:4 * k] = rng.uniform(1e-6, 3e-3, k)                              # displacements (cm)
    b[3 * k:4 * k] = rng.uniform(1e-14, 1e-5, k)                             # squared distances
    a[4 * k:5 * k] = rng.normal(0, 1e-8, k)                                  # forces (dyn)
    b[4 * k:5 * k] = rng.uniform(1e-12, 6e-11, k)                            # masses (g)
    a[5 * k:6 * k] = 2.0 ** rng.integers(-100, 100, k)                       # exact powers of two
    b[5 * k:6 * k] = 2.0 ** rng.integers(-100, 100, k)
    a[6 * k:6 * k + 8] = [0.0, -0.0, 1.0, -1.0, 2.0 ** -1022, 1e308, 4.0, 9.0]
    b[6 * k + 8:6 * k + 12] = [2.0 ** -1074, 1e-310, 1.0, 4.0]               # subnormal divisors
    a[7 * k:7 * k + k // 2] = 3.0 * 2.0 ** rng.integers(-40, 40, k // 2)      # exact product ties
    b[7 * k:7 * k + k // 2] = 1.0 + (2 * rng.integers(0, 1 << 40, k // 2) + 1) * 2.0 ** -52
    out = np.zeros(6 * n)
    assert lib.sl_diag_int_ops(n, _lib.dptr(a), _lib.dptr(b), _lib.dptr(out)) == 0
    q_set, q_newton, s_fix, q_rsqrt, prod, q_neg = out.reshape(6, n)
    with np.errstate(all="ignore"):
        q = a / b
        sa = np.sqrt(np.abs(a))
        qr = a / np.sqrt(np.abs(b))
        ab = a * b

    def same_bits(got, want):
        nan = np.isnan(want)  # NaN payloads differ between hosts; NaN must stay NaN
        assert np.array_equal(np.isnan(got), nan)
        assert np.array_equal(got[~nan].view(np.int64), want[~nan].view(np.int64))

    same_bits(q_set, q)
    same_bits(q_newton, q)
    same_bits(s_fix, sa)
    same_bits(q_rsqrt, qr)
    same_bits(prod, ab)
    same_bits(q_neg, -q)
