"""Collision outcome metrics (slh_collision_outcome) on hand-built states."""
import numpy as np

from spacelab_gb300 import configs, sweep


def _outcome(pos, R, n_t):
    from spacelab_gb300 import _lib
    import ctypes
    lf, sf, rg = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    nc = ctypes.c_int()
    m = np.ones(len(R))
    assert _lib.lib().slh_collision_outcome(len(R), n_t, _lib.dptr(np.ascontiguousarray(pos.reshape(-1))),
                                            _lib.dptr(R), _lib.dptr(m), 0.1, ctypes.byref(lf), ctypes.byref(sf),
                                            ctypes.byref(rg), ctypes.byref(nc)) == 0
    return lf.value, sf.value, rg.value, nc.value


def test_chain_and_separate_projectile():
    R = np.ones(5)
    # target: three touching spheres on x; projectile: two touching spheres far away
    pos = np.array([[0, 0, 0], [1.95, 0, 0], [3.9, 0, 0], [100, 0, 0], [101.95, 0, 0]], dtype=float)
    lf, sf, rg, nc = _outcome(pos, R, 3)
    assert nc == 2 and abs(lf - 0.6) < 1e-12 and sf == 0.0
    assert abs(rg - np.sqrt(((np.array([0, 1.95, 3.9]) - 1.95) ** 2).mean())) < 1e-12


def test_projectile_stuck_and_gap_threshold():
    R = np.ones(4)
    pos = np.array([[0, 0, 0], [2.05, 0, 0], [4.1, 0, 0], [6.3, 0, 0]], dtype=float)  # gaps 0.05, 0.05, 0.2
    lf, sf, rg, nc = _outcome(pos, R, 3)
    assert nc == 2 and abs(lf - 0.75) < 1e-12 and sf == 0.0
    pos[3, 0] = 6.19  # gap 0.09 < 0.1: the projectile sphere joins
    lf, sf, rg, nc = _outcome(pos, R, 3)
    assert nc == 1 and lf == 1.0 and sf == 1.0


def test_cluster_is_one_remnant_and_rg_formula():
    g = configs.build_cluster(300, 5, sigma_v=0.0)
    # a random packing at phi = 0.3 is not connected by touching: many remnants
    lf, sf, rg, nc = _outcome(g.pos / configs.RADIUS, g.R / configs.RADIUS, 300)
    assert nc > 1
    from spacelab_gb300 import _lib
    import ctypes
    r = ctypes.c_double()
    _lib.lib().slh_radius_of_gyration(300, _lib.dptr(np.ascontiguousarray(g.pos.reshape(-1))), _lib.dptr(g.m),
                                      ctypes.byref(r))
    assert abs(r.value / configs.RADIUS - sweep.rg_formula(300)) < 0.1 * sweep.rg_formula(300)
