"""The allocation-free force pass, sl_forces_static.

It serves callers that cannot call cudaMalloc (an application that owns all
device memory and hands out buffers, or a real-time loop where allocation
is not allowed): they pass their own device buffers, and the library's
working memory is a static device array.  Here it must give the same
results as the handle-based entry point (sl_init_forces) -- acc/aacc bit
for bit, the energy totals within the parity tests' bar -- on two calls in a
row with different systems, so that nothing the first call leaves in the
shared working memory leaks into the second.

This file is collected last (tests/test_zz_*), so a run that stops at the
first failure has already run every other test.
"""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from cases import contact_case, material
from spacelab_gb300 import BallGroup, GpuStep, _lib

pytestmark = pytest.mark.gpu

HEADER = Path(__file__).resolve().parents[1] / "include" / "spacelab_gpu.h"


def _capacity() -> int:
    """SL_STATIC_MAX_SPHERES as the public header states it."""
    m = re.search(r"#define\s+SL_STATIC_MAX_SPHERES\s+(\d+)", HEADER.read_text())
    assert m, "SL_STATIC_MAX_SPHERES not found in spacelab_gpu.h"
    return int(m.group(1))


def _handle_reference(c):
    g = BallGroup.from_arrays(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"])
    with GpuStep(g, material(), "exact") as s:
        s.set_scalars(c["dt"], c["kin"], c["kout"])
        e = s.init_conditions()
        s.download()
        return g.acc.copy(), g.aacc.copy(), e.as_array()


def _static_call(torch, c, with_energy=True, expect=None):
    lib = _lib.lib()
    n = len(c["R"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).cuda()  # noqa: E731
    ins = [dev(c[k]) for k in ("pos", "vel", "w", "R", "m", "moi")]
    acc = torch.full((3 * n,), float("nan"), dtype=torch.float64, device="cuda")
    aacc = torch.full((3 * n,), float("nan"), dtype=torch.float64, device="cuda")
    energy = torch.zeros(8, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    mat = material()
    rc = lib.sl_forces_static(n, *[t.data_ptr() for t in ins], ctypes.byref(mat), c["kin"], c["kout"],
                              acc.data_ptr(), aacc.data_ptr(), energy.data_ptr() if with_energy else None, stream)
    if expect is not None:
        assert rc == expect, (rc, lib.sl_last_error())
        return None
    assert rc == _lib.SL_OK, lib.sl_last_error()
    e = energy.cpu().numpy() if with_energy else None
    return acc.cpu().numpy().reshape(-1, 3), aacc.cpu().numpy().reshape(-1, 3), e


def _assert_energy_close(e, ref, c, acc_state=None):
    np.testing.assert_allclose(e[1], ref[1], rtol=1e-12, atol=0)   # KE
    np.testing.assert_allclose(e[0], ref[0], rtol=1e-10, atol=0)   # PE
    m, moi, pos, vel, w = c["m"], c["moi"], c["pos"], c["vel"], c["w"]
    scale_mom = (m[:, None] * np.abs(vel)).sum(0)
    scale_L = (m[:, None] * np.abs(np.cross(pos, vel)) + moi[:, None] * np.abs(w)).sum(0)
    assert np.all(np.abs(e[2:5] - ref[2:5]) <= 1e-12 * scale_mom)
    assert np.all(np.abs(e[5:8] - ref[5:8]) <= 1e-12 * scale_L)


def test_static_force_pass_matches_handle_entry_point_twice():
    torch = pytest.importorskip("torch")
    first = contact_case(200, 4242)
    second = contact_case(97, 4343, vel_sigma=80.0)
    for c in (first, second):
        acc, aacc, e = _static_call(torch, c)
        racc, raacc, re = _handle_reference(c)
        assert np.array_equal(acc, racc)
        assert np.array_equal(aacc, raacc)
        assert np.count_nonzero(aacc) > 0          # contacts exercised
        _assert_energy_close(e, re, c)


def test_static_force_pass_at_capacity_single_sphere_and_without_energy():
    """n = capacity fills the pair and torque buffers exactly; n = 1 is one
    pair block with no pairs; energy = NULL skips the totals."""
    torch = pytest.importorskip("torch")
    cap = _capacity()
    for c, with_energy in ((contact_case(cap, 5151), True), (contact_case(1, 5252), True),
                           (contact_case(150, 5353), False)):
        acc, aacc, e = _static_call(torch, c, with_energy=with_energy)
        racc, raacc, re = _handle_reference(c)
        assert np.array_equal(acc, racc)
        assert np.array_equal(aacc, raacc)
        if with_energy:
            _assert_energy_close(e, re, c)


def test_static_force_pass_rejects_bad_sphere_constants():
    """A zero radius or a NaN mass is refused with SL_ERR_ARG (the handle
    path refuses them at upload), and the next good call is unaffected."""
    torch = pytest.importorskip("torch")
    lib = _lib.lib()
    for key, idx, val in (("R", 3, 0.0), ("m", 10, float("nan")), ("moi", 0, -1.0)):
        c = contact_case(40, 5454)
        c[key] = c[key].copy()
        c[key][idx] = val
        _static_call(torch, c, expect=_lib.SL_ERR_ARG)
        assert b"not finite and > 0" in lib.sl_last_error()
    c = contact_case(40, 5454)
    acc, aacc, _ = _static_call(torch, c)
    racc, raacc, _ = _handle_reference(c)
    assert np.array_equal(acc, racc) and np.array_equal(aacc, raacc)


def test_static_force_pass_rejects_sizes_beyond_capacity():
    lib = _lib.lib()
    mat = material()
    cap = _capacity()
    for n in (0, cap + 1):
        rc = lib.sl_forces_static(n, *([None] * 6), ctypes.byref(mat), 1.0, 0.5, None, None, None, None)
        assert rc == _lib.SL_ERR_ARG
        assert b"static working memory" in lib.sl_last_error()
