"""The reference's save files (simData/energy/constants CSV) and the exact
checkpoint.  Where the reference tree is present, files are exchanged with
the reference's own writer and loader (oracle/_ref): byte-identical writes,
identical parses."""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from cases import contact_case
from oracle.oracle import ref_available
from spacelab_gb300 import BallGroup, EnergyRow, io

ROOT = Path(__file__).resolve().parents[1]


def _group(n=37, seed=5):
    c = contact_case(n, seed)
    return BallGroup.from_arrays(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"])


def test_simdata_format_and_last_row_continue(tmp_path):
    g = _group()
    prefix = str(tmp_path / "run_")
    wr = io.SimWriter(prefix, g, precision=17)
    wr.write_state(g)
    g2 = g.copy()
    g2.pos += 1e-6
    g2.w *= 2
    wr.write_state(g2)
    wr.write_energy(EnergyRow(1.5e-9, -1.0, 2.0, 1.0, 3.0, 4.0))
    text = Path(wr.simdata).read_text()
    lines = text.split("\n")
    assert len(lines) == 3 and not text.endswith("\n")
    cols = lines[0].split(",")
    assert cols[:11] == ["x0", "y0", "z0", "wx0", "wy0", "wz0", "wmag0", "vx0", "vy0", "vz0", "bound0"]
    assert cols[11] == "x1" and cols[-1] == f"bound{g.num_particles - 1}" and len(cols) == 11 * g.num_particles
    row = np.array(lines[2].split(","), dtype=float).reshape(-1, 11)
    np.testing.assert_array_equal(row[:, 10], 0.0)
    np.testing.assert_allclose(row[:, 6], np.linalg.norm(g2.w, axis=1), rtol=1e-15)
    back = io.load_continue(prefix)
    assert np.array_equal(back.pos, g2.pos) and np.array_equal(back.vel, g2.vel) and np.array_equal(back.w, g2.w)
    assert np.array_equal(back.R, g.R) and np.array_equal(back.m, g.m) and np.array_equal(back.moi, g.moi)
    assert Path(wr.energy).read_text() == "Time,PE,KE,E,p,L\n1.5e-09,-1,2,1,3,4"


def test_reference_precision_is_lossy_but_close(tmp_path):
    g = _group(20, 6)
    prefix = str(tmp_path / "p6_")
    io.SimWriter(prefix, g).write_state(g)
    back = io.load_continue(prefix)
    np.testing.assert_allclose(back.pos, g.pos, rtol=5e-6, atol=0)
    np.testing.assert_allclose(back.m, g.m, rtol=5e-6)


def test_trailing_newline_is_accepted(tmp_path):
    g = _group(5, 7)
    prefix = str(tmp_path / "nl_")
    io.SimWriter(prefix, g, precision=17).write_state(g)
    with open(prefix + "simData.csv", "a") as f:
        f.write("\n")
    assert np.array_equal(io.load_continue(prefix).pos, g.pos)


def test_bad_files_raise(tmp_path):
    (tmp_path / "bad_simData.csv").write_text("x0\n1,2,oops")
    (tmp_path / "bad_constants.csv").write_text("1,2,3\n")
    with pytest.raises(OSError):
        io.load_continue(str(tmp_path / "bad_"))
    with pytest.raises(OSError):
        io.load_continue(str(tmp_path / "missing_"))


def test_checkpoint_roundtrip_is_exact(tmp_path):
    g = _group(64, 8)
    g.acc[:] = np.random.default_rng(0).normal(size=g.acc.shape)
    g.aacc[:] = np.random.default_rng(1).normal(size=g.aacc.shape)
    prev = g.pos - 1e-7
    io.save_checkpoint(tmp_path / "c.bin", g, prev, dt=1e-9, kin=3.0, kout=1.2, sim_time=5e-7, step=500)
    d = io.load_checkpoint(tmp_path / "c.bin")
    for k in ("pos", "vel", "w", "acc", "aacc", "R", "m", "moi"):
        assert np.array_equal(getattr(d["group"], k), getattr(g, k)), k
    assert np.array_equal(d["pos_prev"], prev)
    assert (d["dt"], d["kin"], d["kout"], d["sim_time"], d["step"]) == (1e-9, 3.0, 1.2, 5e-7, 500)


_REF_IO = """
import sys, ctypes, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from oracle.oracle import REF_LIB
from cases import contact_case
lib = ctypes.CDLL(str(REF_LIB))
P = ctypes.POINTER(ctypes.c_double)
c = contact_case(23, 9)
arr = [np.ascontiguousarray(np.asarray(c[k], dtype=np.float64).reshape(-1)) for k in ("pos","vel","w","R","m","moi")]
lib.slref_write_sim.argtypes = [ctypes.c_char_p, ctypes.c_int] + [P] * 6
lib.slref_write_sim({prefix!r}.encode(), 23, *[a.ctypes.data_as(P) for a in arr])
lib.slref_load_sim.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)] + [P] * 6
for pre in ({prefix!r}, {mine!r}):
    n = ctypes.c_int(0)
    out = [np.zeros(3 * 100) for _ in range(3)] + [np.zeros(100) for _ in range(3)]
    import os
    d, name = os.path.split(pre)
    assert lib.slref_load_sim((d + "/").encode(), name.encode(), 100, ctypes.byref(n), *[o.ctypes.data_as(P) for o in out]) == 0
    np.savez(pre + "refparse.npz", n=n.value, *[o for o in out])
print("ok")
"""


@pytest.mark.skipif(not ref_available(), reason="reference pin not built (reference tree absent)")
def test_files_exchange_with_reference_writer_and_loader(tmp_path):
    c = contact_case(23, 9)
    g = BallGroup.from_arrays(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"])
    ref_prefix = str(tmp_path / "ref_")
    my_prefix = str(tmp_path / "mine_")
    io.SimWriter(my_prefix, g).write_state(g)          # reference precision (6)
    code = _REF_IO.format(root=str(ROOT), tests=str(ROOT / "tests"), prefix=ref_prefix, mine=my_prefix)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert out.returncode == 0, out.stderr[-2000:]
    # byte-identical simData and constants from the reference's writer and ours
    assert Path(ref_prefix + "simData.csv").read_bytes() == Path(my_prefix + "simData.csv").read_bytes()
    assert Path(ref_prefix + "constants.csv").read_bytes() == Path(my_prefix + "constants.csv").read_bytes()
    # the reference's loader and ours parse both saves identically
    for pre in (ref_prefix, my_prefix):
        r = np.load(pre + "refparse.npz")
        n = int(r["n"])
        mine = io.load_continue(pre)
        assert n == mine.num_particles == 23
        assert np.array_equal(r["arr_0"][:3 * n], mine.pos.reshape(-1))
        assert np.array_equal(r["arr_1"][:3 * n], mine.vel.reshape(-1))
        assert np.array_equal(r["arr_2"][:3 * n], mine.w.reshape(-1))
        assert np.array_equal(r["arr_3"][:n], mine.R)
        assert np.array_equal(r["arr_4"][:n], mine.m)
        assert np.array_equal(r["arr_5"][:n], mine.moi)
