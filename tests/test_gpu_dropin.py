"""The drop-in inside the reference: the reference's own sim_looper
(ColliderSingleCore.cpp:291-375) with its step call switched to the GPU by
the adapter include/spacelab_sim_one_step_gpu.hpp, against the same
sim_looper calling the reference's own sim_one_step.

Both are the reference translation unit compiled from its sources
(oracle/Makefile: the unmodified TU, and the TU after the maintainer's
two-line edit, linked with libspacelab_gb300.so).  Both run
Ball_group::sim_init_write and sim_looper into files; the files must agree:

  simData.csv  -- identical text (every row: x, y, z, wx, wy, wz, |w|, vx,
                  vy, vz, bound per sphere; the GPU state is bit-identical);
  energy.csv   -- identical header and initial row; each looper row
                  (time, PE, KE, E, |p|, |L|) within 1e-10 relative (PE is
                  summed in another order on the GPU, and its log differs by
                  ulps; the file prints 12 significant digits);
  constants.csv -- identical text.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cases import contact_case
from oracle.oracle import REF_LIB, REF_LIB_GPU, RefPin

pytestmark = pytest.mark.gpu

ORACLE = Path(__file__).resolve().parents[1] / "oracle"
SNAPSHOT = ORACLE / "_ref" / "src" / "ColliderSingleCore" / "ColliderSingleCore.cpp"


def _build_adapter():
    if not SNAPSHOT.exists() or not REF_LIB.exists():
        pytest.skip("the reference's sources are not at hand (oracle/_ref/src)")
    proc = subprocess.run(["make", "-s", "-C", str(ORACLE), "adapter"], stdout=subprocess.PIPE,
                          stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, proc.stdout
    assert REF_LIB_GPU.exists()


def _run(lib_path, c, prefix, steps, skip):
    ref = RefPin(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"], c["dt"], c["kin"], c["kout"],
                 lib_path=lib_path)
    used = ref.looper(prefix, steps, skip)
    return {kind: Path(used + f"{kind}.csv").read_text() for kind in ("simData", "energy", "constants")}


def _energy_rows(text):
    lines = text.split("\n")
    return lines[:2], np.array([[float(x) for x in ln.split(",")] for ln in lines[2:] if ln.strip()])


@pytest.mark.parametrize("n,steps,skip", [(200, 301, 10), (64, 121, 1)])
def test_reference_looper_with_gpu_adapter_writes_the_same_files(tmp_path, n, steps, skip):
    _build_adapter()
    c = contact_case(n, 8080 + n)
    cpu = _run(REF_LIB, c, str(tmp_path / "cpu_"), steps, skip)
    gpu = _run(REF_LIB_GPU, c, str(tmp_path / "gpu_"), steps, skip)
    assert cpu["constants"] == gpu["constants"]
    sim_cpu, sim_gpu = cpu["simData"].split("\n"), gpu["simData"].split("\n")
    assert len(sim_cpu) == len(sim_gpu) == 2 + (steps - 1) // skip
    for k, (a, b) in enumerate(zip(sim_cpu, sim_gpu)):
        assert a == b, f"simData.csv line {k} differs"
    head_cpu, rows_cpu = _energy_rows(cpu["energy"])
    head_gpu, rows_gpu = _energy_rows(gpu["energy"])
    assert head_cpu == head_gpu
    assert rows_cpu.shape == rows_gpu.shape == ((steps - 1) // skip, 6)
    np.testing.assert_array_equal(rows_gpu[:, 0], rows_cpu[:, 0])          # time
    np.testing.assert_allclose(rows_gpu[:, 1:], rows_cpu[:, 1:], rtol=1e-10, atol=0)
