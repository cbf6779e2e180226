"""Generate tests/golden/*.npz from the reference's own sim_one_step.

Runs oracle/_ref/libslref.so -- the unmodified reference translation unit
ColliderSingleCore/ColliderSingleCore.cpp compiled by oracle/Makefile -- on
the seeded cases of tests/cases.py and stores inputs, the state after the
checkpoint steps, the energy totals of every write step and the step-0
contact set.  Needs the reference tree (for building the pin); the fixtures
it writes are what the tests use everywhere else.

    make -C oracle REF=<root of the reference tree> && python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from cases import GOLDEN_CASES, GOLDEN_CHECKPOINTS, MATERIAL, golden_case_inputs  # noqa: E402
from oracle.oracle import RefPin, ref_available  # noqa: E402


def contacts(pos, R):
    out = []
    n = len(R)
    for A in range(1, n):
        d = np.sqrt(((pos[:A] - pos[A]) ** 2).sum(axis=1))
        for B in np.nonzero(R[A] + R[:A] - d > 0)[0]:
            out.append((A, int(B)))
    return np.array(out, dtype=np.int32).reshape(-1, 2)


def main() -> int:
    if not ref_available():
        print("oracle/_ref/libslref.so is not built (needs the reference tree)", file=sys.stderr)
        return 1
    mat = RefPin.material()
    want = tuple(MATERIAL[k] for k in ("G", "Ha", "u_s", "u_r", "h_min"))
    assert mat == want, (mat, want)
    # the pin holds one global Ball_group: run each case in a fresh process
    if len(sys.argv) > 1:
        name = sys.argv[1]
        spec = [c for c in GOLDEN_CASES if c[0] == name][0]
        _, n, seed, steps, every = spec
        c = golden_case_inputs(name)
        ref = RefPin(c["pos"], c["vel"], c["w"], c["R"], c["m"], c["moi"], c["dt"], c["kin"], c["kout"])
        out = {f"in_{k}": np.asarray(v) for k, v in c.items()}
        out["init_energy"] = ref.e0
        st = ref.state()
        out["init_acc"], out["init_aacc"] = st["acc"], st["aacc"]
        out["contacts0"] = contacts(np.asarray(c["pos"]), np.asarray(c["R"]))
        energies = []
        for s in range(1, steps + 1):
            write = s % every == 0
            e = ref.step(write)
            if write:
                energies.append(e)
            if s in GOLDEN_CHECKPOINTS:
                st = ref.state()
                for k, v in st.items():
                    out[f"step{s}_{k}"] = v
        out["energies"] = np.array(energies)
        out["write_every"] = np.array(every)
        np.savez_compressed(ROOT / "tests" / "golden" / f"{name}.npz", **out)
        print(f"{name}: n={n} steps={steps} contacts0={len(out['contacts0'])}")
        return 0
    import subprocess
    for name, *_ in GOLDEN_CASES:
        subprocess.run([sys.executable, __file__, name], check=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
