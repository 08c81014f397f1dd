"""Write the golden fixtures of tests/golden/: one COUPLED_ENERGY_EQS step of a
small seeded shell (16 x 24 x 12, dt = 100 s, EPSMAT = 1e-10) by the C oracle,
with the theta boundary rows (shell_step.npz) and with the one-rank pole
shifts of inc_poles = 1 (poles_step.npz).

The reference ships no tests or golden vectors and cannot be built here, so
these fixtures pin the oracle (and the GPU path checked against it) to its
own output: regression fixtures, not reference pins.

    python tests/golden/make_golden.py [shell_step] [poles_step]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from conftest import oracle_from_shell  # noqa: E402
from ttcode_gb300.synthetic import make_shell  # noqa: E402

NX, NY, NZ, DELT, EPS = 16, 24, 12, 100.0, 1e-10
CASES = {"shell_step": dict(seed=11, poles=False), "poles_step": dict(seed=13, poles=True)}


def write(name):
    seed, poles = CASES[name]["seed"], CASES[name]["poles"]
    sh = make_shell(NX, NY, NZ, seed=seed, delt=DELT, poles=poles)
    o = oracle_from_shell(sh, eps=EPS)
    assert o.call("coupled_energy_eqs", 1) == 0
    er = o.f("ER")[2:NX + 2, 2:NY + 2, 2:NZ + 2].copy()
    t = o.f("T")[2:NX + 2, 2:NY + 2, 2:NZ + 2].copy()
    extra = dict(poles=1) if poles else {}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), nx=NX, ny=NY, nz=NZ, seed=seed, delt=DELT, eps=EPS,
                        sor_total=int(o.get("sor_total")), energy_iter=int(o.get("energy_iter")), ER=er, T=t,
                        **extra)
    print(f"wrote {name}.npz:", int(o.get("sor_total")), "sweeps,", int(o.get("energy_iter")), "outer iterations")


if __name__ == "__main__":
    for n in sys.argv[1:] or list(CASES):
        write(n)
