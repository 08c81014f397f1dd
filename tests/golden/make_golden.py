"""Write tests/golden/shell_step.npz: one COUPLED_ENERGY_EQS step of a small
seeded shell (16 x 24 x 12, dt = 100 s, EPSMAT = 1e-10) by the C oracle.

The reference ships no tests or golden vectors and cannot be built here, so
this fixture pins the oracle (and the GPU path checked against it) to its
own output: a regression fixture, not a reference pin.

    python tests/golden/make_golden.py
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

NX, NY, NZ, SEED, DELT, EPS = 16, 24, 12, 11, 100.0, 1e-10


def main():
    sh = make_shell(NX, NY, NZ, seed=SEED, delt=DELT)
    o = oracle_from_shell(sh, eps=EPS)
    assert o.call("coupled_energy_eqs", 1) == 0
    er = o.f("ER")[2:NX + 2, 2:NY + 2, 2:NZ + 2].copy()
    t = o.f("T")[2:NX + 2, 2:NY + 2, 2:NZ + 2].copy()
    np.savez_compressed(os.path.join(HERE, "shell_step.npz"), nx=NX, ny=NY, nz=NZ, seed=SEED, delt=DELT, eps=EPS,
                        sor_total=int(o.get("sor_total")), energy_iter=int(o.get("energy_iter")), ER=er, T=t)
    print("wrote shell_step.npz:", int(o.get("sor_total")), "sweeps,", int(o.get("energy_iter")), "outer iterations")


if __name__ == "__main__":
    main()
