import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def oracle_from_shell(sh, eps=1e-10, itmax=200000, start=True):
    """An oracle state loaded with a synthetic shell (and the main program's set-up
    BOUNDS at III=0 followed by KAPPA when start=True)."""
    from oracle import Oracle
    from ttcode_gb300.grid import full_1d
    nx, ny, nz = sh.dims
    o = Oracle(nx, ny, nz)
    for n in sh.grid.m:
        a = full_1d(sh.grid, n)
        o.f(n)[:a.size] = a
    for n, a in sh.fields.items():
        o.f(n)[...] = a
    for k, v in sh.params.items():
        if k == "kappa_model":
            continue
        o.set(k, v)
    o.set("epsmat", eps)
    o.set("itmax", itmax)
    if start:
        o.set("iii", 0)
        assert o.call("bounds") == 0
        assert o.call("kappa") == 0
        o.set("iii", sh.params.get("iii", 1))
    return o


def fld_from_shell(sh, eps=1e-10, itmax=200000):
    from ttcode_gb300.fld import start_run
    sh.params["epsmat"] = eps
    sh.params["itmax"] = itmax
    return start_run(sh)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle
