"""ttfld_sor_solve_noalloc: the allocation-free SOR solve, through the C ABI.

Some callers cannot let a library allocate device memory (their device
memory is all owned by their own pool or offload data region, or a hidden
cudaMalloc/cudaFree would synchronise the device under their running
kernels).  For them the entry point solves on device arrays they pass in and
keeps its working memory in one fixed-size __device__ array.  This test
checks, twice in a row (the array keeps the previous call's contents), that
its result equals the context-based exact FP64 solve bit for bit with the
same sweep count, and that a grid too large for the fixed array is refused.
The file is collected at the end, after the tests of the other paths.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SYSTEM = ("SOR_A", "SOR_B", "SOR_C", "SOR_D", "SOR_E", "SOR_F", "SOR_G", "RHS_ER")


@pytest.fixture(scope="module")
def solved_context():
    import torch
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import make_shell
    torch.cuda.init()
    sh = make_shell(40, 64, 32, seed=5, delt=100.0)
    sh.params["epsmat"] = 1e-10
    f = start_run(sh)
    f.set_solver("sor64_exact")
    f.coupled_energy_eqs(True)          # leaves a real SOLVE_WITH_SOR system on the device
    st = f.solve_system()               # the existing entry point's answer
    return sh, f, st, f.download("DELTA_ER")


def test_noalloc_matches_context_solve_twice(solved_context):
    import torch
    from ttcode_gb300 import _ffi
    sh, f, st_ref, x_ref = solved_context
    L = _ffi.lib()
    nx, ny, nz = sh.dims
    ptrs = [L.ttfld_device_ptr(f.h, _ffi.FIELDS[n]) for n in SYSTEM]
    assert all(ptrs)
    x = torch.zeros((nz + 4, ny + 4, nx + 4), dtype=torch.float64, device="cuda")  # Fortran (i fastest)
    for call in range(2):
        x.zero_()
        torch.cuda.synchronize()
        it, rn, bn = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        rc = L.ttfld_sor_solve_noalloc(*ptrs, x.data_ptr(), nx, ny, nz, f.params["sorparam"],
                                       f.params["epsmat"], 1, f.params["itmax"], None,
                                       ctypes.byref(it), ctypes.byref(rn), ctypes.byref(bn))
        assert rc == 0, (call, rc)
        got = x.cpu().numpy().transpose(2, 1, 0)
        assert it.value == st_ref.sor_iter, call
        assert np.array_equal(got, x_ref), call
        assert abs(bn.value - st_ref.rhsnorm) <= 1e-13 * st_ref.rhsnorm


def test_noalloc_rejects_grids_beyond_its_scratch():
    from ttcode_gb300 import _ffi
    L = _ffi.lib()
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    it = ctypes.c_int()
    rc = L.ttfld_sor_solve_noalloc(*([dummy] * 9), 16, 1024, 256, 1.7, 1e-10, 1, 10, None,
                                   ctypes.byref(it), None, None)
    assert rc == -1
