"""The allocation-free pressure solve against the context solve.

dsg_mglin_noalloc serves callers that cannot allocate device memory when they
solve (their host owns the device arrays and forbids allocation after set-up,
or the solve runs where an allocation would synchronize the device).  It must
give the same pressure as dsg_mglin in the reference's fixed-cycle mode, on
two calls in a row (its static scratch keeps the previous call's contents),
and reject grids beyond its 66^3-node capacity or whose sides do not all halve
evenly down to the coarsest level.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-10


def _lib(dsg):
    lib = dsg.load()
    fn = lib.dsg_mglin_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * 6 + [C.c_int] * 7 + [C.c_double] * 3 + [C.c_void_p]
    return lib


def _device_copy(torch, solver, name):
    """Caller-owned device copy of a context field (Fortran order, flat)."""
    return torch.from_numpy(np.ascontiguousarray(solver.field(name).reshape(-1, order="F"))).cuda()


@pytest.mark.parametrize("n", [16, 64])
def test_noalloc_matches_context_solve(gpu_lib, n):
    import torch
    dsg = gpu_lib
    lib = _lib(dsg)
    inp = dsg.config.droplet(n, mode=dsg.config.MODE_REF_EXACT)
    s = dsg.Solver(inp)
    s.step(1)  # realistic rhs and coefficients on the finest level
    shape = s.shape
    ncell = shape[0] * shape[1] * shape[2]
    arrays = {nm: _device_copy(torch, s, nm) for nm in ("rhs", "a", "b", "c", "ei")}
    sc = s.scalars()
    s.mglin()  # context solve of the same system (reference fixed-cycle FMG)
    p_ref = s.field("p")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        p = torch.full((ncell,), 7.0, dtype=torch.float64, device="cuda")
        rc = lib.dsg_mglin_noalloc(p.data_ptr(), arrays["rhs"].data_ptr(), arrays["a"].data_ptr(),
                                   arrays["b"].data_ptr(), arrays["c"].data_ptr(), arrays["ei"].data_ptr(),
                                   shape[0], shape[1], shape[2], inp.cycles, sc.npre, sc.npost, sc.ntop,
                                   inp.omega, sc.lengthsize, sc.lengthscale, stream)
        assert rc == 0, lib.dsg_last_error(None)
        torch.cuda.synchronize()
        got = p.cpu().numpy().reshape(shape, order="F")
        assert relerr(got, p_ref) <= FIELD_TOL, (call, relerr(got, p_ref))
    s.close()


def test_noalloc_rejects_large_grid(gpu_lib):
    import torch
    dsg = gpu_lib
    lib = _lib(dsg)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    ptr = x.data_ptr()
    rc = lib.dsg_mglin_noalloc(ptr, ptr, ptr, ptr, ptr, ptr, 130, 130, 130, 2, 4, 4, 4, 1.5, 1.0, 1.0, None)
    assert rc == -1
    assert b"capacity" in lib.dsg_last_error(None)


def test_noalloc_rejects_uneven_grid(gpu_lib):
    """34 x 34 x 64 nodes: the 62-cell side does not halve evenly over the
    five levels its 32-cell sides give."""
    import torch
    dsg = gpu_lib
    lib = _lib(dsg)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    ptr = x.data_ptr()
    rc = lib.dsg_mglin_noalloc(ptr, ptr, ptr, ptr, ptr, ptr, 34, 34, 64, 2, 4, 4, 4, 1.5, 1.0, 1.0, None)
    assert rc == -1
    assert b"evenly" in lib.dsg_last_error(None)
