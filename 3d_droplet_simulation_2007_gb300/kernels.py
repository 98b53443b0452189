"""Array-level kernels of the C ABI on torch CUDA tensors.

Each function takes Fortran-ordered (nx,ny,nz) data held in a flat CUDA
tensor (``to_device``/``to_host`` convert from/to numpy) and calls the entry
point of include/dsg.h with the reference subroutine's argument list.  torch
supplies device memory and the current stream only; the kernels are
``libdsg.so``'s.
"""
import numpy as np

from . import _lib


def _torch():
    import torch
    return torch


def to_device(a, device="cuda"):
    """Flat float64 CUDA tensor holding numpy array ``a`` in Fortran order."""
    torch = _torch()
    flat = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))
    return torch.from_numpy(flat).to(device)


def to_host(t, shape):
    return t.detach().cpu().numpy().reshape(shape, order="F")


def _stream():
    return _torch().cuda.current_stream().cuda_stream


def _p(t):
    if t is None:
        return None
    assert t.is_cuda and t.dtype == _torch().float64 and t.is_contiguous()
    return t.data_ptr()


def _call(name, *args):
    lib = _lib.load()
    _lib.check(getattr(lib, name)(*args))


def relax(u, lengthsize, rhs, a, b, c, ei, shape, omega):
    _call("dsg_relax", _p(u), lengthsize, _p(rhs), _p(a), _p(b), _p(c), _p(ei), *shape, omega, _stream())


def resid(lengthsize, res, u, rhs, a, b, c, shape):
    _call("dsg_resid", lengthsize, _p(res), _p(u), _p(rhs), _p(a), _p(b), _p(c), *shape, _stream())


def rstrct(uc, uf, coarse_shape):
    _call("dsg_rstrct", _p(uc), _p(uf), *coarse_shape, _stream())


def interp(uf, uc, fine_shape):
    _call("dsg_interp", _p(uf), _p(uc), *fine_shape, _stream())


def addint(uf, uc, res, fine_shape):
    _call("dsg_addint", _p(uf), _p(uc), _p(res), *fine_shape, _stream())


def acfromac(a, b, c, ei, a2, b2, c2, coarse_shape):
    _call("dsg_acfromac", _p(a), _p(b), _p(c), _p(ei), _p(a2), _p(b2), _p(c2), *coarse_shape, _stream())


def abcei(a, b, c, ei, cc, r1, r2, shape):
    _call("dsg_abcei", _p(a), _p(b), _p(c), _p(ei), _p(cc), r1, r2, *shape, _stream())


def bc(name, s, shape):
    _call("dsg_" + name, _p(s), *shape, _stream())


def filterc27(cc, cf, shape):
    _call("dsg_filterc27", _p(cc), _p(cf), *shape, _stream())
