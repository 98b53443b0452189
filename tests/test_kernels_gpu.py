"""Per-kernel parity of the array-level C ABI against the oracle.

Random inputs on grids of 6^3..34^3 nodes and a non-cubic grid; the FP64
kernels are built without FMA contraction and keep the reference's operation
order, so results must be bit-identical (max abs difference 0), including
ghost cells.
"""
import numpy as np
import pytest

import oracle.oracle as oo

pytestmark = pytest.mark.gpu

SHAPES = [(6, 6, 6), (10, 10, 10), (18, 18, 18), (34, 34, 34), (34, 18, 18)]


def rng(seed):
    return np.random.default_rng(seed)


def coeffs(shape, r):
    return [r.uniform(1.0, 833.0, size=shape) for _ in range(3)]


@pytest.mark.parametrize("shape", SHAPES)
def test_relax_resid(gpu_lib, shape):
    K = gpu_lib.kernels
    r = rng(1)
    u = r.standard_normal(shape)
    rhs = r.standard_normal(shape)
    a, b, c = coeffs(shape, r)
    ei = 1.0 / (a + b + c + 1.0)
    ls, om = 1.0, 1.5
    ref_u = oo.relax(u, ls, rhs, a, b, c, ei, om)
    du = K.to_device(u)
    dev = [K.to_device(x) for x in (rhs, a, b, c, ei)]
    K.relax(du, ls, *dev, shape, om)
    got = K.to_host(du, shape)
    assert np.array_equal(got, ref_u)
    # resid on the relaxed field
    ref_r = oo.resid(ls, ref_u, rhs, a, b, c)
    dres = K.to_device(np.zeros(shape))
    K.resid(ls, dres, du, dev[0], dev[1], dev[2], dev[3], shape)
    assert np.array_equal(K.to_host(dres, shape), ref_r)


@pytest.mark.parametrize("shape", [(6, 6, 6), (10, 10, 10), (18, 10, 10), (34, 34, 34)])
def test_transfer(gpu_lib, shape):
    K = gpu_lib.kernels
    r = rng(2)
    fine = tuple(2 * n - 2 for n in shape)
    uf = r.standard_normal(fine)
    # rstrct
    ref_c = oo.rstrct(uf, shape)
    duc = K.to_device(np.zeros(shape))
    K.rstrct(duc, K.to_device(uf), shape)
    assert np.array_equal(K.to_host(duc, shape), ref_c)
    # interp
    uc = r.standard_normal(shape)
    ref_f = oo.interp(uc, fine)
    duf = K.to_device(np.zeros(fine))
    K.interp(duf, K.to_device(uc), fine)
    assert np.array_equal(K.to_host(duf, fine), ref_f)
    # addint
    u0 = r.standard_normal(fine)
    ref_u, ref_res = oo.addint(u0, uc)
    du, dres = K.to_device(u0), K.to_device(np.zeros(fine))
    K.addint(du, K.to_device(uc), dres, fine)
    assert np.array_equal(K.to_host(du, fine), ref_u)
    assert np.array_equal(K.to_host(dres, fine), ref_res)


@pytest.mark.parametrize("shape", [(6, 6, 6), (10, 10, 10), (18, 10, 10)])
def test_acfromac(gpu_lib, shape):
    K = gpu_lib.kernels
    r = rng(3)
    fine = tuple(2 * n - 2 for n in shape)
    a2, b2, c2 = coeffs(fine, r)
    init = [r.standard_normal(shape) for _ in range(4)]
    ref = oo.acfromac(a2, b2, c2, shape, init=init)
    outs = [K.to_device(x) for x in init]
    K.acfromac(*outs, K.to_device(a2), K.to_device(b2), K.to_device(c2), shape)
    for o, rr in zip(outs, ref):
        assert np.array_equal(K.to_host(o, shape), rr)


@pytest.mark.parametrize("shape", [(6, 6, 6), (18, 18, 18), (34, 18, 18)])
def test_abcei(gpu_lib, shape):
    K = gpu_lib.kernels
    r = rng(4)
    cc = np.clip(r.uniform(-0.2, 1.2, size=shape), 0.0, 1.0)
    init = [r.standard_normal(shape) for _ in range(4)]
    r1, r2 = 0.5 * (1.0 - 0.0012), 0.0012
    ref = oo.abcei(cc, r1, r2, init=init)
    outs = [K.to_device(x) for x in init]
    K.abcei(*outs, K.to_device(cc), r1, r2, shape)
    for o, rr in zip(outs, ref):
        assert np.array_equal(K.to_host(o, shape), rr)


@pytest.mark.parametrize("name", ["bc_scalar", "bc_resid", "bc_out"])
@pytest.mark.parametrize("shape", [(6, 6, 6), (18, 10, 34)])
def test_bc(gpu_lib, name, shape):
    K = gpu_lib.kernels
    s = rng(5).standard_normal(shape)
    ref = oo.bc(name, s)
    d = K.to_device(s)
    K.bc(name, d, shape)
    assert np.array_equal(K.to_host(d, shape), ref)


@pytest.mark.parametrize("shape", [(6, 6, 6), (34, 34, 34)])
def test_filterc27(gpu_lib, shape):
    K = gpu_lib.kernels
    r = rng(6)
    cc = r.uniform(0.0, 1.0, size=shape)
    cc[cc > 0.7] = 1.0
    out0 = r.standard_normal(shape)
    ref = oo.filterc27(cc, out0)
    d = K.to_device(out0)
    K.filterc27(K.to_device(cc), d, shape)
    assert np.array_equal(K.to_host(d, shape), ref)


def test_bad_arguments_rejected(gpu_lib):
    """The C ABI returns DSG_E_ARG (never aborts) on invalid sizes/pointers."""
    lib = gpu_lib.load()
    assert lib.dsg_relax(None, 1.0, None, None, None, None, None, 6, 6, 6, 1.5, None) == -1
    assert lib.dsg_interp(None, None, 7, 6, 6, None) == -1
    assert lib.dsg_bc_scalar(None, 2, 2, 2, None) == -1
