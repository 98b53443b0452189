"""dsg_step_host: a step whose state travels through host arrays, with the
copies overlapped with the step's phases, computes the same bits as
upload + dsg_step + download.

Each input's device copy is overwritten with zeros before the call, and the
host arrays hold values the step itself overwrites (nonzero ghost faces and
first interior z-plane on the off-diagonal stresses, which csf's bc_tensor
zeroes: with surface tension on they arrive after csf and the step writes
those faces again; random face coefficients and
previous pressure, which the pressure phase rebuilds), so an input that
arrived after the first phase touching it would change the result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INS = ["cc", "u", "v", "w", "s11", "s22", "s33", "s12", "s13", "s23", "a", "b", "c", "pprev"]
OUTS = ["p", "cc", "u", "v", "w", "s11", "s22", "s33", "s12", "s13", "s23", "rhon", "mun"]


def _variants(dsg):
    c = dsg.config
    base = c.droplet(32, mode=c.MODE_TOL_MIXED, tol=1e-9, impact_speed=3.0)
    return {
        "csf": (base, 3),
        "sgip": (base.replace(surfacet=5, hswitch=1), 3),
        "sgip2_fp64": (base.replace(surfacet=6, hswitch=1, mode=c.MODE_TOL_FP64), 2),
        "no_tension": (base.replace(sigma_si=0.0), 3),
        "keps": (base.replace(iturb=3), 1),
    }


def _perturbed(name, arr, rng):
    """The host copy of an input, changed where the step writes before it reads."""
    a = np.array(arr, order="F")
    if name in ("s12", "s13", "s23"):
        for sl in ((0,), (-1,)):
            a[sl[0], :, :] = 7.0
            a[:, sl[0], :] = 7.0
            a[:, :, sl[0]] = 7.0
        if name in ("s13", "s23"):
            a[:, :, 1] = 7.0  # the first interior z-plane, which bc_tensor also zeroes
    elif name in ("a", "b", "c", "pprev"):
        a[...] = rng.uniform(1.0, 2.0, a.shape)
    return np.ascontiguousarray(a.ravel(order="F"))


@pytest.mark.parametrize("name", ["csf", "sgip", "sgip2_fp64", "no_tension", "keps"])
def test_step_host_matches_step(gpu_lib, name):
    dsg = gpu_lib
    cfg, steps = _variants(dsg)[name]
    ins = INS + (["ktur", "eps", "mut"] if name == "keps" else [])
    outs = OUTS + (["ktur", "eps", "mut"] if name == "keps" else [])
    with dsg.Solver(cfg) as a, dsg.Solver(cfg) as b:
        a.step(1)
        b.step(1)
        rng = np.random.default_rng(5)
        for t in range(2, 2 + steps):
            host_in = {k: _perturbed(k, b.field(k), rng) for k in ins}
            for k in ins:
                a.set_field(k, host_in[k].reshape(a.shape, order="F"))
                b.set_field(k, np.zeros(b.shape))  # stale device copies: only the host arrays hold the state
            host_out = {k: np.empty(b.shape[0] * b.shape[1] * b.shape[2]) for k in outs}
            sa = a.step(t)
            sb = b.step_host(host_in, host_out, t)
            assert sa["vcycles"] == sb["vcycles"], (t, sa, sb)
            for k in outs:
                ref = a.field(k).ravel(order="F")
                assert np.array_equal(host_out[k], ref, equal_nan=True), (name, t, k)
                assert np.array_equal(b.field(k).ravel(order="F"), ref, equal_nan=True), (name, t, k)


def test_step_host_rejects_bad_fields(gpu_lib):
    dsg = gpu_lib
    with dsg.Solver(dsg.config.droplet(16, mode=dsg.config.MODE_TOL_MIXED, tol=1e-9)) as s:
        n = s.shape[0] * s.shape[1] * s.shape[2]
        lib = dsg.load()
        import ctypes as C
        st = dsg._lib.DsgMgStats()
        bad = (C.c_int * 1)(99)
        ptr = (C.c_void_p * 1)(np.empty(n).ctypes.data)
        rc = lib.dsg_step_host(s.ctx, 1, C.byref(st), 1, bad, ptr, 0, None, None)
        assert rc == -1 and b"bad input" in lib.dsg_last_error(s.ctx)
        rc = lib.dsg_step_host(s.ctx, 1, C.byref(st), -1, None, None, 0, None, None)
        assert rc == -1
