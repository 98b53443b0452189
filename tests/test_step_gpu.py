"""Whole-step parity of the GPU path against the FP64 oracle.

Per-step pressure, velocity and VOF fields must agree within 1e-10 relative
(max-norm relative to the field's max) and the liquid volume SUMFIELD(cc)
within 1e-12 relative, both in the reference's fixed-cycle FMG mode and in the
tolerance mode.
"""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-10
VOLUME_TOL = 1e-12
CHECK = ["cc", "u", "v", "w", "p", "s11", "s22", "s33", "s12", "s13", "s23", "rhon", "mun"]


def _pair(dsg, n, steps_cfg, **kw):
    from oracle import Oracle
    inp = dsg.config.droplet(n, **kw)
    return inp, Oracle(inp.as_dict()), dsg.Solver(inp)


@pytest.mark.parametrize("n,mode,steps", [(16, 0, 6), (32, 0, 12), (32, 1, 12)])
def test_step_parity(gpu_lib, n, mode, steps):
    dsg = gpu_lib
    inp, ora, gpu = _pair(dsg, n, steps, mode=mode, tol=1e-9, steps=steps)
    for name in CHECK + ["rhs"]:
        e = relerr(gpu.field(name), ora.field(name))
        assert e <= FIELD_TOL, ("init", name, e)
    for t in range(1, steps + 1):
        ora.step(t)
        st = gpu.step(t)
        for name in CHECK:
            e = relerr(gpu.field(name), ora.field(name))
            assert e <= FIELD_TOL, (t, name, e)
        vg, vo = gpu.liquid_volume(), ora.liquid_volume()
        assert abs(vg - vo) <= VOLUME_TOL * abs(vo), (t, vg, vo)
        so = ora.scalars()
        sg = gpu.scalars()
        assert sg.tau == so.tau and sg.tswap == so.tswap
        assert (sg.npre, sg.npost, sg.ntop) == (so.npre, so.npost, so.ntop)
        if mode == 1:
            assert st["converged"] == 1
            assert st["vcycles"] == so.last_vcycles
            assert st["relres"] < inp.tol


def test_noncubic_step(gpu_lib):
    """66x34x34 nodes (the shipped inputdata.in grid): ng from the smallest side."""
    dsg = gpu_lib
    from oracle import Oracle
    inp = dsg.config.droplet(32, steps=4).replace(nx=66)
    ora, gpu = Oracle(inp.as_dict()), dsg.Solver(inp)
    for t in range(1, 5):
        ora.step(t)
        gpu.step(t)
    for name in ["cc", "u", "v", "w", "p"]:
        assert relerr(gpu.field(name), ora.field(name)) <= FIELD_TOL, name


@pytest.mark.parametrize("n,mode", [(48, 0), (48, 1), (40, 1)])
def test_generalised_grid_step(gpu_lib, n, mode):
    """Sides that are not 2^k (the reference stops on them): the multigrid
    coarsens while the interior stays even, down to 3 (48) or 5 (40) cells."""
    dsg = gpu_lib
    inp, ora, gpu = _pair(dsg, n, 4, mode=mode, tol=1e-9, steps=4)
    assert gpu.scalars().ng == ora.scalars().ng
    for t in range(1, 5):
        ora.step(t)
        st = gpu.step(t)
        for name in ("cc", "u", "v", "w", "p"):
            assert relerr(gpu.field(name), ora.field(name)) <= FIELD_TOL, (t, name)
        if mode == 1:
            assert st["converged"] == 1 and st["vcycles"] == ora.scalars().last_vcycles


def test_isolated_interface_cell(gpu_lib):
    """An isolated partial cell has an all-zero Youngs normal (FL3D would
    divide 0/0); GPU and oracle both advect it as a uniformly filled cell."""
    dsg = gpu_lib
    from oracle import Oracle
    inp = dsg.config.droplet(16, noise_si=0.0)
    ora, gpu = Oracle(inp.as_dict()), dsg.Solver(inp, init=False)
    shape = ora.shape
    rng = np.random.default_rng(7)
    cc = np.zeros(shape)
    cc[8, 8, 8] = 0.3
    cc[4, 12, 9] = 0.7
    for name, val in (("cc", cc), ("u", rng.uniform(-1, 1, shape)), ("v", rng.uniform(-1, 1, shape)),
                      ("w", rng.uniform(-1, 1, shape))):
        ora.field(name)[:] = val
        gpu.set_field(name, val)
    ora.vofmethod()
    gpu.vofmethod()
    g, o = gpu.field("cc"), ora.field("cc")
    assert np.all(np.isfinite(o)) and np.all(np.isfinite(g))
    assert relerr(g, o) <= FIELD_TOL


def test_step_against_golden_fixture(gpu_lib):
    """The CUDA path reproduces the committed oracle fixture of a 16^3 droplet
    (3 steps) within 1e-10 of each field's max-norm."""
    import json
    import os
    dsg = gpu_lib
    from golden.make_golden import FIELDS, droplet16, field_digest
    with open(os.path.join(os.path.dirname(__file__), "golden", "step16.json")) as f:
        ref = json.load(f)["values"]
    gpu = dsg.Solver(droplet16())
    for t in (1, 2, 3):
        gpu.step(t)
        for name in FIELDS:
            a = gpu.field(name)
            n = a.size
            got = [float.fromhex(x) for x in field_digest(a)]
            exp = [float.fromhex(x) for x in ref["t%d_%s" % (t, name)]]
            scale = max(exp[2], 1e-300)
            tols = [1e-10 * scale * n, 1e-10 * scale * scale * n] + [1e-10 * scale] * (len(exp) - 2)
            for g, e, tol in zip(got, exp, tols):
                assert abs(g - e) <= tol, (t, name, g, e)
        vol = float.fromhex(ref["t%d_volume" % t])
        assert abs(gpu.liquid_volume() - vol) <= 1e-12 * vol
        assert gpu.scalars().tau == float.fromhex(ref["t%d_tau" % t])


def test_tol_fp64_fma_form_tracks_exact_order(gpu_lib):
    """The tolerance mode's FP64 multigrid in fused multiply-add form (the
    default) takes the same V-cycles as the reference's operation order and
    lands within 1e-12 of it; both stay within the field tolerance of the
    oracle."""
    dsg = gpu_lib
    from oracle import Oracle
    inp = dsg.config.droplet(32, mode=dsg.config.MODE_TOL_FP64, tol=1e-10, steps=5)
    ora = Oracle(inp.as_dict())
    with dsg.Solver(inp) as fma, dsg.Solver(inp.replace(fp64_exact=1)) as exact:
        for t in range(1, 6):
            ora.step(t)
            sf, se = fma.step(t), exact.step(t)
            assert sf["vcycles"] == se["vcycles"] == ora.scalars().last_vcycles, (t, sf, se)
            for name in ("p", "u", "v", "w", "cc"):
                assert relerr(fma.field(name), exact.field(name)) <= 1e-12, (t, name)
                assert relerr(fma.field(name), ora.field(name)) <= FIELD_TOL, (t, name)
                assert relerr(exact.field(name), ora.field(name)) <= FIELD_TOL, (t, name)
