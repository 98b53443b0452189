"""k-epsilon turbulence (iturb = 3) on the GPU against the oracle.

The reference's explicit k-epsilon update is unstable on the drop case: with
the inijet-style initial state the gas has eps ~ 1e-14 while production
raises k by ~1e-3 per step, so mut = 0.09 rho k^2 / eps grows by orders of
magnitude and the fields overflow on the third step (the oracle shows the same,
tests/test_oracle.py).  Parity is checked on the two steps before that.
"""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

FIELDS = ["cc", "u", "v", "w", "p", "ktur", "eps", "mut", "rhon", "mun"]


@pytest.mark.parametrize("n,mode", [(32, 0), (24, 1)])
def test_keps_matches_oracle(gpu_lib, n, mode):
    dsg = gpu_lib
    from oracle import Oracle
    inp = dsg.config.droplet(n, mode=mode, tol=1e-9, impact_speed=3.0).replace(iturb=3)
    ora, gpu = Oracle(inp.as_dict()), dsg.Solver(inp)
    for name in ("ktur", "eps", "mut"):
        assert relerr(gpu.field(name), ora.field(name)) == 0.0, ("init", name)
    for t in (1, 2):
        ora.step(t)
        gpu.step(t)
        for name in FIELDS:
            e = relerr(gpu.field(name), ora.field(name))
            assert e <= 1e-10, (t, name, e)
        assert np.isfinite(gpu.field("mut")).all()


def test_only_laminar_and_keps(gpu_lib):
    dsg = gpu_lib
    with pytest.raises(dsg.DsgError) as e:
        dsg.Solver(dsg.config.droplet(16).replace(iturb=1))
    assert e.value.code == -1
