"""Mixed-precision pressure solve (FP32 V-cycles inside FP64 defect
correction) against the FP64 oracle.

Both solvers start every step from the same state (the oracle's state is
uploaded to the GPU before each step), so the comparison measures the error
of one mixed-precision step against the FP64 oracle at the same tolerance.
"""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

STATE = ["cc", "u", "v", "w", "s11", "s22", "s33", "s12", "s13", "s23", "res"]


def _sync_state(gpu, ora):
    for name in STATE:
        gpu.set_field(name, ora.field(name))
    s = gpu.scalars()
    so = ora.scalars()
    for f in ("tau", "tauh", "time", "tauh2", "tswap", "npre", "npost", "ntop"):
        setattr(s, f, getattr(so, f))
    gpu.set_scalars(s)


@pytest.mark.parametrize("n,prolong,krylov", [(16, 0, 0), (32, 0, 0), (32, 1, 0), (16, 0, 1), (32, 0, 1),
                                               (32, 1, 1), (64, 0, 1)])
def test_mixed_matches_fp64_oracle(gpu_lib, n, prolong, krylov):
    """prolong 0: trilinear FP32 prolongation, 1: the reference's injection;
    krylov 1: each V-cycle preconditions a GCR step."""
    dsg = gpu_lib
    from oracle import Oracle
    tol = 1e-10
    ora = Oracle(dsg.config.droplet(n, mode=dsg.config.MODE_TOL_FP64, tol=tol).as_dict())
    gpu = dsg.Solver(dsg.config.droplet(n, mode=dsg.config.MODE_TOL_MIXED, tol=tol).replace(
        mg32_prolong=prolong, mg32_krylov=krylov), init=False)
    for t in range(1, 6):
        _sync_state(gpu, ora)
        ora.step(t)
        st = gpu.step(t)
        assert st["converged"] == 1 and st["relres"] < tol, st
        assert st["mode"] == dsg.config.MODE_TOL_MIXED
        for name in ("p", "u", "v", "w", "cc"):
            e = relerr(gpu.field(name), ora.field(name))
            assert e < 1e-7, (t, name, e)


def test_mixed_free_run_volume(gpu_lib):
    """A free mixed-precision run tracks the FP64 oracle's liquid volume."""
    dsg = gpu_lib
    from oracle import Oracle
    ora = Oracle(dsg.config.droplet(32, mode=dsg.config.MODE_TOL_FP64, tol=1e-10).as_dict())
    gpu = dsg.Solver(dsg.config.droplet(32, mode=dsg.config.MODE_TOL_MIXED, tol=1e-10))
    for t in range(1, 11):
        ora.step(t)
        gpu.step(t)
    vo, vg = ora.liquid_volume(), gpu.liquid_volume()
    assert abs(vg - vo) / vo < 1e-9, (vg, vo)
    assert relerr(gpu.field("p"), ora.field("p")) < 1e-5


@pytest.mark.parametrize("n,tail,prolong,mid,small", [(32, 0, 0, 0, 0), (48, 0, 0, 0, 0), (64, 0, 0, 0, 0),
                                                     (64, 10 ** 6, 0, 0, 0), (64, 10 ** 6, 1, 0, 0),
                                                     (64, 10 ** 6, 0, 4, 0), (32, 10 ** 6, 0, 3, 0),
                                                     (64, 0, 0, 0, 2), (64, 10 ** 6, 0, 0, 3)])
def test_coarse_tail_is_bit_identical(gpu_lib, n, tail, prolong, mid, small):
    """The single-block coarse tail computes the same bits as one launch per
    pass, with fewer launches.  tail=10**6 runs every level below the finest
    in the tail kernel.  prolong: 0 trilinear, 1 injection; mid: own sweep
    counts (mid, mid+2) on the level below the finest; small: (small,
    small+1) on the levels of at most 18^3 nodes."""
    dsg = gpu_lib
    lib = dsg.load()
    base = dsg.config.droplet(n, mode=dsg.config.MODE_TOL_MIXED, tol=1e-9, impact_speed=2.0).replace(
        mg32_prolong=prolong, mg32_mid_npre=mid, mg32_mid_npost=mid + 2 if mid else 0,
        mg32_small_npre=small, mg32_small_npost=small + 1 if small else 0)
    runs = {}
    for key, tn in (("pass", -1), ("tail", tail)):
        with dsg.Solver(base.replace(tail_nodes=tn)) as s:
            l0 = lib.dsg_launch_count()
            vc = [s.step(t)["vcycles"] for t in range(1, 6)]
            s.synchronize()
            runs[key] = (lib.dsg_launch_count() - l0, vc, {f: s.field(f).copy() for f in ("p", "u", "v", "w", "cc")})
    assert runs["pass"][1] == runs["tail"][1]
    for f in ("p", "u", "v", "w", "cc"):
        assert np.array_equal(runs["pass"][2][f], runs["tail"][2][f]), f
    assert runs["tail"][0] < runs["pass"][0], (runs["tail"][0], runs["pass"][0])


def test_mixed_generalised_grid(gpu_lib):
    """48^3 interior (coarsest level 3^3): mixed solve against the FP64 oracle."""
    dsg = gpu_lib
    from oracle import Oracle
    tol = 1e-10
    ora = Oracle(dsg.config.droplet(48, mode=dsg.config.MODE_TOL_FP64, tol=tol).as_dict())
    gpu = dsg.Solver(dsg.config.droplet(48, mode=dsg.config.MODE_TOL_MIXED, tol=tol), init=False)
    assert gpu.scalars().ng == 5
    for t in range(1, 4):
        _sync_state(gpu, ora)
        ora.step(t)
        st = gpu.step(t)
        assert st["converged"] == 1 and st["relres"] < tol, st
        for name in ("p", "u", "v", "w", "cc"):
            assert relerr(gpu.field(name), ora.field(name)) < 1e-7, (t, name)


def test_gcr_cuts_vcycles_and_is_deterministic(gpu_lib):
    """GCR over the FP32 V-cycle (mg32_krylov = 1) reaches the tolerance with
    fewer V-cycles over eight steps than the V-cycles iterated alone, keeps the
    liquid volume of the stationary run, and repeats its own bits."""
    dsg = gpu_lib
    base = dsg.config.droplet(64, mode=dsg.config.MODE_TOL_MIXED, tol=1e-10, impact_speed=3.0, noise_si=1e-4)
    runs = {}
    for key, kr in (("stationary", 0), ("gcr", 1), ("gcr_again", 1)):
        with dsg.Solver(base.replace(mg32_krylov=kr)) as s:
            sts = [s.step(t) for t in range(1, 9)]
            assert all(st["converged"] == 1 and st["relres"] < 1e-10 for st in sts), sts
            runs[key] = ([st["vcycles"] for st in sts], s.liquid_volume(),
                         {f: s.field(f).copy() for f in ("p", "u", "v", "w", "cc")})
    vs, vg = runs["stationary"][0], runs["gcr"][0]
    assert sum(vg) < sum(vs), (vg, vs)
    assert abs(runs["gcr"][1] - runs["stationary"][1]) / runs["stationary"][1] < 1e-9
    assert runs["gcr"][0] == runs["gcr_again"][0]
    for f in ("p", "u", "v", "w", "cc"):
        assert np.array_equal(runs["gcr"][2][f], runs["gcr_again"][2][f]), f
        assert relerr(runs["gcr"][2][f], runs["stationary"][2][f]) < 1e-5, f



@pytest.mark.parametrize("start", [1, 2])
def test_mixed_other_starts_reach_the_same_solution(gpu_lib, start):
    """The mixed solve from the previous-step pressure (1) or from zero (2)
    reaches the tolerance and the same step as from the FP32 FMG start."""
    dsg = gpu_lib
    base = dsg.config.droplet(32, mode=dsg.config.MODE_TOL_MIXED, tol=1e-10, impact_speed=3.0, noise_si=1e-4)
    runs = {}
    for key, ws in (("fmg", 0), ("other", start)):
        with dsg.Solver(base.replace(warm_start=ws)) as s:
            sts = [s.step(t) for t in range(1, 5)]
            assert all(st["converged"] == 1 and st["relres"] < 1e-10 for st in sts), sts
            runs[key] = {f: s.field(f).copy() for f in ("p", "u", "v", "w", "cc")}
    for f in ("p", "u", "v", "w", "cc"):
        assert relerr(runs["other"][f], runs["fmg"][f]) < 1e-6, f
