"""The ensemble on the GPU: members step exactly as standalone solvers do,
failures are reported per member, the autotuner keeps a valid plan."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIDES = [16, 32, 48, 24, 40]


def _inputs(dsg, mode):
    return [dsg.config.droplet(n, mode=mode, tol=1e-9, impact_speed=1.5 + 0.5 * k, seed=10 + k)
            for k, n in enumerate(SIDES)]


@pytest.mark.parametrize("mode,workers", [(2, 2), (2, 5), (1, 3)])
def test_members_match_standalone(gpu_lib, mode, workers):
    dsg = gpu_lib
    inputs = _inputs(dsg, mode)
    ref = []
    for inp in inputs:
        with dsg.Solver(inp) as s:
            stats = [s.step(t) for t in range(1, 6)]
            ref.append(({f: s.field(f) for f in ("p", "u", "v", "w", "cc")}, [x["vcycles"] for x in stats]))
    with dsg.Ensemble(inputs, workers=workers) as e:
        assert e.workers == workers
        vc = [[] for _ in inputs]
        for t in range(1, 6):
            for i, st in enumerate(e.step(t)):
                assert st["converged"] == 1
                vc[i].append(st["vcycles"])
        for i in range(len(inputs)):
            m = e.member(i)
            assert vc[i] == ref[i][1]
            for f in ("p", "u", "v", "w", "cc"):
                assert np.array_equal(m.field(f), ref[i][0][f]), (i, f)


def test_failing_member_is_reported(gpu_lib):
    dsg = gpu_lib
    inputs = _inputs(dsg, dsg.config.MODE_TOL_MIXED)
    inputs[3] = inputs[3].replace(mode=dsg.config.MODE_LEARNED)  # no network attached
    with dsg.Ensemble(inputs, workers=2) as e:
        with pytest.raises(dsg.DsgError) as ex:
            e.step(1)
        assert ex.value.code == -6 and "member 3" in str(ex.value)
        # the other members completed their step
        for i in (0, 1, 2, 4):
            assert e.member(i).scalars().last_vcycles > 0


def test_autotune(gpu_lib):
    dsg = gpu_lib
    with dsg.Ensemble(_inputs(dsg, dsg.config.MODE_TOL_MIXED), workers=1) as e:
        bw = e.autotune(steps_per_trial=1)
        assert 1 <= bw <= len(SIDES) and e.workers == bw
        assert e.t >= 3
        assert (e.member_ms() > 0).all()
        e.step()


def _standalone(dsg, inputs, steps):
    ref = []
    for inp in inputs:
        with dsg.Solver(inp) as s:
            stats = [s.step(t) for t in range(1, steps + 1)]
            ref.append(({f: s.field(f) for f in ("p", "u", "v", "w", "cc")}, [x["vcycles"] for x in stats]))
    return ref


def _mixed_tolerances(dsg):
    """Members of different sizes and tolerances: the looser ones converge
    first and sit the later V-cycles of a batched iteration out."""
    inputs = _inputs(dsg, dsg.config.MODE_TOL_MIXED)
    return [inp.replace(tol=tol) for inp, tol in zip(inputs, (1e-9, 1e-7, 1e-9, 1e-6, 1e-10))]


@pytest.mark.parametrize("workers,groups", [(1, 1), (3, 1), (3, 2), (2, 3)])
def test_batched_members_match_standalone(gpu_lib, workers, groups):
    """Batched pressure solves (one launch per multigrid pass over a group of
    members, groups side by side) give every member the bits of its own
    dsg_step."""
    dsg = gpu_lib
    inputs = _mixed_tolerances(dsg)
    ref = _standalone(dsg, inputs, 6)
    with dsg.Ensemble(inputs, workers=workers, batched=groups) as e:
        assert e.batched == groups
        vc = [[] for _ in inputs]
        for t in range(1, 7):
            for i, st in enumerate(e.step(t)):
                assert st["converged"] == 1 and st["relres"] < inputs[i].tol
                vc[i].append(st["vcycles"])
            assert (e.phase_ms() > 0).all()
        for i in range(len(inputs)):
            assert vc[i] == ref[i][1], (i, vc[i], ref[i][1])
            for f in ("p", "u", "v", "w", "cc"):
                assert np.array_equal(e.member(i).field(f), ref[i][0][f]), (i, f)


def test_batched_autotune_keeps_bits(gpu_lib):
    """The autotuner changes the coarse-tail depth and the thread-block
    shapes of the batched passes, not their results."""
    dsg = gpu_lib
    inputs = _mixed_tolerances(dsg)
    ref = _standalone(dsg, inputs, 5)
    with dsg.Ensemble(inputs, workers=2, batched=2) as e:
        e.step(1)
        e.step(2)
        tuned = e.autotune_tiles(reps=2)
        assert tuned > 0 and e.batch_tail_nodes > 0
        for t in range(3, 6):
            e.step(t)
        for i in range(len(inputs)):
            for f in ("p", "u", "v", "w", "cc"):
                assert np.array_equal(e.member(i).field(f), ref[i][0][f]), (i, f)


def test_batched_study_sizes(gpu_lib):
    """The droplet-study grids (48 to 160 cells per side, Weber 50-800)
    batched match their standalone steps."""
    dsg = gpu_lib
    inputs = dsg.ensemble.study_configs(6, seed=1000)
    assert len({x.nx - 2 for x in inputs}) >= 3
    ref = _standalone(dsg, inputs, 2)
    with dsg.Ensemble(inputs, workers=4, batched=1) as e:
        e.step(1)
        e.step(2)
        for i in range(len(inputs)):
            for f in ("p", "u", "v", "w", "cc"):
                assert np.array_equal(e.member(i).field(f), ref[i][0][f]), (i, f)


def test_batched_needs_mixed_members(gpu_lib):
    dsg = gpu_lib
    inputs = _inputs(dsg, dsg.config.MODE_TOL_MIXED)
    inputs[2] = inputs[2].replace(mode=dsg.config.MODE_TOL_FP64)
    with dsg.Ensemble(inputs, workers=2) as e:
        with pytest.raises(dsg.DsgError) as ex:
            e.set_batched(1)
        assert ex.value.code == -1 and "member 2" in str(ex.value)
        assert e.batched == 0
        e.step(1)
