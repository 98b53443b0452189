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
