"""Ensemble host logic without a GPU: the member plan and the study configs."""
import numpy as np


def test_plan_is_longest_processing_time_first(dsg):
    ens = dsg.ensemble
    costs = np.array([5.0, 1.0, 4.0, 3.0, 3.0, 2.0, 2.0])
    a = ens.plan(costs, 3)
    loads = np.bincount(a, weights=costs, minlength=3)
    # costs in decreasing order, each to the least-loaded worker: {5, 2}, {4, 2, 1}, {3, 3}
    assert sorted(loads.tolist()) == [6.0, 7.0, 7.0]
    assert set(a.tolist()) <= {0, 1, 2}
    # one worker takes everything; more workers than members leave some idle
    assert (ens.plan(costs, 1) == 0).all()
    b = ens.plan(costs[:2], 5)
    assert b[0] != b[1]


def test_plan_balances_the_droplet_study(dsg):
    ens = dsg.ensemble
    cfgs = ens.study_configs(64)
    cost = np.array([(c.nx - 2) ** 3 + 2e6 for c in cfgs])
    for w in (4, 8, 16):
        loads = np.bincount(ens.plan(cost, w), weights=cost, minlength=w)
        assert loads.max() <= loads.sum() / w + cost.max()


def test_study_configs(dsg):
    ens = dsg.ensemble
    cfgs = ens.study_configs(64)
    assert len(cfgs) == 64
    sides = {c.nx - 2 for c in cfgs}
    assert sides <= {48, 64, 96, 128, 160} and len(sides) == 5
    we = [1000.0 * c.yvel1_si ** 2 * 2e-3 / 0.072 for c in cfgs]
    assert 50.0 <= min(we) and max(we) <= 800.0
    assert [c.noise_seed for c in cfgs] == list(range(1000, 1064))
    assert cfgs == ens.study_configs(64)  # seeded
