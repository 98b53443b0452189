"""The learned initial guess: tensor-core network kernels against the numpy
oracle, training, and the guarded learned solve.

The oracle (oracle/nn_oracle.py) rounds to bfloat16 where the GPU stores
bfloat16; what remains is FP32 accumulation order, which can flip the bf16
rounding of single stored values (2^-8 relative), so forward outputs are
compared at 2e-2 of their max-norm and gradients per layer at 3e-2 of their
norm with a cosine above 0.999.
"""
import numpy as np
import pytest

import oracle.nn_oracle as NO
from conftest import relerr

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16, 16), (8, 16, 24)]  # (D, H, W)
# large enough for the z-marching conv columns: 4 planes per CTA at 64^3, 8 at 32x256x256
DEEP_SHAPES = [(64, 64, 64), (32, 256, 256)]


def _net(dsg, shape, seed=3):
    from importlib import import_module
    learned = import_module(dsg.__name__ + ".learned")
    D, H, W = shape
    return learned.Net(W, H, D, seed=seed), learned


def _inputs(shape, seed):
    r = np.random.default_rng(seed)
    x = r.standard_normal(shape + (NO.CIN,)).astype(np.float32)
    x[..., 0] = r.uniform(0.0, 1.0, size=shape)
    t = r.standard_normal(shape).astype(np.float32) * 0.1
    return x, t


def test_param_count(gpu_lib):
    assert gpu_lib.load().dsg_net_param_count() == NO.param_count() == 251649
    assert gpu_lib._lib.NET_INPUTS == NO.CIN


@pytest.mark.parametrize("shape", SHAPES)
def test_forward_matches_oracle(gpu_lib, shape):
    net, _ = _net(gpu_lib, shape)
    # larger biases and a non-trivial output layer so every path is exercised
    p = net.params.copy()
    r = np.random.default_rng(5)
    p += (r.standard_normal(p.size) * 0.02).astype(np.float32)
    net.params = p
    x, _ = _inputs(shape, 1)
    y = net.forward(x)
    y_ref, _ = NO.forward(p.astype(np.float64), x.astype(np.float64), bf16=True)
    assert np.all(np.isfinite(y))
    assert relerr(y, y_ref) < 2e-2, relerr(y, y_ref)


@pytest.mark.parametrize("shape", SHAPES)
def test_gradients_match_oracle(gpu_lib, shape):
    net, _ = _net(gpu_lib, shape, seed=7)
    p = net.params.copy()
    p += (np.random.default_rng(6).standard_normal(p.size) * 0.02).astype(np.float32)
    net.params = p
    x, t = _inputs(shape, 2)
    loss, g = net.loss_grad(x, t)
    loss_ref, g_ref, _ = NO.loss_and_grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - loss_ref) <= 1e-2 * loss_ref
    off = 0
    for l, (ci, co, _) in enumerate(NO.LAYERS):
        n = 27 * ci * co + co
        a, b = g[off:off + n].astype(np.float64), g_ref[off:off + n]
        off += n
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = float(a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30))
        assert err < 3e-2 and cos > 0.999, (l, err, cos)


@pytest.mark.parametrize("shape", DEEP_SHAPES)
def test_forward_deep_columns_match_oracle(gpu_lib, shape):
    net, _ = _net(gpu_lib, shape, seed=11)
    p = net.params.copy()
    p += (np.random.default_rng(12).standard_normal(p.size) * 0.02).astype(np.float32)
    net.params = p
    x, _ = _inputs(shape, 13)
    y = net.forward(x)
    y_ref, _ = NO.forward(p.astype(np.float64), x.astype(np.float64), bf16=True)
    assert relerr(y, y_ref) < 2e-2, relerr(y, y_ref)


def test_gradients_deep_columns_match_oracle(gpu_lib):
    shape = DEEP_SHAPES[0]
    net, _ = _net(gpu_lib, shape, seed=14)
    p = net.params.copy()
    p += (np.random.default_rng(15).standard_normal(p.size) * 0.02).astype(np.float32)
    net.params = p
    x, t = _inputs(shape, 16)
    _, g = net.loss_grad(x, t)
    _, g_ref, _ = NO.loss_and_grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
    off = 0
    for l, (ci, co, _) in enumerate(NO.LAYERS):
        n = 27 * ci * co + co
        a, b = g[off:off + n].astype(np.float64), g_ref[off:off + n]
        off += n
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = float(a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30))
        assert err < 3e-2 and cos > 0.999, (l, err, cos)


def test_gradients_close_to_fp64(gpu_lib):
    """Against the oracle without bf16 rounding: the gradient direction holds."""
    shape = (16, 16, 16)
    net, _ = _net(gpu_lib, shape, seed=8)
    p = net.params
    x, t = _inputs(shape, 4)
    _, g = net.loss_grad(x, t)
    _, g64, _ = NO.loss_and_grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64), bf16=False)
    cos = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
    assert cos > 0.99, cos


def test_training_on_solver_snapshots_reduces_loss(gpu_lib):
    dsg = gpu_lib
    net, learned = _net(dsg, (32, 32, 32), seed=1)
    inp = dsg.config.droplet(32, mode=dsg.config.MODE_TOL_MIXED, tol=1e-9, impact_speed=2.0)
    losses = []
    with dsg.Solver(inp) as s:
        net.attach(s, record=True)
        for t in range(1, 61):
            s.step(t)
            if t > 1:
                losses.append(net.train_step(2e-3))
        learned.detach(s)
    assert all(np.isfinite(losses))
    assert np.mean(losses[-10:]) < 0.5 * np.mean(losses[:5]), (losses[:5], losses[-10:])


def test_learned_mode_converges_and_guards(gpu_lib):
    """Learned mode reaches the tolerance; the guard either keeps the
    full-multigrid start untouched (fallback) or adds the network's correction,
    whose defect it predicted from three sums over the FP32 defect (to 1e-4); the network rests 1, 2,
    4 .. solves after each rejection; fields match the FP64 oracle from the
    same state."""
    dsg = gpu_lib
    from oracle import Oracle
    from test_mixed_gpu import _sync_state
    tol = 1e-10
    net, _ = _net(dsg, (32, 32, 32), seed=2)
    ora = Oracle(dsg.config.droplet(32, mode=dsg.config.MODE_TOL_FP64, tol=tol).as_dict())
    gpu = dsg.Solver(dsg.config.droplet(32, mode=dsg.config.MODE_LEARNED, tol=tol), init=False)
    net.attach(gpu)
    hist = np.zeros(ora.shape)
    rest, backoff = 0, 1
    for t in range(1, 9):
        _sync_state(gpu, ora)
        gpu.set_field("pprev", hist)
        ora.step(t)
        st = gpu.step(t)
        assert st["converged"] == 1 and st["relres"] < tol, st
        if rest > 0:  # the network rests: full-multigrid start, no inference
            assert st["relres_net"] == -1.0 and st["fallback"] == 1, (t, st)
            rest -= 1
        else:
            assert st["relres_net"] >= 0.0, (t, st)
            # the minimal-residual step is never worse than the start
            assert st["relres_net"] <= st["relres_base"] * (1 + 1e-9), st
            if st["fallback"] == 0:
                assert abs(st["relres_init"] - st["relres_net"]) <= 1e-4 * st["relres_net"], st
                backoff = 1
            else:
                assert st["relres_init"] == st["relres_base"], st
                rest, backoff = backoff, min(2 * backoff, 32)
        for name in ("p", "u", "v", "w", "cc"):
            assert relerr(gpu.field(name), ora.field(name)) < 1e-7, (t, name)
        hist = ora.field("p").copy()


def test_learned_rejection_keeps_the_full_multigrid_start(gpu_lib):
    """A network whose correction is rejected leaves the solve bit-identical
    to the mode without it (tol_mixed) from the same state."""
    dsg = gpu_lib
    net, _ = _net(dsg, (32, 32, 32), seed=4)
    p = net.params
    p[:] = 0.0  # zero output: the correction is zero and cuts nothing
    net.params = p
    inp = dsg.config.droplet(32, mode=dsg.config.MODE_TOL_MIXED, tol=1e-9)
    with dsg.Solver(inp) as a, dsg.Solver(inp.replace(mode=dsg.config.MODE_LEARNED)) as b:
        net.attach(b)
        for t in range(1, 6):
            sa, sb = a.step(t), b.step(t)
            assert sb["fallback"] == 1 and sb["relres_base"] == sa["relres_init"], (t, sa, sb)
            assert sb["vcycles"] == sa["vcycles"]
            for name in ("p", "u", "v", "w", "cc"):
                assert np.array_equal(a.field(name), b.field(name)), (t, name)


def test_learned_mode_needs_network(gpu_lib):
    dsg = gpu_lib
    with dsg.Solver(dsg.config.droplet(16, mode=dsg.config.MODE_LEARNED, tol=1e-8)) as s:
        with pytest.raises(dsg.DsgError) as e:
            s.step(1)
        assert e.value.code == -6


def test_trained_network_against_the_full_multigrid_start(gpu_lib):
    """The committed network (trained on the solver's own 128^3 and 256^3
    snapshots) on a droplet it was not trained on, against the method without
    it: the full-multigrid start of tol_mixed.  Its scaled correction never
    raises the start's defect; what it gains is recorded (median defect ratio,
    V-cycles); and the guard keeps learned mode no slower than tol_mixed: no
    more V-cycles in total and at most 10 % more time over 60 steps."""
    dsg = gpu_lib
    import time
    from importlib import import_module
    learned = import_module(dsg.__name__ + ".learned")
    import os
    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("no trained weights")
    net = learned.Net(128).load()
    base = dsg.config.droplet(128, steps=1000, impact_speed=2.5, diameter=1.8e-3, mode=dsg.config.MODE_TOL_MIXED,
                              tol=1e-8, npre=4, npost=4, ntop=4, seed=77)
    runs = {}
    for name, inp in (("tol_mixed", base), ("learned", learned.learned_config(base))):
        rec = {"vcycles": 0, "ratios": [], "kept": 0, "ms": 0.0}
        with dsg.Solver(inp) as s:
            if name == "learned":
                net.attach(s)
            for t in range(1, 61):
                s.synchronize()
                t0 = time.perf_counter()
                st = s.step(t)
                s.synchronize()
                if t > 10:
                    rec["ms"] += 1e3 * (time.perf_counter() - t0)
                assert st["converged"] == 1
                rec["vcycles"] += st["vcycles"]
                if name == "learned" and st["relres_net"] >= 0:
                    assert st["relres_net"] <= st["relres_base"] * (1 + 1e-9), (t, st)
                    rec["ratios"].append(st["relres_net"] / st["relres_base"])
                    rec["kept"] += 1 - st["fallback"]
            if name == "learned":
                learned.detach(s)
        runs[name] = rec
    lr, tm = runs["learned"], runs["tol_mixed"]
    print("learned vs tol_mixed over 60 steps: V-cycles %d vs %d, ms (steps 11-60) %.1f vs %.1f, "
          "network ran %d times, kept %d, median defect ratio %.3f"
          % (lr["vcycles"], tm["vcycles"], lr["ms"], tm["ms"], len(lr["ratios"]), lr["kept"],
             float(np.median(lr["ratios"])) if lr["ratios"] else float("nan")))
    assert lr["ratios"], "the network never ran"
    assert lr["vcycles"] <= tm["vcycles"]
    assert lr["ms"] <= 1.10 * tm["ms"], (lr["ms"], tm["ms"])
