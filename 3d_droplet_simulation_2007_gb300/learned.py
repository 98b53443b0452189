"""The learned multigrid initial guess: host wrapper and training driver.

A ``Net`` is the 3D convolutional U-Net of ``csrc/nn.cu`` (BF16 tcgen05
tensor-core kernels, FP32 accumulation) sized for one interior grid.  The
method without it starts every mixed-precision pressure solve from the FP32
full-multigrid (FMG) guess p0; the network predicts the correction of p0 --
from the volume fraction (density), the divergence right-hand side, the FP64
defect of p0, p0 itself and the previous-step pressure -- and in
``MODE_LEARNED`` the solver adds it, scaled to the least FP64 defect, only
when that cuts the V-cycles it expects to need (otherwise it keeps p0 and
rests the network for 1, 2, 4 .. 32 solves).

``train`` runs the solver itself on droplets of random diameter (1-3 mm) and
impact speed (0.5-4 m/s), records after every pressure solve the pair
(features at the start, solved pressure minus p0) and takes one Adam step on
it: the network learns from the solver's own snapshots, on the fly.  Training
runs at 128^3 and is then continued at the grid the network will serve (the
parameters carry over between grid sizes: the network is convolutional).
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from .config import InputData, MODE_LEARNED, MODE_TOL_MIXED, droplet

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "warmstart_weights.npy")


class Net:
    """One network instance on the current CUDA device."""

    def __init__(self, W, H=None, D=None, seed=0):
        self.lib = _lib.load()
        H = W if H is None else H
        D = W if D is None else D
        h = C.c_void_p()
        _lib.check(self.lib.dsg_net_create(W, H, D, seed, C.byref(h)))
        self.h = h
        self.shape = (D, H, W)
        self.nparams = int(self.lib.dsg_net_param_count())

    def close(self):
        if getattr(self, "h", None):
            self.lib.dsg_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        out = np.empty(self.nparams, dtype=np.float32)
        _lib.check(self.lib.dsg_net_get_params(self.h, out.ctypes.data, self.nparams))
        return out

    @params.setter
    def params(self, value):
        v = np.ascontiguousarray(value, dtype=np.float32)
        if v.size != self.nparams:
            raise ValueError("expected %d parameters" % self.nparams)
        _lib.check(self.lib.dsg_net_set_params(self.h, v.ctypes.data, self.nparams))

    def forward(self, x):
        """x: (D, H, W, NET_INPUTS) -> (D, H, W)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        assert x.shape == self.shape + (_lib.NET_INPUTS,)
        y = np.empty(self.shape, dtype=np.float32)
        _lib.check(self.lib.dsg_net_forward_host(self.h, x.ctypes.data, y.ctypes.data))
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_float()
        _lib.check(self.lib.dsg_net_grad_host(self.h, x.ctypes.data, t.ctypes.data, C.byref(loss), g.ctypes.data))
        return float(loss.value), g

    def train_step(self, lr):
        loss = C.c_float()
        _lib.check(self.lib.dsg_net_train_step(self.h, lr, C.byref(loss)))
        return float(loss.value)

    def attach(self, solver, record=False):
        _lib.check(self.lib.dsg_attach_net(solver.ctx, self.h, 1 if record else 0), solver.ctx)
        solver.net = self

    def save(self, path=WEIGHTS):
        np.save(path, self.params)

    def load(self, path=WEIGHTS):
        self.params = np.load(path)
        return self


def detach(solver):
    _lib.check(_lib.load().dsg_attach_net(solver.ctx, None, 0), solver.ctx)
    solver.net = None


def training_instances(count, seed=0):
    """Droplet diameters U[1,3] mm and impact speeds U[0.5,4] m/s (seeded)."""
    rng = np.random.default_rng(seed)
    return [(float(rng.uniform(1e-3, 3e-3)), float(rng.uniform(0.5, 4.0))) for _ in range(count)]


def train(n=128, instances=20, steps=1000, lr=1e-3, seed=0, log=None, tol=1e-8, max_seconds=None, net=None):
    """Train a network on the solver's own snapshots at n^3 (one Adam step per
    solved time step from the third step on).  Continues ``net`` if given
    (sized n^3).  Stops early, between instances, once ``max_seconds`` of wall
    clock have passed.  Returns (net, history of losses)."""
    import time
    from .solver import Solver
    net = Net(n, seed=seed) if net is None else net
    losses = []
    t0 = time.perf_counter()
    for k, (diam, speed) in enumerate(training_instances(instances, seed)):
        if max_seconds is not None and k > 0 and time.perf_counter() - t0 > max_seconds:
            break
        inp = droplet(n, steps=steps, impact_speed=speed, diameter=diam, noise_si=1e-4, mode=MODE_TOL_MIXED,
                      tol=tol, npre=4, npost=4, ntop=4, seed=seed * 1000 + k)
        with Solver(inp) as s:
            net.attach(s, record=True)
            for t in range(1, steps + 1):
                try:
                    s.step(t)
                except _lib.DsgError as e:  # an unconverged or blown-up run ends its instance
                    if log:
                        log("instance %d stopped at step %d: %s" % (k, t, e))
                    break
                if t > 2:  # the first two steps lack a pressure history
                    losses.append(net.train_step(lr))
            detach(s)
        if log:
            log("n=%d instance %d (D=%.2f mm, v=%.2f m/s): mean loss of its last 50 steps %.4g"
                % (n, k, diam * 1e3, speed, float(np.mean(losses[-50:])) if losses else float("nan")))
    return net, losses


def resized(net, n):
    """A network for an n^3 grid with the parameters of ``net``."""
    out = Net(n)
    out.params = net.params
    return out


def learned_config(inp):
    """The same run with the learned initial guess."""
    d = inp.as_dict() if isinstance(inp, InputData) else dict(inp)
    d["mode"] = MODE_LEARNED
    return InputData(**d)


def evaluate(inp, net=None, steps=8, warmup=2):
    """Run `steps` time steps (after `warmup`) and report V-cycles, initial
    residuals, guard fallbacks and ms per step."""
    import time
    from .solver import Solver
    keys = ("vcycles", "relres_init", "fallback", "relres_net", "relres_base")
    out = {k: [] for k in keys}
    with Solver(inp) as s:
        if net is not None:
            net.attach(s)
        for t in range(1, warmup + 1):
            s.step(t)
        s.synchronize()
        t0 = time.perf_counter()
        for t in range(warmup + 1, warmup + steps + 1):
            st = s.step(t)
            for k in keys:
                out[k].append(st[k])
        s.synchronize()
        out["ms_per_step"] = 1e3 * (time.perf_counter() - t0) / steps
        if net is not None:
            detach(s)
    return out


def compare_starts(n, net, steps=8, warmup=20, speed=3.0, diameter=2e-3, seed=0):
    """V-cycles and time per step at n^3 from the FP32 full-multigrid start
    (the method without the network), from the previous-step pressure, and
    from the guarded learned correction of the full-multigrid start."""
    base = droplet(n, steps=1000, impact_speed=speed, diameter=diameter, noise_si=1e-4, mode=MODE_TOL_MIXED,
                   tol=1e-8, npre=4, npost=4, ntop=4, seed=seed)
    return {"fmg_start": evaluate(base, steps=steps, warmup=warmup),
            "previous_pressure_start": evaluate(base.replace(warm_start=1), steps=steps, warmup=warmup),
            "learned_start": evaluate(learned_config(base), net, steps=steps, warmup=warmup)}


def main(argv=None):
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description="train the learned initial guess on solver snapshots")
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--instances", type=int, default=20)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--fine-n", type=int, default=256, help="grid of the second training phase (0: none)")
    ap.add_argument("--fine-instances", type=int, default=4)
    ap.add_argument("--fine-steps", type=int, default=400)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval-steps", type=int, default=8)
    ap.add_argument("--eval-warmup", type=int, default=20)
    ap.add_argument("--max-seconds", type=float, default=None)
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    net, losses = train(a.n, a.instances, a.steps, a.lr, a.seed, log=print, max_seconds=a.max_seconds)
    t1 = time.perf_counter()
    rec = {"snapshots": len(losses), "train_s": t1 - t0, "loss_first": float(np.mean(losses[:50])),
           "loss_last": float(np.mean(losses[-200:]))}
    if a.fine_n:
        net = resized(net, a.fine_n)
        net, l2 = train(a.fine_n, a.fine_instances, a.fine_steps, 0.5 * a.lr, a.seed + 1, log=print, net=net)
        rec.update({"fine_n": a.fine_n, "fine_snapshots": len(l2), "fine_train_s": time.perf_counter() - t1,
                    "fine_loss_first": float(np.mean(l2[:20])), "fine_loss_last": float(np.mean(l2[-100:]))})
    net.save(a.out)
    print(json.dumps(rec))
    if a.eval_steps:
        n = a.fine_n or a.n
        ev = resized(net, n)
        print(json.dumps({"n": n, **compare_starts(n, ev, a.eval_steps, a.eval_warmup)}))


if __name__ == "__main__":
    main()
