"""Many independent droplet simulations stepped together on one GPU.

:class:`Ensemble` wraps ``dsg_ensemble`` (include/dsg.h): n contexts, each a
full simulation with its fields resident in HBM, stepped by a pool of host
threads on their own CUDA streams so that the members' kernels overlap on the
GPU.  The autotuner measures each member's step time and picks the number of
worker threads by timing real steps.  In batched mode (``batched=groups``) the
members' pressure solves run as batched solves -- one launch per multigrid
pass over all members of a cost-balanced group, under CUDA graphs, the groups
side by side -- and ``autotune_tiles`` picks the coarse-tail depth and the
thread-block shape of every batched pass by timing.  The reference runs one
case per process; this is the batched study of droplet sizes and Weber
numbers.
"""
import ctypes as C
import math

import numpy as np

from . import _lib
from .config import InputData, MODE_TOL_MIXED, droplet
from .solver import Solver, to_config


def study_configs(count=64, sides=(48, 64, 96, 128, 160), we_range=(50.0, 800.0), diameter=2e-3, seed=1000,
                  mode=MODE_TOL_MIXED, tol=1e-8, steps=1000, **kw):
    """The droplet study: member i has seed ``seed + i``, a grid side drawn
    from ``sides`` and a Weber number rho1 v^2 D / sigma log-uniform in
    ``we_range`` (impact speed v = sqrt(We sigma / (rho1 D)))."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        n = int(sides[int(rng.integers(len(sides)))])
        we = math.exp(rng.uniform(math.log(we_range[0]), math.log(we_range[1])))
        speed = math.sqrt(we * 0.072 / (1000.0 * diameter))
        out.append(droplet(n, steps=steps, impact_speed=speed, diameter=diameter, noise_si=1e-4, mode=mode,
                           tol=tol, npre=4, npost=4, ntop=4, seed=seed + i, **kw))
    return out


class Ensemble:
    """n simulations stepped together; ``member(i)`` is a Solver view."""

    def __init__(self, inputs, workers=0, batched=0):
        self.lib = _lib.load()
        self.inputs = [x if isinstance(x, InputData) else InputData(**x) for x in inputs]
        n = len(self.inputs)
        cfgs = (_lib.DsgConfig * n)(*[to_config(x) for x in self.inputs])
        h = C.c_void_p()
        _lib.check(self.lib.dsg_ensemble_create(cfgs, n, workers, C.byref(h)))
        self.h = h
        self.n = n
        self.t = 0
        self._members = [Solver(self.inputs[i], ctx=self.lib.dsg_ensemble_member(h, i)) for i in range(n)]
        if batched:
            self.set_batched(int(batched))

    def set_batched(self, groups=1):
        """Solve the members' pressures as `groups` batched solves per step
        (True = 1 group), each over a cost-balanced group of members on its
        own stream, or each member on its own (0 / False)."""
        self._ck(self.lib.dsg_ensemble_set_batched(self.h, int(groups)))

    @property
    def batched(self):
        """Number of batched groups (0: per-member solves)."""
        return int(self.lib.dsg_ensemble_batched(self.h))

    @property
    def batch_tail_nodes(self):
        """Largest level (nodes) of the members' coarse tails in the batch."""
        return int(self.lib.dsg_ensemble_batch_tail_nodes(self.h))

    def autotune_tiles(self, reps=5):
        """Pick the coarse-tail depth and the thread-block shape of every
        batched pass by timing; returns the number of passes tuned."""
        k = C.c_int()
        self._ck(self.lib.dsg_ensemble_autotune_tiles(self.h, reps, C.byref(k)))
        return k.value

    def phase_ms(self):
        """Batched mode: host time of the last step's phases (up to the
        solves, the batched solves, after the solves), ms."""
        out = np.zeros(3)
        self._ck(self.lib.dsg_ensemble_phase_ms(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def close(self):
        if getattr(self, "h", None):
            for m in self._members:
                m.ctx = None
            self.lib.dsg_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, rc):
        if rc != _lib.DSG_OK:
            msg = self.lib.dsg_ensemble_last_error(self.h) or self.lib.dsg_last_error(None)
            raise _lib.DsgError(rc, msg.decode() if msg else "")
        return rc

    def member(self, i):
        return self._members[i]

    @property
    def workers(self):
        return self.lib.dsg_ensemble_workers(self.h)

    def set_workers(self, w):
        self._ck(self.lib.dsg_ensemble_set_workers(self.h, w))

    def step(self, t=None):
        """One time step of every member; returns their solve statistics."""
        t = self.t + 1 if t is None else t
        st = (_lib.DsgMgStats * self.n)()
        self._ck(self.lib.dsg_ensemble_step(self.h, t, st))
        self.t = t
        return [s.as_dict() for s in st]

    @property
    def last_ms(self):
        return self.lib.dsg_ensemble_last_ms(self.h)

    def member_ms(self):
        out = np.zeros(self.n)
        self._ck(self.lib.dsg_ensemble_member_ms(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def autotune(self, steps_per_trial=2):
        """Run real steps to measure member costs and pick the worker count."""
        tn, bw = C.c_int(), C.c_int()
        self._ck(self.lib.dsg_ensemble_autotune(self.h, self.t + 1, steps_per_trial, C.byref(tn), C.byref(bw)))
        self.t = tn.value - 1
        return bw.value


def member_cost(inp):
    """Cost model of one member's step: launch-bound floor + interior cells."""
    return float((inp.nx - 2) * (inp.ny - 2) * (inp.nz - 2)) + 2.0e6


def shard(inputs, rank, world):
    """Indices of the members that rank `rank` of `world` steps: members are
    independent, so the ensemble splits across GPUs with no data exchange,
    balanced longest-processing-time-first on the cost model."""
    if world <= 1:
        return list(range(len(inputs)))
    owner = plan([member_cost(x) for x in inputs], world)
    return [i for i in range(len(inputs)) if owner[i] == rank]


def plan(costs, workers):
    """Worker of each member under the longest-processing-time-first plan."""
    lib = _lib.load()
    c = np.ascontiguousarray(costs, dtype=np.float64)
    out = np.zeros(len(c), dtype=np.int32)
    _lib.check(lib.dsg_ensemble_plan(c.ctypes.data_as(C.POINTER(C.c_double)), len(c), workers,
                                     out.ctypes.data_as(C.POINTER(C.c_int))))
    return out
