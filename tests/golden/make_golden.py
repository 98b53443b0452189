"""Generate the golden fixtures of the CPU oracle.

    python tests/golden/make_golden.py

writes one JSON file per case next to this script.  Values are stored as
float.hex strings so the fixtures pin the oracle bit for bit.  The reference
(main.f) cannot be compiled here (no Fortran compiler), so these fixtures are
generated by the oracle itself: they pin it against regressions, and the GPU
tests check the CUDA path against them.
"""
import importlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle.oracle as oo  # noqa: E402

FIELDS = ("cc", "p", "u", "v", "w", "s11", "s12")


def _hex(x):
    return float(x).hex()


def field_digest(a):
    """Size-independent digest of a field: sum, sum of squares, max |.|, and
    a few fixed probes."""
    a = np.asarray(a, dtype=np.float64)
    flat = a.reshape(-1, order="F")
    probes = [flat[(len(flat) * q) // 7] for q in range(1, 7)]
    return [_hex(flat.sum()), _hex((flat * flat).sum()), _hex(np.abs(flat).max())] + [_hex(v) for v in probes]


def case_al3d_fl3d():
    rng = np.random.default_rng(11)
    out = {}
    for n in range(24):
        m = rng.uniform(0.0, 1.0, size=3)
        m /= m.sum()
        c = float(rng.uniform(0.0, 1.0))
        al = oo.al3d(m[0], m[1], m[2], c)
        out["al3d_%02d" % n] = _hex(al)
        out["fl3d_%02d" % n] = _hex(oo.fl3d(m[0], m[1], m[2], al, 0.1, 0.7))
    return out


def case_relax10():
    rng = np.random.default_rng(12)
    shape = (10, 10, 10)
    a, b, c = (rng.uniform(1.0, 833.0, size=shape) for _ in range(3))
    ei = 1.0 / (a + b + c + 1.0)
    rhs = rng.standard_normal(shape)
    u = rng.standard_normal(shape)
    u1 = oo.relax(u, 1.0, rhs, a, b, c, ei, 1.5)
    r = oo.resid(1.0, u1, rhs, a, b, c)
    return {"u": field_digest(u1), "res": field_digest(r)}


def droplet16():
    dsg = importlib.import_module("3d_droplet_simulation_2007_gb300.config")
    return dsg.droplet(16, steps=3, noise_si=1e-4, mode=oo.MODE_REF_EXACT)


def case_step16():
    o = oo.Oracle(droplet16().as_dict())
    out = {}
    for t in (1, 2, 3):
        o.step(t)
        for name in FIELDS:
            out["t%d_%s" % (t, name)] = field_digest(o.field(name))
        out["t%d_volume" % t] = _hex(o.liquid_volume())
        out["t%d_tau" % t] = _hex(o.scalars().tau)
    return out


CASES = {"al3d_fl3d": case_al3d_fl3d, "relax10": case_relax10, "step16": case_step16}


def compute(fn):
    return fn()


def main():
    for name, fn in CASES.items():
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump({"case": name, "values": fn()}, f, indent=1, sort_keys=True)
        print("wrote", name)


if __name__ == "__main__":
    main()
