"""Oracle trajectories of the droplet-on-wall study, as per-step field digests.

    python tests/golden/trajectory.py [name ...]

runs the CPU oracle (test infrastructure) over the whole time loop of each case
and writes ``<name>.npz`` next to this script (``<name>_env`` writes the
case's round-off envelope, see :func:`generate_envelope`):

* ``traj64_ref``  -- 64^3 interior (66^3 nodes), 200 steps, 1 m/s, seeded
  +-1e-4 m/s noise, mglin exactly as the reference runs it (FMG, fixed cycles);
* ``traj64_tol``  -- the same case with the multigrid driven to a relative
  residual of 1e-10 (FMG, then V-cycles until ||rhs - L p|| / ||rhs|| < 1e-10);
* ``traj128_ref`` -- 128^3 interior (130^3 nodes), 500 steps, the reference's
  fixed-cycle mglin.

A full 130^3 field is 17.6 MB, so the fixtures hold digests instead of fields:
for each of p, u, v, w, cc after every step, five aggregates over the whole
array (ghosts included) -- sum, sum of |.|, sum of squares, max |.| and a sum
weighted by fixed pseudo-random weights in [-1, 1] -- and every ``sample_every``
steps the values at 16 fixed cells.  Per step also: tau, the liquid volume
SUMFIELD(cc) (main.f:4783-4801), NPRE, NPOST, NTOP, tswap and the V-cycle count
of the tolerance mode.  The GPU tests compute the same digests from their own
fields and compare them within the field tolerance (1e-10) and the volume
tolerance (1e-12), or within ten times the algorithm's own round-off envelope
where a sensitive step of the flow amplifies one-ulp differences beyond those
(see :func:`generate_envelope`, :func:`bars`, :func:`compare`).
"""
import importlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DIGEST_FIELDS = ("p", "u", "v", "w", "cc")
AGGREGATES = ("sum", "sumabs", "sumsq", "maxabs", "wsum")
N_SAMPLES = 16
SCALARS = ("tau", "volume", "npre", "npost", "ntop", "tswap", "vcycles")
ENV_COLUMNS = DIGEST_FIELDS + ("volume", "tau")


def _config():
    return importlib.import_module("3d_droplet_simulation_2007_gb300.config")


def cases():
    cfg = _config()
    return {
        "traj64_ref": dict(inp=cfg.droplet(64, steps=200, mode=cfg.MODE_REF_EXACT), sample_every=1),
        "traj64_tol": dict(inp=cfg.droplet(64, steps=200, mode=cfg.MODE_TOL_FP64, tol=1e-10), sample_every=1),
        "traj128_ref": dict(inp=cfg.droplet(128, steps=500, mode=cfg.MODE_REF_EXACT), sample_every=10),
    }


def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


_WEIGHTS = {}


def weights(n):
    """Fixed weights in [-1, 1) for a flat field of n values (column-major)."""
    if n not in _WEIGHTS:
        with np.errstate(over="ignore"):
            h = _splitmix64(np.arange(n, dtype=np.uint64))
        _WEIGHTS[n] = (h >> np.uint64(11)).astype(np.float64) * (2.0 ** -52) - 1.0
    return _WEIGHTS[n]


def sample_index(n):
    """16 fixed flat indices spread over a field of n values."""
    with np.errstate(over="ignore"):
        h = _splitmix64(np.arange(1000, 1000 + N_SAMPLES, dtype=np.uint64))
    return (h % np.uint64(n)).astype(np.int64)


def digest(a):
    """Five aggregates of a field (Fortran-ordered array, ghosts included)."""
    flat = np.asarray(a, dtype=np.float64).reshape(-1, order="F")
    ab = np.abs(flat)
    return np.array([flat.sum(), ab.sum(), (flat * flat).sum(), ab.max(), (flat * weights(flat.size)).sum()])


def samples(a):
    flat = np.asarray(a, dtype=np.float64).reshape(-1, order="F")
    return flat[sample_index(flat.size)]


def record(fields, scalars):
    """One step's digests from a dict of fields and a dict of scalars."""
    agg = np.stack([digest(fields[f]) for f in DIGEST_FIELDS])
    smp = np.stack([samples(fields[f]) for f in DIGEST_FIELDS])
    sc = np.array([float(scalars[k]) for k in SCALARS])
    return agg, smp, sc


def generate(name, spec, verbose=True):
    from oracle import Oracle
    inp = spec["inp"]
    o = Oracle(inp.as_dict())
    steps = inp.tmax
    agg = np.zeros((steps, len(DIGEST_FIELDS), len(AGGREGATES)))
    smp_steps = list(range(spec["sample_every"], steps + 1, spec["sample_every"]))
    smp = np.zeros((len(smp_steps), len(DIGEST_FIELDS), N_SAMPLES))
    sc = np.zeros((steps, len(SCALARS)))
    t0 = time.time()
    for t in range(1, steps + 1):
        o.step(t)
        s = o.scalars()
        fields = {f: o.field(f) for f in DIGEST_FIELDS}
        scal = dict(tau=s.tau, volume=o.liquid_volume(), npre=s.npre, npost=s.npost, ntop=s.ntop,
                    tswap=s.tswap, vcycles=s.last_vcycles)
        a, m, c = record(fields, scal)
        agg[t - 1], sc[t - 1] = a, c
        if t in smp_steps:
            smp[smp_steps.index(t)] = m
        if verbose and t % 50 == 0:
            print("%s: step %d/%d  %.1f s" % (name, t, steps, time.time() - t0), flush=True)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), agg=agg, smp=smp, smp_steps=np.array(smp_steps),
                        sc=sc, n=np.array([inp.nx - 2]), mode=np.array([inp.mode]), tol=np.array([inp.tol]))


def generate_envelope(name, spec, verbose=True):
    """Round-off sensitivity of the algorithm itself: the oracle against the
    oracle started from velocities one ulp larger (u, v, w times 1 + 2^-52):
    max-norm relative error of p, u, v, w, cc, then the relative difference
    of the liquid volume and of tau, after every step (ENV_COLUMNS).  Written to
    ``<name>_env.npz``.  An implementation that rounds differently (another
    compiler, libm, FMA contraction or reduction order) cannot be expected to
    stay closer to the oracle than this."""
    from oracle import Oracle
    inp = spec["inp"]
    a, b = Oracle(inp.as_dict()), Oracle(inp.as_dict())
    for f in ("u", "v", "w"):
        x = b.field(f)
        x[...] = x * (1.0 + 2.0 ** -52)
    steps = inp.tmax
    err = np.zeros((steps, len(ENV_COLUMNS)))
    t0 = time.time()
    for t in range(1, steps + 1):
        a.step(t)
        b.step(t)
        for q, f in enumerate(DIGEST_FIELDS):
            x, y = b.field(f), a.field(f)
            scale = float(np.max(np.abs(y)))
            err[t - 1, q] = float(np.max(np.abs(x - y))) / (scale if scale > 0 else 1.0)
        va, vb = a.liquid_volume(), b.liquid_volume()
        err[t - 1, len(DIGEST_FIELDS)] = abs(vb - va) / abs(va)
        ta, tb = a.scalars().tau, b.scalars().tau
        err[t - 1, len(DIGEST_FIELDS) + 1] = abs(tb - ta) / abs(ta)
        if verbose and t % 50 == 0:
            print("%s envelope: step %d/%d  %.1f s" % (name, t, steps, time.time() - t0), flush=True)
    np.savez_compressed(os.path.join(HERE, name + "_env.npz"), err=err)


def load_envelope(name):
    return np.load(os.path.join(HERE, name + "_env.npz"))["err"]


def load(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    return {k: z[k] for k in z.files}


def bars(env, t, field_tol=1e-10, volume_tol=1e-12, tau_tol=1e-12, factor=10.0):
    """Per-quantity bar of step t: the fixed tolerance, or `factor` times the
    algorithm's own round-off envelope at that step where that is larger."""
    e = env[t - 1]
    out = {}
    for q, f in enumerate(ENV_COLUMNS):
        base = {"volume": volume_tol, "tau": tau_tol}.get(f, field_tol)
        out[f] = max(base, factor * float(e[q]))
    return out


def compare(ref, t, agg, smp, sc, bar):
    """Digest differences of step t against the oracle trajectory, in units of
    the field tests (max|x - oracle| / max|oracle|), and the first quantity
    above its bar (None if all are within).

    Each digest difference is a lower bound of the field's max-norm relative
    error: for N values and m = max|oracle|, |sum x - sum y|, |sum|x| - sum|y||
    and the weighted-sum difference are at most N m e, the sum of squares
    differs by at most 2 N m^2 e, max|.| and the sampled values by m e.  So a
    field within its bar e never fails here.  The liquid volume and tau are
    compared relatively; the adaptive sweep counts, tswap and the V-cycle
    count of the tolerance mode must be equal.  bar maps p, u, v, w, cc,
    volume, tau to their bars (see :func:`bars`)."""
    ra, rs = ref["agg"][t - 1], ref["sc"][t - 1]
    n = float(int(ref["n"][0]) + 2) ** 3
    errs = {}
    bad = None
    for q, f in enumerate(DIGEST_FIELDS):
        mx = ra[q, 3] if ra[q, 3] > 0 else 1.0
        scales = [n * mx, n * mx, 2.0 * n * mx * mx, mx, n * mx]
        for k, name in enumerate(AGGREGATES):
            e = abs(agg[q, k] - ra[q, k]) / scales[k]
            errs["%s.%s" % (f, name)] = e
            if e > bar[f] and bad is None:
                bad = ("%s.%s" % (f, name), e, bar[f])
    if smp is not None:
        i = list(ref["smp_steps"]).index(t)
        for q, f in enumerate(DIGEST_FIELDS):
            mx = ra[q, 3] if ra[q, 3] > 0 else 1.0
            e = float(np.max(np.abs(smp[q] - ref["smp"][i, q]))) / mx
            errs["%s.samples" % f] = e
            if e > bar[f] and bad is None:
                bad = ("%s.samples" % f, e, bar[f])
    for k, f in ((1, "volume"), (0, "tau")):
        e = abs(sc[k] - rs[k]) / abs(rs[k])
        errs[f] = e
        if e > bar[f] and bad is None:
            bad = (f, e, bar[f])
    exact = (2, 3, 4, 5, 6) if int(ref["mode"][0]) != 0 else (2, 3, 4, 5)
    for k in exact:
        if sc[k] != rs[k] and bad is None:
            bad = (SCALARS[k], sc[k], rs[k])
    return errs, bad


def main(names):
    allc = cases()
    for name in names or list(allc) + [n + "_env" for n in allc]:
        if name.endswith("_env"):
            generate_envelope(name[:-4], allc[name[:-4]])
        else:
            generate(name, allc[name])
        print("wrote", name + ".npz", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
