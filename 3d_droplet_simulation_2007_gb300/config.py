"""Run configuration: the reference's ``inputdata.in`` interface plus additions.

``readinput`` (main.f:185-272) reads 38 positional, list-directed values, one
per line, in a fixed order.  :class:`InputData` keeps that order and the same
names; :func:`parse_inputdata` / :func:`format_inputdata` read and write the
file format (first token of each line, the rest is a comment).  Note the
reference line order NPRE, NTOP, NPOST (main.f:195-197).

The additions that have no reference counterpart (solver mode, residual
tolerance, velocity noise) sit after the 38 values and are not written to the
file.
"""
from dataclasses import dataclass, fields, asdict
import math

MODE_REF_EXACT = 0   # mglin exactly: FMG with a fixed number of V-cycles
MODE_TOL_FP64 = 1    # FMG, then FP64 V-cycles until the relative residual < tol
MODE_TOL_MIXED = 2   # FP64 defect correction around FP32 V-cycles, to tol
MODE_LEARNED = 3     # MODE_TOL_MIXED with the learned initial guess (guarded)

MODE_NAMES = {"ref_exact": MODE_REF_EXACT, "tol_fp64": MODE_TOL_FP64,
              "tol_mixed": MODE_TOL_MIXED, "learned": MODE_LEARNED}

# inputdata.in order (main.f:188-234)
_FILE_ORDER = [
    ("nx", int), ("ny", int), ("nz", int), ("tmax", int), ("nfilter", int),
    ("cycles", int), ("omega", float), ("npre", int), ("ntop", int), ("npost", int),
    ("restart", int), ("maxcfl", float), ("iturb", int), ("convectype", int),
    ("hswitch", int), ("xvel1_si", float), ("yvel1_si", float), ("zvel1_si", float),
    ("xvel2_si", float), ("yvel2_si", float), ("zvel2_si", float), ("rho2_si", float),
    ("rho1_si", float), ("sigma_si", float), ("visc2_si", float), ("visc1_si", float),
    ("grav_si", float), ("grav1_si", float), ("icase", int), ("ibc", int),
    ("length_si", float), ("radius_si", float), ("y0_si", float), ("z0_si", float),
    ("tprint", int), ("ntecplot", int), ("tsave", int), ("surfacet", int),
]


@dataclass
class InputData:
    nx: int = 66
    ny: int = 66
    nz: int = 66
    tmax: int = 200
    nfilter: int = 0
    cycles: int = 2
    omega: float = 1.5
    npre: int = 5
    ntop: int = 4
    npost: int = 5
    restart: int = 0
    maxcfl: float = 0.1
    iturb: int = 0
    convectype: int = 2
    hswitch: int = 0
    xvel1_si: float = 0.0
    yvel1_si: float = -1.0
    zvel1_si: float = 0.0
    xvel2_si: float = 0.0
    yvel2_si: float = 0.0
    zvel2_si: float = 0.0
    rho2_si: float = 1.2
    rho1_si: float = 1000.0
    sigma_si: float = 0.072
    visc2_si: float = 1.8e-5
    visc1_si: float = 1.0e-3
    grav_si: float = -9.81
    grav1_si: float = 0.0
    icase: int = 2
    ibc: int = 2
    length_si: float = 0.008
    radius_si: float = 0.001
    y0_si: float = 1.2e-3
    z0_si: float = 1000.0
    tprint: int = 5
    ntecplot: int = 50
    tsave: int = 1000000
    surfacet: int = 2
    # additions (no reference counterpart)
    mode: int = MODE_REF_EXACT
    tol: float = 1e-8
    max_vcycles: int = 200
    noise_si: float = 0.0
    noise_seed: int = 0
    inner_vcycles: int = 0
    use_graphs: int = 1
    tail_nodes: int = 0
    warm_start: int = 0
    # FP32 V-cycles of the mixed modes (the FP64 defect correction's inner
    # solver): trilinear prolongation (0; 1 = the reference's injection),
    # relaxation factor 1.5, 3 pre-/post-sweeps on the finest level and 8 on
    # the coarser ones (mg32_fine_npre/npost below).  Fastest in sweeps on the
    # 256^3 splash: 4 V-cycles and 17.2 ms per step, against 5 V-cycles and
    # 18.8 ms with V(5,5) on every level at omega 1.6, and 8-9 V-cycles and
    # 22.5 ms with injection, V(4,4), omega 1.4.
    mg32_omega: float = 1.5
    mg32_npre: int = 8
    mg32_npost: int = 8
    mg32_prolong: int = 0
    # V-cycles per level of the FP32 FMG start (0: cycles) below the finest
    # level, and on the finest level (mg32_fmg_fine_cycles below).  One below
    # and two on the finest: 14.63 ms per 256^3 step with 4 V-cycles after the
    # start, against 15.69 ms with two everywhere (three below and two on the
    # finest: 16.76 ms; two below and one on the finest: 6-7 V-cycles,
    # 18.38 ms).
    mg32_fmg_cycles: int = 1
    # sweeps of the FP32 V-cycles on the finest level (0: mg32_npre/mg32_npost)
    mg32_fine_npre: int = 3
    mg32_fine_npost: int = 3
    # sweeps on the level below the finest (0: mg32_npre/mg32_npost)
    mg32_mid_npre: int = 0
    mg32_mid_npost: int = 0
    # sweeps on the levels of at most 18^3 nodes (0: mg32_npre/mg32_npost)
    mg32_small_npre: int = 0
    mg32_small_npost: int = 0
    # tolerance mode: 0 = FP64 multigrid in fused multiply-add form (within
    # ulps of the oracle), 1 = the reference's exact operation order
    fp64_exact: int = 0
    # mixed modes: 1 = each FP32 V-cycle preconditions one GCR step (one
    # previous direction kept), 0 = the V-cycles iterate on one correction
    mg32_krylov: int = 0
    # V-cycles of the FP32 FMG start on the finest level (0: mg32_fmg_cycles)
    mg32_fmg_fine_cycles: int = 2

    def as_dict(self):
        return asdict(self)

    def replace(self, **kw):
        d = self.as_dict()
        d.update(kw)
        return InputData(**d)


def parse_inputdata(text):
    """Parse the text of an ``inputdata.in`` file (first token of each line)."""
    lines = [ln for ln in text.splitlines() if ln.strip()]
    if len(lines) < len(_FILE_ORDER):
        raise ValueError("inputdata.in: expected %d values, got %d" % (len(_FILE_ORDER), len(lines)))
    kw = {}
    for (name, typ), ln in zip(_FILE_ORDER, lines):
        tok = ln.split()[0].rstrip(",")
        kw[name] = typ(float(tok)) if typ is int else typ(tok.replace("d", "e").replace("D", "e"))
    return InputData(**kw)


def format_inputdata(inp):
    """Text of an ``inputdata.in`` file holding the 38 reference values."""
    out = []
    for name, typ in _FILE_ORDER:
        v = getattr(inp, name)
        out.append(("%d" % v if typ is int else repr(float(v))) + "\t\t\t\t" + name)
    return "\n".join(out) + "\n"


def droplet(n, steps=200, impact_speed=1.0, noise_si=1e-4, mode=MODE_REF_EXACT, tol=1e-10,
            npre=5, npost=5, ntop=4, cycles=2, diameter=2e-3, seed=0):
    """Droplet impacting a flat wall on an n^3-cell grid.

    n = 2^k gives the reference's multigrid hierarchy; other even sides
    (48, 96, 160, ...) coarsen while the interior stays even.

    Cubic domain of 4 droplet diameters, drop centre 0.1 D above the wall
    (y0 = R + 0.1 D), liquid/gas density 1000/1.2, viscosity 1e-3/1.8e-5,
    sigma 0.072, gravity -9.81 along y, CSF surface tension, central
    convection, laminar, maxcfl 0.1, omega 1.5.
    """
    if n < 4:
        raise ValueError("n must be at least 4")
    r = 0.5 * diameter
    return InputData(
        nx=n + 2, ny=n + 2, nz=n + 2, tmax=steps, cycles=cycles, npre=npre, ntop=ntop,
        npost=npost, yvel1_si=-abs(impact_speed), length_si=4.0 * diameter, radius_si=r,
        y0_si=r + 0.1 * diameter, mode=mode, tol=tol, noise_si=noise_si, noise_seed=seed)


# The workloads of the droplet-on-wall study (grid side = interior cells).
def config_small():
    """FP64 plain method, 64^3 interior (66^3 nodes), 200 steps, 1 m/s, noise 1e-4."""
    return droplet(64, steps=200, impact_speed=1.0, noise_si=1e-4, mode=MODE_REF_EXACT)


def config_parity():
    """FP64 plain method, 128^3 interior, 500 steps, 1 m/s."""
    return droplet(128, steps=500, impact_speed=1.0, noise_si=1e-4, mode=MODE_REF_EXACT)


def config_splash(mode=MODE_TOL_FP64, tol=1e-8):
    """Splash on wall, 256^3 interior, 3 m/s, 4 pre/4 post sweeps, residual 1e-8."""
    return droplet(256, steps=1000, impact_speed=3.0, noise_si=1e-4, mode=mode, tol=tol,
                   npre=4, npost=4, ntop=4)


def weber_speed(we, diameter=2e-3, sigma=0.072, rho=1000.0):
    """Impact speed that gives Weber number ``we`` = rho v^2 D / sigma."""
    return math.sqrt(we * sigma / (rho * diameter))


FIELD_NAMES = [f.name for f in fields(InputData)]
