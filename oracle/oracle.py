"""ctypes wrapper of the C oracle (test infrastructure only).

The oracle restates main.f of farzan-t/3D_Droplet_simulation_2007 on the CPU
(see dsg_oracle.c for the routine-by-routine citations).  Parity is unpinned
against the reference itself: no Fortran compiler and no reference fixtures
exist, so the oracle is pinned by analytic known-answer tests instead.
"""
import ctypes as C

import numpy as np

from . import build as _build

FIELDS = ["cc", "p", "res", "rhs", "a", "b", "c", "ei", "u", "v", "w",
          "s11", "s22", "s33", "s12", "s13", "s23", "rhon", "mun"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
FIELD_ID.update({"ktur": 21, "eps": 22, "mut": 23, "hxmin": 24, "hxmax": 25, "hymin": 26, "hymax": 27,
                 "hzmin": 28, "hzmax": 29})

MODE_REF_EXACT = 0
MODE_TOL_FP64 = 1


class OracleInput(C.Structure):
    """Mirror of ``ora_input``: inputdata.in order (main.f:188-234) + additions."""
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("tmax", C.c_int),
        ("nfilter", C.c_int), ("cycles", C.c_int), ("omega", C.c_double),
        ("npre", C.c_int), ("ntop", C.c_int), ("npost", C.c_int), ("restart", C.c_int),
        ("maxcfl", C.c_double), ("iturb", C.c_int), ("convectype", C.c_int),
        ("hswitch", C.c_int),
        ("xvel1_si", C.c_double), ("yvel1_si", C.c_double), ("zvel1_si", C.c_double),
        ("xvel2_si", C.c_double), ("yvel2_si", C.c_double), ("zvel2_si", C.c_double),
        ("rho2_si", C.c_double), ("rho1_si", C.c_double), ("sigma_si", C.c_double),
        ("visc2_si", C.c_double), ("visc1_si", C.c_double), ("grav_si", C.c_double),
        ("grav1_si", C.c_double), ("icase", C.c_int), ("ibc", C.c_int),
        ("length_si", C.c_double), ("radius_si", C.c_double), ("y0_si", C.c_double),
        ("z0_si", C.c_double), ("tprint", C.c_int), ("ntecplot", C.c_int),
        ("tsave", C.c_int), ("surfacet", C.c_int),
        ("mode", C.c_int), ("tol", C.c_double), ("max_vcycles", C.c_int),
        ("noise_si", C.c_double), ("noise_seed", C.c_uint64),
    ]


class OracleScalars(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "tau", "tauh", "time", "h", "rho1", "rho2", "mu1", "mu2", "sigma", "g", "g1",
        "lengthsize", "lengthscale", "vscale", "radius", "y0", "z0",
        "xvel1", "yvel1", "zvel1", "xvel2", "yvel2", "zvel2")] + [
        (n, C.c_int) for n in ("tauh2", "npre", "npost", "ntop", "cycles", "tswap", "ng",
                               "last_vcycles")] + [
        ("last_relres", C.c_double), ("last_relres_fmg", C.c_double),
        ("last_epsdiv", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_LIB = None
_DP = C.POINTER(C.c_double)


def load():
    """Build (if needed) and load the oracle shared library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    lib = C.CDLL(_build.build())
    vp = C.c_void_p
    lib.ora_create.restype = vp
    lib.ora_create.argtypes = [C.POINTER(OracleInput)]
    lib.ora_destroy.argtypes = [vp]
    lib.ora_level_count.argtypes = [C.c_int, C.c_int, C.c_int]
    lib.ora_field.restype = _DP
    lib.ora_field.argtypes = [vp, C.c_int]
    lib.ora_level_field.restype = _DP
    lib.ora_level_field.argtypes = [vp, C.c_int, C.c_int]
    lib.ora_level_dims.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.ora_get_scalars.argtypes = [vp, C.POINTER(OracleScalars)]
    lib.ora_set_scalars.argtypes = [vp, C.POINTER(OracleScalars)]
    lib.ora_calch3d.argtypes = [vp]
    lib.ora_calch3d.restype = C.c_int
    lib.ora_error.argtypes = [vp, C.POINTER(C.c_longlong)]
    lib.ora_error.restype = C.c_int
    for fn in ("ora_vofmethod", "ora_kepsmodel", "ora_checktime", "ora_csf", "ora_sgip", "ora_sgip2", "ora_mglin"):
        getattr(lib, fn).argtypes = [vp]
    lib.ora_solvelpres.argtypes = [vp, C.c_int]
    lib.ora_step.argtypes = [vp, C.c_int]
    lib.ora_relres.restype = C.c_double
    lib.ora_relres.argtypes = [vp]
    for fn in ("ora_nx", "ora_ny", "ora_nz"):
        getattr(lib, fn).argtypes = [vp]
        getattr(lib, fn).restype = C.c_int
    d, i = C.c_double, C.c_int
    lib.ora_relax.argtypes = [_DP, d, _DP, _DP, _DP, _DP, _DP, i, i, i, d]
    lib.ora_resid.argtypes = [d, _DP, _DP, _DP, _DP, _DP, _DP, i, i, i]
    lib.ora_rstrct.argtypes = [_DP, _DP, i, i, i]
    lib.ora_interp.argtypes = [_DP, _DP, i, i, i]
    lib.ora_addint.argtypes = [_DP, _DP, _DP, i, i, i]
    lib.ora_acfromac.argtypes = [_DP] * 7 + [i, i, i]
    lib.ora_abcei.argtypes = [_DP] * 5 + [d, d, i, i, i]
    for fn in ("ora_bc_scalar", "ora_bc_resid", "ora_bc_out"):
        getattr(lib, fn).argtypes = [_DP, i, i, i]
    lib.ora_filterc27.argtypes = [_DP, _DP, i, i, i]
    lib.ora_csf_curvature.argtypes = [_DP, _DP, i, i, i]
    lib.ora_al3d.restype = d
    lib.ora_al3d.argtypes = [d, d, d, d]
    lib.ora_fl3d.restype = d
    lib.ora_fl3d.argtypes = [d] * 6
    lib.ora_swp.argtypes = [vp, _DP, _DP, _DP, _DP, _DP, i]
    lib.ora_sumfield.restype = d
    lib.ora_sumfield.argtypes = [_DP, i, i, i]
    lib.ora_fmodmax.restype = d
    lib.ora_fmodmax.argtypes = [_DP, i, i, i]
    lib.ora_noise_unit.restype = d
    lib.ora_noise_unit.argtypes = [C.c_uint64, C.c_int, C.c_int64]
    _LIB = lib
    return lib


def ptr(a):
    """double* of a C-contiguous float64 numpy array."""
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_DP)


def make_input(cfg):
    """OracleInput from any object/dict carrying the inputdata.in names."""
    get = cfg.get if isinstance(cfg, dict) else (lambda k, d=None: getattr(cfg, k, d))
    oi = OracleInput()
    for name, _ in OracleInput._fields_:
        val = get(name, None)
        if val is not None:
            setattr(oi, name, val)
    return oi


class Oracle:
    """One oracle solver state (arrays are Fortran-ordered numpy views)."""

    def __init__(self, cfg):
        self.lib = load()
        self.inp = make_input(cfg)
        self.h = self.lib.ora_create(C.byref(self.inp))
        if not self.h:
            raise ValueError("oracle: grid needs at least 2 interior cells per side")
        self.shape = (self.lib.ora_nx(self.h), self.lib.ora_ny(self.h), self.lib.ora_nz(self.h))

    def close(self):
        if self.h:
            self.lib.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, name):
        """Writable view of a fine-level field, shape (nx,ny,nz), Fortran order."""
        p = self.lib.ora_field(self.h, FIELD_ID[name])
        n = self.shape[0] * self.shape[1] * self.shape[2]
        flat = np.ctypeslib.as_array(p, shape=(n,))
        return flat.reshape(self.shape, order="F")

    def level_dims(self, level):
        x, y, z = C.c_int(), C.c_int(), C.c_int()
        self.lib.ora_level_dims(self.h, level, C.byref(x), C.byref(y), C.byref(z))
        return (x.value, y.value, z.value)

    def level_field(self, name, level):
        dims = self.level_dims(level)
        p = self.lib.ora_level_field(self.h, FIELD_ID[name], level)
        flat = np.ctypeslib.as_array(p, shape=(dims[0] * dims[1] * dims[2],))
        return flat.reshape(dims, order="F")

    def scalars(self):
        s = OracleScalars()
        self.lib.ora_get_scalars(self.h, C.byref(s))
        return s

    def set_scalars(self, s):
        self.lib.ora_set_scalars(self.h, C.byref(s))

    def step(self, t):
        self.lib.ora_step(self.h, t)

    def vofmethod(self):
        self.lib.ora_vofmethod(self.h)

    def kepsmodel(self):
        self.lib.ora_kepsmodel(self.h)

    def calch3d(self):
        return self.lib.ora_calch3d(self.h)

    def sgip(self):
        self.lib.ora_sgip(self.h)

    def error(self):
        cell = C.c_longlong()
        return self.lib.ora_error(self.h, C.byref(cell)), cell.value

    def checktime(self):
        self.lib.ora_checktime(self.h)

    def csf(self):
        self.lib.ora_csf(self.h)

    def solvelpres(self, t):
        self.lib.ora_solvelpres(self.h, t)

    def mglin(self):
        self.lib.ora_mglin(self.h)

    def relres(self):
        return self.lib.ora_relres(self.h)

    def liquid_volume(self):
        cc = np.asfortranarray(self.field("cc"))
        flat = cc.reshape(-1, order="F")
        return self.lib.ora_sumfield(ptr(np.ascontiguousarray(flat)), *self.shape)


# ---- array-level helpers (arrays are Fortran-ordered 3D float64) ----------

def _flat(a):
    f = a.reshape(-1, order="F")
    if not f.flags["C_CONTIGUOUS"] or f.base is None and f is not a:
        f = np.ascontiguousarray(f)
    return f


class Arr:
    """Holds a Fortran-ordered array and its contiguous flat buffer."""

    def __init__(self, a):
        self.shape = a.shape
        self.flat = np.ascontiguousarray(a.reshape(-1, order="F")).astype(np.float64)

    @property
    def p(self):
        return ptr(self.flat)

    def array(self):
        return self.flat.reshape(self.shape, order="F").copy()


def relax(u, lengthsize, rhs, a, b, c, ei, omega):
    lib = load()
    U, R, A, B, Cc, E = (Arr(x) for x in (u, rhs, a, b, c, ei))
    lib.ora_relax(U.p, lengthsize, R.p, A.p, B.p, Cc.p, E.p, *u.shape, omega)
    return U.array()


def resid(lengthsize, u, rhs, a, b, c, res0=None):
    lib = load()
    res = Arr(res0 if res0 is not None else np.zeros_like(u))
    U, R, A, B, Cc = (Arr(x) for x in (u, rhs, a, b, c))
    lib.ora_resid(lengthsize, res.p, U.p, R.p, A.p, B.p, Cc.p, *u.shape)
    return res.array()


def rstrct(uf, coarse_shape, uc0=None):
    lib = load()
    uc = Arr(uc0 if uc0 is not None else np.zeros(coarse_shape))
    F = Arr(uf)
    lib.ora_rstrct(uc.p, F.p, *coarse_shape)
    return uc.array()


def interp(uc, fine_shape, uf0=None):
    lib = load()
    uf = Arr(uf0 if uf0 is not None else np.zeros(fine_shape))
    Cc = Arr(uc)
    lib.ora_interp(uf.p, Cc.p, *fine_shape)
    return uf.array()


def addint(uf, uc, res0=None):
    lib = load()
    U, Cc = Arr(uf), Arr(uc)
    R = Arr(res0 if res0 is not None else np.zeros_like(uf))
    lib.ora_addint(U.p, Cc.p, R.p, *uf.shape)
    return U.array(), R.array()


def acfromac(a2, b2, c2, coarse_shape, init=None):
    lib = load()
    outs = [Arr(init[q] if init is not None else np.zeros(coarse_shape)) for q in range(4)]
    A2, B2, C2 = Arr(a2), Arr(b2), Arr(c2)
    lib.ora_acfromac(outs[0].p, outs[1].p, outs[2].p, outs[3].p, A2.p, B2.p, C2.p, *coarse_shape)
    return tuple(o.array() for o in outs)


def abcei(cc, r1, r2, init=None):
    lib = load()
    outs = [Arr(init[q] if init is not None else np.zeros_like(cc)) for q in range(4)]
    CC = Arr(cc)
    lib.ora_abcei(outs[0].p, outs[1].p, outs[2].p, outs[3].p, CC.p, r1, r2, *cc.shape)
    return tuple(o.array() for o in outs)


def bc(name, s):
    lib = load()
    S = Arr(s)
    getattr(lib, "ora_" + name)(S.p, *s.shape)
    return S.array()


def filterc27(cc, out0=None):
    lib = load()
    CC = Arr(cc)
    out = Arr(out0 if out0 is not None else np.zeros_like(cc))
    lib.ora_filterc27(CC.p, out.p, *cc.shape)
    return out.array()


def csf_curvature(ccf, out0=None):
    """csf's curvature of a filtered fraction (dsg_oracle.c ora_csf_curvature)."""
    lib = load()
    F = Arr(ccf)
    out = Arr(out0 if out0 is not None else np.zeros_like(ccf))
    lib.ora_csf_curvature(out.p, F.p, *ccf.shape)
    return out.array()


def al3d(b1, b2, b3, cc):
    return load().ora_al3d(b1, b2, b3, cc)


def fl3d(m1, m2, m3, alpha, r0, dr0):
    return load().ora_fl3d(m1, m2, m3, alpha, r0, dr0)


def sumfield(u):
    U = Arr(u)
    return load().ora_sumfield(U.p, *u.shape)


def fmodmax(u):
    U = Arr(u)
    return load().ora_fmodmax(U.p, *u.shape)


def noise_unit(seed, field, lin):
    return load().ora_noise_unit(seed, field, lin)
