"""ctypes binding of ``libdsg.so`` (declarations in include/dsg.h).

The library is the product: there is no Python or CPU fallback.  Importing
this module does not need a GPU, but loading fails loudly if the library has
not been built (``build.build()`` or ``__graft_entry__.build()``).
"""
import ctypes as C
import os

from . import build as _build

DSG_OK = 0
DSG_E_ARG = -1
DSG_E_CUDA = -2
DSG_E_NOMEM = -3
DSG_E_NOT_CONVERGED = -4
DSG_E_NONFINITE = -5
DSG_E_STATE = -6
NET_INPUTS = 5  # DSG_NET_INPUTS

ERROR_NAMES = {0: "DSG_OK", -1: "DSG_E_ARG", -2: "DSG_E_CUDA", -3: "DSG_E_NOMEM",
               -4: "DSG_E_NOT_CONVERGED", -5: "DSG_E_NONFINITE", -6: "DSG_E_STATE"}

FIELDS = ["cc", "p", "res", "rhs", "a", "b", "c", "ei", "u", "v", "w",
          "s11", "s22", "s33", "s12", "s13", "s23", "rhon", "mun", "pprev", "pprev2",
          "ktur", "eps", "mut", "hxmin", "hxmax", "hymin", "hymax", "hzmin", "hzmax"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}


class DsgConfig(C.Structure):
    """struct dsg_config: inputdata.in order (main.f:188-234), then additions."""
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
        ("inner_vcycles", C.c_int), ("use_graphs", C.c_int), ("tail_nodes", C.c_int),
        ("warm_start", C.c_int), ("mg32_omega", C.c_double), ("mg32_npre", C.c_int), ("mg32_npost", C.c_int),
        ("mg32_prolong", C.c_int), ("mg32_fmg_cycles", C.c_int), ("mg32_fine_npre", C.c_int),
        ("mg32_fine_npost", C.c_int), ("mg32_mid_npre", C.c_int), ("mg32_mid_npost", C.c_int),
        ("mg32_small_npre", C.c_int), ("mg32_small_npost", C.c_int), ("fp64_exact", C.c_int),
        ("mg32_krylov", C.c_int), ("mg32_fmg_fine_cycles", C.c_int),
    ]


class DsgScalars(C.Structure):
    """struct dsg_scalars."""
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


class DsgProfile(C.Structure):
    """struct dsg_profile."""
    _fields_ = [("launches", C.c_int64), ("relax_calls", C.c_int64), ("relax_ms", C.c_double),
                ("relax_bytes", C.c_double), ("relax_bits", C.c_int), ("phase_ms", C.c_double * 6)]

    PHASES = ("vof", "cfl", "csf", "momentum", "pressure", "projection")

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "phase_ms"}
        d["phase_ms"] = dict(zip(self.PHASES, list(self.phase_ms)))
        return d


class DsgMgStats(C.Structure):
    """struct dsg_mg_stats."""
    _fields_ = [("mode", C.c_int), ("vcycles", C.c_int), ("fine_sweeps", C.c_int),
                ("relres_init", C.c_double), ("relres", C.c_double), ("converged", C.c_int),
                ("fallback", C.c_int), ("epsdiv", C.c_double), ("relres_base", C.c_double),
                ("relres_net", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


# (name, restype, argtypes) of every exported symbol of include/dsg.h
_vp, _dp, _i, _d = C.c_void_p, C.c_void_p, C.c_int, C.c_double
_PP = C.POINTER(C.c_void_p)
_IP = C.POINTER(C.c_int)
_DPP = C.POINTER(C.c_double)
SIGNATURES = [
    ("dsg_create", _i, [C.POINTER(DsgConfig), _PP]),
    ("dsg_destroy", None, [_vp]),
    ("dsg_last_error", C.c_char_p, [_vp]),
    ("dsg_set_stream", _i, [_vp, _vp]),
    ("dsg_synchronize", _i, [_vp]),
    ("dsg_device_bytes", C.c_int64, [_vp]),
    ("dsg_upload", _i, [_vp, _i, _vp]),
    ("dsg_download", _i, [_vp, _i, _vp]),
    ("dsg_level_ptr", _i, [_vp, _i, _i, _PP, _IP, _IP, _IP]),
    ("dsg_field_ptr", _i, [_vp, _i, _PP]),
    ("dsg_get_scalars", _i, [_vp, C.POINTER(DsgScalars)]),
    ("dsg_set_scalars", _i, [_vp, C.POINTER(DsgScalars)]),
    ("dsg_init_drop", _i, [_vp]),
    ("dsg_vofmethod", _i, [_vp]),
    ("dsg_kepsmodel", _i, [_vp]),
    ("dsg_calch3d", _i, [_vp]),
    ("dsg_checktime", _i, [_vp]),
    ("dsg_csf", _i, [_vp]),
    ("dsg_solvelpres", _i, [_vp, _i, C.POINTER(DsgMgStats)]),
    ("dsg_mglin", _i, [_vp, C.POINTER(DsgMgStats)]),
    ("dsg_step", _i, [_vp, _i, C.POINTER(DsgMgStats)]),
    ("dsg_step_host", _i, [_vp, _i, C.POINTER(DsgMgStats), _i, _IP, C.POINTER(_vp), _i, _IP, C.POINTER(_vp)]),
    ("dsg_liquid_volume", _i, [_vp, _DPP]),
    ("dsg_max_divergence", _i, [_vp, _DPP]),
    ("dsg_relres", _i, [_vp, _DPP]),
    ("dsg_profile_enable", _i, [_vp, _i]),
    ("dsg_profile_read", _i, [_vp, _vp]),
    ("dsg_launch_count", C.c_int64, []),
    ("dsg_relax", _i, [_dp, _d, _dp, _dp, _dp, _dp, _dp, _i, _i, _i, _d, _vp]),
    ("dsg_resid", _i, [_d, _dp, _dp, _dp, _dp, _dp, _dp, _i, _i, _i, _vp]),
    ("dsg_rstrct", _i, [_dp, _dp, _i, _i, _i, _vp]),
    ("dsg_interp", _i, [_dp, _dp, _i, _i, _i, _vp]),
    ("dsg_addint", _i, [_dp, _dp, _dp, _i, _i, _i, _vp]),
    ("dsg_acfromac", _i, [_dp] * 7 + [_i, _i, _i, _vp]),
    ("dsg_abcei", _i, [_dp] * 5 + [_d, _d, _i, _i, _i, _vp]),
    ("dsg_bc_scalar", _i, [_dp, _i, _i, _i, _vp]),
    ("dsg_bc_resid", _i, [_dp, _i, _i, _i, _vp]),
    ("dsg_bc_out", _i, [_dp, _i, _i, _i, _vp]),
    ("dsg_filterc27", _i, [_dp, _dp, _i, _i, _i, _vp]),
    ("dsg_mglin_noalloc", _i, [_dp] * 6 + [_i] * 7 + [_d] * 3 + [_vp]),
    ("dsg_net_param_count", C.c_int64, []),
    ("dsg_net_create", _i, [_i, _i, _i, C.c_uint64, _PP]),
    ("dsg_net_destroy", None, [_vp]),
    ("dsg_net_device_bytes", C.c_int64, [_vp]),
    ("dsg_net_get_params", _i, [_vp, _vp, C.c_int64]),
    ("dsg_net_set_params", _i, [_vp, _vp, C.c_int64]),
    ("dsg_net_forward_host", _i, [_vp, _vp, _vp]),
    ("dsg_net_grad_host", _i, [_vp, _vp, _vp, C.POINTER(C.c_float), _vp]),
    ("dsg_net_train_step", _i, [_vp, C.c_float, C.POINTER(C.c_float)]),
    ("dsg_attach_net", _i, [_vp, _vp, _i]),
    ("dsg_snapshot", _i, [_vp, _i]),
    ("dsg_snapshot_wait", _i, [_vp, _IP]),
    ("dsg_snapshot_field", _i, [_vp, _i, _vp]),
    ("dsg_write_tecplot", _i, [_vp, C.c_char_p]),
    ("dsg_write_pressure_slice", _i, [_vp, C.c_char_p]),
    ("dsg_savedata", _i, [_vp, C.c_char_p, _i]),
    ("dsg_iniget", _i, [_vp, C.c_char_p, _IP]),
    ("dsg_printout", _i, [_vp, _i, C.c_char_p]),
    ("dsg_ensemble_create", _i, [C.POINTER(DsgConfig), _i, _i, _PP]),
    ("dsg_ensemble_destroy", None, [_vp]),
    ("dsg_ensemble_size", _i, [_vp]),
    ("dsg_ensemble_workers", _i, [_vp]),
    ("dsg_ensemble_member", _vp, [_vp, _i]),
    ("dsg_ensemble_last_error", C.c_char_p, [_vp]),
    ("dsg_ensemble_set_workers", _i, [_vp, _i]),
    ("dsg_ensemble_step", _i, [_vp, _i, C.POINTER(DsgMgStats)]),
    ("dsg_ensemble_last_ms", _d, [_vp]),
    ("dsg_ensemble_member_ms", _i, [_vp, _DPP]),
    ("dsg_ensemble_set_batched", _i, [_vp, _i]),
    ("dsg_ensemble_batched", _i, [_vp]),
    ("dsg_ensemble_phase_ms", _i, [_vp, _DPP]),
    ("dsg_ensemble_autotune_tiles", _i, [_vp, _i, C.POINTER(_i)]),
    ("dsg_ensemble_batch_tail_nodes", C.c_int64, [_vp]),
    ("dsg_ensemble_autotune", _i, [_vp, _i, _i, _IP, _IP]),
    ("dsg_ensemble_plan", _i, [_DPP, _i, _i, _IP]),
]

_LIB = None


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load libdsg.so.  Raises if it is missing (no fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError("libdsg.so is not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class DsgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERROR_NAMES.get(code, "?"), code, msg))
        self.code = code


def check(rc, ctx=None):
    if rc != DSG_OK:
        lib = load()
        msg = lib.dsg_last_error(ctx)
        raise DsgError(rc, msg.decode() if msg else "")
    return rc
