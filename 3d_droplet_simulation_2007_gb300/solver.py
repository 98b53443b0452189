"""Host-side mirror of the reference driver over the C ABI.

:class:`Solver` owns one ``dsg_ctx`` (all fields resident in HBM) and exposes
the routines of main.f's time loop under their reference names:
``vofmethod`` (main.f:795), ``checktime`` (2152), ``csf`` (2363),
``solvelpres`` (3236), ``mglin`` (3645) and ``step`` (the loop body 19-73).
Errors surface as :class:`DsgError` carrying the C status code, the way the
reference ``STOP``s.  Fields move to the host only on request
(:meth:`field`), like the reference's print/dump steps.
"""
import ctypes as C

import numpy as np

from . import _lib
from .config import InputData

FIELDS = _lib.FIELDS


def to_config(inp):
    """DsgConfig from an InputData (or a dict of the same names)."""
    d = inp.as_dict() if isinstance(inp, InputData) else dict(inp)
    cfg = _lib.DsgConfig()
    for name, _ in _lib.DsgConfig._fields_:
        if name in d and d[name] is not None:
            setattr(cfg, name, d[name])
    return cfg


class Solver:
    """One droplet simulation resident on the current CUDA device."""

    def __init__(self, inp, init=True, ctx=None):
        """ctx: wrap an existing context (an ensemble member) without owning it."""
        self.lib = _lib.load()
        self.inp = inp if isinstance(inp, InputData) else InputData(**inp)
        self._cfg = to_config(self.inp)
        self._owned = ctx is None
        if ctx is None:
            h = C.c_void_p()
            _lib.check(self.lib.dsg_create(C.byref(self._cfg), C.byref(h)))
            ctx = h
        self.ctx = ctx if isinstance(ctx, C.c_void_p) else C.c_void_p(ctx)
        self.shape = (self.inp.nx, self.inp.ny, self.inp.nz)
        self.t = 0
        self.last_stats = None
        if init and self._owned:
            self.init_drop()

    # ---- lifecycle -------------------------------------------------------
    def close(self):
        if getattr(self, "ctx", None):
            if self._owned:
                self.lib.dsg_destroy(self.ctx)
            self.ctx = None

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
        return _lib.check(rc, self.ctx)

    def set_stream(self, stream_handle):
        """Run on an external cudaStream_t (int handle), None = own stream."""
        self._ck(self.lib.dsg_set_stream(self.ctx, stream_handle))

    def synchronize(self):
        self._ck(self.lib.dsg_synchronize(self.ctx))

    @property
    def device_bytes(self):
        return self.lib.dsg_device_bytes(self.ctx)

    # ---- state -----------------------------------------------------------
    def field(self, name):
        """Host copy of a fine field, shape (nx,ny,nz), Fortran order."""
        out = np.empty(self.shape, dtype=np.float64, order="F")
        self._ck(self.lib.dsg_download(self.ctx, _lib.FIELD_ID[name], out.ctypes.data))
        return out

    def set_field(self, name, arr):
        a = np.asfortranarray(arr, dtype=np.float64)
        if a.shape != self.shape:
            raise ValueError("shape %s != %s" % (a.shape, self.shape))
        self._ck(self.lib.dsg_upload(self.ctx, _lib.FIELD_ID[name], a.ctypes.data))

    def upload(self, name, arr):
        """Host->device copy straight from a Fortran-ordered float64 array
        (e.g. pinned memory); no staging copy."""
        if arr.dtype != np.float64 or arr.size != self.shape[0] * self.shape[1] * self.shape[2] or not (
                arr.flags["F_CONTIGUOUS"] or arr.ndim == 1):
            raise ValueError("upload needs a contiguous float64 array of the field size")
        self._ck(self.lib.dsg_upload(self.ctx, _lib.FIELD_ID[name], arr.ctypes.data))

    def download_into(self, name, out):
        """Device->host copy into a caller-owned Fortran-ordered float64 array."""
        if out.dtype != np.float64 or out.size != self.shape[0] * self.shape[1] * self.shape[2] or not (
                out.flags["F_CONTIGUOUS"] or out.ndim == 1):
            raise ValueError("download_into needs a contiguous float64 array of the field size")
        self._ck(self.lib.dsg_download(self.ctx, _lib.FIELD_ID[name], out.ctypes.data))
        return out

    def level_ptr(self, name, level):
        p = C.c_void_p()
        nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
        self._ck(self.lib.dsg_level_ptr(self.ctx, _lib.FIELD_ID[name], level, C.byref(p),
                                        C.byref(nx), C.byref(ny), C.byref(nz)))
        return p.value, (nx.value, ny.value, nz.value)

    def field_ptr(self, name):
        p = C.c_void_p()
        self._ck(self.lib.dsg_field_ptr(self.ctx, _lib.FIELD_ID[name], C.byref(p)))
        return p.value

    def scalars(self):
        s = _lib.DsgScalars()
        self._ck(self.lib.dsg_get_scalars(self.ctx, C.byref(s)))
        return s

    def set_scalars(self, s):
        self._ck(self.lib.dsg_set_scalars(self.ctx, C.byref(s)))

    # ---- routines of the time loop ----------------------------------------
    def init_drop(self):
        self._ck(self.lib.dsg_init_drop(self.ctx))

    def vofmethod(self):
        self._ck(self.lib.dsg_vofmethod(self.ctx))

    def calch3d(self):
        self._ck(self.lib.dsg_calch3d(self.ctx))

    def kepsmodel(self):
        self._ck(self.lib.dsg_kepsmodel(self.ctx))

    def checktime(self):
        self._ck(self.lib.dsg_checktime(self.ctx))

    def csf(self):
        self._ck(self.lib.dsg_csf(self.ctx))

    def mglin(self):
        st = _lib.DsgMgStats()
        self._ck(self.lib.dsg_mglin(self.ctx, C.byref(st)))
        self.last_stats = st.as_dict()
        return self.last_stats

    def solvelpres(self, t):
        st = _lib.DsgMgStats()
        self._ck(self.lib.dsg_solvelpres(self.ctx, t, C.byref(st)))
        self.last_stats = st.as_dict()
        return self.last_stats

    def step(self, t=None):
        """One body of the main.f time loop; returns the pressure-solve stats."""
        if t is None:
            t = self.t + 1
        st = _lib.DsgMgStats()
        self._ck(self.lib.dsg_step(self.ctx, t, C.byref(st)))
        self.t = t
        self.last_stats = st.as_dict()
        return self.last_stats

    def step_host(self, inputs, outputs, t=None):
        """dsg_step with the state exchanged through host arrays: `inputs` and
        `outputs` map field names to contiguous float64 arrays of the field
        size (page-locked for asynchronous copies).  The inputs are copied in
        and the outputs out on a second stream, overlapped with the step."""
        if t is None:
            t = self.t + 1
        n = self.shape[0] * self.shape[1] * self.shape[2]

        def check(arr):
            if arr.dtype != np.float64 or arr.size != n or not (arr.flags["F_CONTIGUOUS"] or arr.ndim == 1):
                raise ValueError("step_host needs contiguous float64 arrays of the field size")
            return arr.ctypes.data

        ins, outs = list(inputs.items()), list(outputs.items())
        fi = (C.c_int * max(1, len(ins)))(*[_lib.FIELD_ID[k] for k, _ in ins])
        pi = (C.c_void_p * max(1, len(ins)))(*[check(a) for _, a in ins])
        fo = (C.c_int * max(1, len(outs)))(*[_lib.FIELD_ID[k] for k, _ in outs])
        po = (C.c_void_p * max(1, len(outs)))(*[check(a) for _, a in outs])
        st = _lib.DsgMgStats()
        self._ck(self.lib.dsg_step_host(self.ctx, t, C.byref(st), len(ins), fi, pi, len(outs), fo, po))
        self.t = t
        self.last_stats = st.as_dict()
        return self.last_stats

    def run(self, steps):
        for _ in range(steps):
            self.step()
        return self.last_stats

    # ---- snapshots and output files (printout, main.f:5020-5104) ------------
    def snapshot(self, t=None):
        """Stage p, u, v, w, cc now; the host copy overlaps the next steps."""
        self._ck(self.lib.dsg_snapshot(self.ctx, self.t if t is None else t))

    def snapshot_wait(self):
        t = C.c_int()
        self._ck(self.lib.dsg_snapshot_wait(self.ctx, C.byref(t)))
        return t.value

    def snapshot_field(self, name):
        out = np.empty(self.shape, dtype=np.float64, order="F")
        self._ck(self.lib.dsg_snapshot_field(self.ctx, _lib.FIELD_ID[name], out.ctypes.data))
        return out

    def write_tecplot(self, path):
        self._ck(self.lib.dsg_write_tecplot(self.ctx, str(path).encode()))

    def write_pressure_slice(self, path):
        self._ck(self.lib.dsg_write_pressure_slice(self.ctx, str(path).encode()))

    def savedata(self, path, t0=None):
        self._ck(self.lib.dsg_savedata(self.ctx, str(path).encode(), self.t if t0 is None else t0))

    def iniget(self, path):
        """Load a restart file; returns its step index t0."""
        t0 = C.c_int()
        self._ck(self.lib.dsg_iniget(self.ctx, str(path).encode(), C.byref(t0)))
        self.t = t0.value
        return t0.value

    def printout(self, t, directory=None):
        self._ck(self.lib.dsg_printout(self.ctx, t, None if directory is None else str(directory).encode()))

    # ---- instrumentation ------------------------------------------------------
    def profile_enable(self, on=True):
        self._ck(self.lib.dsg_profile_enable(self.ctx, 1 if on else 0))

    def profile_read(self):
        p = _lib.DsgProfile()
        self._ck(self.lib.dsg_profile_read(self.ctx, C.byref(p)))
        return p.as_dict()

    # ---- reductions ---------------------------------------------------------
    def liquid_volume(self):
        out = C.c_double()
        self._ck(self.lib.dsg_liquid_volume(self.ctx, C.byref(out)))
        return out.value

    def max_divergence(self):
        out = C.c_double()
        self._ck(self.lib.dsg_max_divergence(self.ctx, C.byref(out)))
        return out.value

    def relres(self):
        out = C.c_double()
        self._ck(self.lib.dsg_relres(self.ctx, C.byref(out)))
        return out.value
