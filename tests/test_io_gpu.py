"""Snapshots and the reference's output files: Tecplot main####.plt, the
pressure slice, the savedata/iniget restart pair and printout's schedule."""
import re
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E15 = r" [ -]0\.\d{7}E[+-]\d\d"  # E15.7: a blank of width, then [-]0.dddddddE+ee


def _solver(dsg, n=16, **kw):
    s = dsg.Solver(dsg.config.droplet(n, mode=dsg.config.MODE_TOL_FP64, tol=1e-9, impact_speed=2.0).replace(**kw))
    for t in range(1, 4):
        s.step(t)
    return s


def test_snapshot_overlaps_the_next_step(gpu_lib):
    dsg = gpu_lib
    s = _solver(dsg)
    want = {f: s.field(f) for f in ("p", "u", "v", "w", "cc")}
    s.snapshot(3)
    s.step(4)  # runs while the copy is in flight; the snapshot keeps step 3
    assert s.snapshot_wait() == 3
    for f, a in want.items():
        assert np.array_equal(s.snapshot_field(f), a), f
    with pytest.raises(dsg.DsgError):
        s.snapshot_field("rhs")


def _rows(path, ncol):
    lines = open(path).read().splitlines()
    rows = lines[2:]
    assert all(re.fullmatch(("( %s)" % E15) * ncol, r) for r in rows[:50]), rows[:2]
    return lines[:2], np.array([[float(x) for x in r.split()] for r in rows])


def test_tecplot_file(gpu_lib, tmp_path):
    dsg = gpu_lib
    s = _solver(dsg)
    nx, ny, nz = s.shape
    s.snapshot(3)
    path = tmp_path / "main.plt"
    s.write_tecplot(path)
    head, a = _rows(path, 7)
    assert head[0] == ' VARIABLES="X","Y","Z","U","V","W","CC"'
    assert head[1] == " zone i=%12d j=%12d k=%12d" % (nx, ny - 1, nz)
    assert a.shape == (nx * (ny - 1) * nz, 7)
    u, v, w, cc = (s.field(f) for f in ("u", "v", "w", "cc"))
    sc = s.scalars()
    un = np.concatenate([0.5 * (u[:-1] + u[1:]), u[-1:]], axis=0)
    vn = np.concatenate([0.5 * (v[:, :-1] + v[:, 1:]), v[:, -1:]], axis=1)
    wn = np.concatenate([0.5 * (w[:, :, :-1] + w[:, :, 1:]), w[:, :, -1:]], axis=2)
    sl = (slice(None), slice(1, None), slice(None))  # j = 2..ny
    exp = [f[sl].transpose(2, 1, 0).reshape(-1) for f in (un, vn, wn, cc)]
    for col, e in zip(range(3, 7), exp):
        assert np.allclose(a[:, col], e, rtol=6e-7, atol=1e-300), col
    i = np.arange(1, nx + 1)
    assert np.allclose(a[:nx, 0], i * sc.h * sc.lengthscale * 1000, rtol=6e-7)


def test_pressure_slice(gpu_lib, tmp_path):
    dsg = gpu_lib
    s = _solver(dsg)
    nx, ny, nz = s.shape
    path = tmp_path / "pressure.plt"
    s.snapshot(3)
    s.write_pressure_slice(path)
    head, a = _rows(path, 3)
    assert head == [' VARIABLES="x","y","p"', " zone i=%12dj=%12d" % (nx - 2, ny - 2)]
    sc = s.scalars()
    k = (nz - 2) // 2
    p = s.field("p")[1:-1, 1:-1, k - 1].T.reshape(-1) / (sc.tauh * sc.tauh) * s.inp.rho1_si
    assert np.allclose(a[:, 2], p, rtol=6e-7, atol=1e-30)


def test_restart_pair(gpu_lib, tmp_path):
    dsg = gpu_lib
    s = _solver(dsg, n=16, iturb=0)
    s.snapshot(3)
    path = tmp_path / "save.dat"
    s.savedata(path, 3)
    # gfortran sequential records: 4-byte length, payload, 4-byte length
    raw = path.read_bytes()
    n0, = struct.unpack_from("<i", raw, 0)
    assert n0 == 4 and struct.unpack_from("<i", raw, 4)[0] == 3
    nx, ny, nz = s.shape
    assert len(raw) == 19 * 12 + 17 * 16 + nx * ny * nz * 40  # 19 INTEGER, 17 DOUBLE records
    body = np.frombuffer(raw, dtype=np.uint8)[19 * 12 + 17 * 16:].reshape(-1, 40)
    assert (body[:, :4].view("<i4") == 32).all() and (body[:, 36:].view("<i4") == 32).all()
    vals = body[:, 4:36].copy().view("<f8").reshape(-1, 4)
    for c, f in enumerate(("u", "v", "w", "cc")):
        assert np.array_equal(vals[:, c], s.field(f).reshape(-1, order="F")), f
    # iniget loads them and applies bc_c, bc_v, calcrho as the reference's
    # restart does (main.f:174-177); the interior is the saved state
    r = dsg.Solver(s.inp, init=False)
    assert r.iniget(path) == 3
    inner = (slice(2, -2),) * 3
    for f in ("u", "v", "w", "cc", "rhon", "mun"):
        assert np.array_equal(r.field(f)[inner], s.field(f)[inner]), f
    other = dsg.Solver(dsg.config.droplet(32), init=False)
    with pytest.raises(dsg.DsgError):
        other.iniget(path)


def test_printout_schedule(gpu_lib, tmp_path):
    dsg = gpu_lib
    s = dsg.Solver(dsg.config.droplet(16).replace(ntecplot=2, tsave=4))
    for t in range(1, 5):
        s.step(t)
        s.printout(t, tmp_path)
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["main0001.plt", "main0002.plt", "save.dat"]
