"""CPU-side checks of the C ABI library and the host mirror (no GPU calls).

* libdsg.so loads and exports every function include/dsg.h declares, and the
  ctypes mirror binds each of them;
* without a GPU, entry points fail with a status code, never abort;
* the inputdata.in parser reads the reference's positional format.
"""
import os
import re

import pytest

from conftest import ROOT, pkg


def header_functions():
    text = open(os.path.join(ROOT, "include", "dsg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dsg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_header_symbols():
    dsg = pkg()
    dsg.build.build()
    lib = dsg.load()
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_mirror_covers_header():
    dsg = pkg()
    bound = {n for n, _, _ in dsg._lib.SIGNATURES}
    assert set(header_functions()) <= bound, set(header_functions()) - bound


def test_struct_layouts_match_header():
    """Field order of the ctypes structs equals the C structs in dsg.h."""
    dsg = pkg()
    text = open(os.path.join(ROOT, "include", "dsg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for cname, pyst in (("dsg_config", dsg._lib.DsgConfig), ("dsg_scalars", dsg._lib.DsgScalars),
                        ("dsg_mg_stats", dsg._lib.DsgMgStats), ("dsg_profile", dsg._lib.DsgProfile)):
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (cname, cname), text, re.S).group(1)
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            parts = decl.split(None, 1)
            fields += [f.strip().split("[")[0] for f in parts[1].split(",")]
        assert fields == [n for n, _ in pyst._fields_], cname


def test_no_gpu_returns_status():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; this checks the no-GPU error path")
    dsg = pkg()
    with pytest.raises(dsg.DsgError) as e:
        dsg.Solver(dsg.config.droplet(16))
    assert e.value.code in (-2, -3)


def test_inputdata_roundtrip():
    dsg = pkg()
    inp = dsg.config.droplet(64, impact_speed=2.5)
    text = dsg.format_inputdata(inp)
    back = dsg.parse_inputdata(text)
    for name in ("nx", "ny", "nz", "npre", "ntop", "npost", "omega", "yvel1_si", "rho1_si", "rho2_si",
                 "sigma_si", "length_si", "radius_si", "y0_si", "z0_si", "surfacet"):
        assert getattr(back, name) == getattr(inp, name), name


def test_inputdata_positional_order():
    """NPRE, NTOP, NPOST come in that order in the file (main.f:195-197)."""
    dsg = pkg()
    lines = ["66 nx", "34 ny", "34 nz", "400 tmax", "0 nfilter", "2 cycles", "1.5 OMEGA", "5 NPRE",
             "3 NTOP", "7 NPOST", "0 restart", "0.1 maxcfl", "0 iturb", "2 convectype", "1 hswitch",
             "0.0", "0.0", "0.0", "0.5", "0.0", "0.0", "500. rho2", "1000.0 rho1", "0.0728 sigma",
             "0.001", "0.001", "0.0", "0.0", "2 icase", "2 ibc", "0.008", "0.001", "-0.00017365",
             "1000", "5", "50", "10000", "5 surfacet"]
    inp = dsg.parse_inputdata("\n".join(lines))
    assert (inp.npre, inp.ntop, inp.npost) == (5, 3, 7)
    assert (inp.nx, inp.ny, inp.nz) == (66, 34, 34)
    assert inp.rho2_si == 500.0 and inp.sigma_si == 0.0728 and inp.surfacet == 5
    assert inp.y0_si == -0.00017365


def test_fortran_binding_matches_config():
    """The ISO_C_BINDING type of include/dsg_binding.f90 lists dsg_config's
    fields in the C order with matching kinds, so a Fortran host that uses
    it passes its values where the library reads them."""
    text = open(os.path.join(ROOT, "include", "dsg_binding.f90")).read()
    block = re.search(r"type, bind\(C\) :: dsg_config\n(.*?)\n\s*end type", text, re.S).group(1)
    fortran = []
    for line in block.splitlines():
        kind, names = line.split("::")
        k = re.search(r"\((c_\w+)\)", kind).group(1)
        fortran += [(n.strip(), k) for n in names.split(",")]
    dsg = pkg()
    import ctypes as C
    kinds = {C.c_int: "c_int", C.c_double: "c_double", C.c_uint64: "c_int64_t"}
    want = [(n, kinds[t]) for n, t in dsg._lib.DsgConfig._fields_]
    assert fortran == want


def test_fortran_interfaces_name_declared_entry_points():
    """Every bind(C) interface of include/dsg_binding.f90 names a function
    that dsg.h declares, with the same number of arguments."""
    f90 = open(os.path.join(ROOT, "include", "dsg_binding.f90")).read()
    hdr = open(os.path.join(ROOT, "include", "dsg.h")).read()
    decls = re.findall(r"(?:function|subroutine)\s+(\w+)\(([^)]*)\)\s*(?:&\s*\n\s*([^)]*)\))?\s*bind\(C, name='(\w+)'\)",
                       f90)
    assert len(decls) >= 10
    for fname, args, more, cname in decls:
        assert fname == cname
        nargs = len([a for a in (args + ("," + more if more else "")).split(",") if a.strip()])
        m = re.search(r"\b%s\(([^;]*)\);" % cname, hdr, re.S)
        assert m, cname
        assert len([a for a in m.group(1).split(",") if a.strip()]) == nargs, cname
