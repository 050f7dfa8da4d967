"""The shipped Fortran binding (fortran/mhd_gpu_binding.f90) against the C
header -- no Fortran compiler exists here, so the binding is checked as text:
the bind(C) derived type must lay out exactly like ``mhd_params``, and every
bind(C) interface must name a declared entry point with the same number of
arguments passed the same way (by value / by reference, pointer depth, element
type).  A drifted field or argument would otherwise only show up as corrupted
data in the Fortran driver.
"""
import ctypes
import re
from pathlib import Path

import pytest

from mhd3d_mpi_fortran_gb300.abi import CParams

ROOT = Path(__file__).resolve().parents[1]
HEADER = (ROOT / "include" / "mhd_gpu.h").read_text()
F90 = (ROOT / "mhd3d_mpi_fortran_gb300" / "fortran" / "mhd_gpu_binding.f90").read_text()


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def _f90_lines(s):
    """Fortran source without comments, continuation lines joined."""
    out, cur = [], ""
    for line in s.splitlines():
        line = line.split("!")[0].rstrip()
        if not line.strip():
            continue
        if cur:
            line = cur + " " + line.strip()
            cur = ""
        if line.endswith("&"):
            cur = line[:-1].rstrip()
            continue
        out.append(line.strip())
    return out


def c_struct_fields():
    body = re.search(r"typedef struct mhd_params \{(.*?)\} mhd_params;", _strip_c_comments(HEADER), re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        kind = {"int32_t": "int32", "double": "double"}[ctype]
        for n in names.split(","):
            m = re.fullmatch(r"\s*(\w+)(?:\[(\d+)\])?\s*", n)
            fields.append((m.group(1), kind, int(m.group(2) or 1)))
    return fields


def f90_type_fields():
    lines = _f90_lines(F90)
    start = lines.index("type, bind(C) :: mhd_params")
    fields = []
    for line in lines[start + 1:]:
        if line.startswith("end type"):
            break
        ftype, names = [x.strip() for x in line.split("::")]
        kind = {"integer(c_int32_t)": "int32", "real(c_double)": "double"}[ftype]
        for n in re.findall(r"\w+(?:\(\d+\))?", names):
            m = re.fullmatch(r"(\w+)(?:\((\d+)\))?", n)
            fields.append((m.group(1), kind, int(m.group(2) or 1)))
    return fields


def test_derived_type_matches_the_c_struct():
    assert f90_type_fields() == c_struct_fields()


def test_c_struct_matches_the_ctypes_mirror():
    ct = []
    for name, t in CParams._fields_:
        n = getattr(t, "_length_", 1)
        elem = t._type_ if n > 1 or hasattr(t, "_length_") else t
        assert elem in (ctypes.c_double, ctypes.c_int32), (name, elem)
        ct.append((name, "double" if elem is ctypes.c_double else "int32", n))
    assert ct == c_struct_fields()


def c_prototypes():
    protos = {}
    for m in re.finditer(r"\bint\s+(mhd_\w+)\s*\(([^;]*?)\)\s*;", _strip_c_comments(HEADER), re.S):
        args = [a.strip() for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        protos[m.group(1)] = [_c_arg_class(a) for a in args]
    return protos


def _c_arg_class(arg):
    a = re.sub(r"\bconst\b", "", arg)
    a = re.sub(r"\s+", " ", a).strip()
    base = a.split()[0].rstrip("*")
    depth = a.count("*") + a.count("[")  # an array parameter is passed as a pointer
    elem = {"int32_t": "int32", "uint32_t": "int32", "int": "int32"}.get(base, base)
    return elem + "*" * depth


def f90_interfaces():
    lines = _f90_lines(F90)
    out = {}
    i = 0
    while i < len(lines):
        m = re.match(r"integer\(c_int\) function (\w+)\(([^)]*)\)\s*bind\(C, name=\"(\w+)\"\)", lines[i])
        if not m:
            i += 1
            continue
        fname, args, cname = m.group(1), [a.strip() for a in m.group(2).split(",")], m.group(3)
        decls = {}
        i += 1
        while not lines[i].startswith("end function"):
            if "::" in lines[i] and not lines[i].startswith("import"):
                spec, names = [x.strip() for x in lines[i].split("::")]
                for n in re.findall(r"(\w+)(\(\*\))?", names):
                    decls[n[0]] = (spec, bool(n[1]))
            i += 1
        out[cname] = (fname, [_f90_arg_class(*decls[a]) for a in args])
    return out


def _f90_arg_class(spec, is_array):
    value = "value" in spec
    if spec.startswith("type(c_ptr)"):
        return "void*" if value else "void**"
    if spec.startswith("type(mhd_params)"):
        return "mhd_params*"
    elem = "double" if spec.startswith("real(c_double)") else "int32"
    return elem if (value and not is_array) else elem + "*"


def test_every_interface_names_a_declared_entry_point():
    protos = c_prototypes()
    ifaces = f90_interfaces()
    assert set(ifaces) >= {"mhd_init", "mhd_step", "mhd_step_n", "mhd_fetch", "mhd_free", "mhd_diagnostics"}
    for cname, (fname, _) in ifaces.items():
        assert fname == cname
        assert cname in protos, cname


@pytest.mark.parametrize("name", ["mhd_init", "mhd_step", "mhd_step_n", "mhd_fetch", "mhd_free", "mhd_diagnostics",
                                  "mhd_set_tau"])
def test_interface_arguments_match_the_prototype(name):
    _, fargs = f90_interfaces()[name]
    assert fargs == c_prototypes()[name], (name, fargs, c_prototypes()[name])


def test_step_stop_mask_is_nan_or_negative_density():
    """gpu_step stops on iand(status, 3): MHD_ST_NAN | MHD_ST_NEG_RHO, the
    checks the reference's diagnostics stop on."""
    bits = {m.group(1): int(m.group(2)) for m in re.finditer(r"(MHD_ST_\w+)\s*=\s*1u\s*<<\s*(\d+)", HEADER)}
    mask = int(re.search(r"iand\(status, (\d+)\)", F90).group(1))
    assert mask == (1 << bits["MHD_ST_NAN"]) | (1 << bits["MHD_ST_NEG_RHO"])


def test_step_passes_tau_both_ways():
    """mhd_step's tau is in/out (the driver's module tau, mhd3d3.f90:3285-3286):
    the interface declares it intent(inout), and gpu_step hands the driver's
    own variable through unchanged."""
    lines = _f90_lines(F90)
    i = lines.index('integer(c_int) function mhd_step(h, tau, status) bind(C, name="mhd_step")')
    decl = next(x for x in lines[i:] if x.startswith("real(c_double)"))
    assert "intent(inout)" in decl and decl.endswith(":: tau")
    j = lines.index("subroutine gpu_step(tau)")
    assert lines[j + 1] == "real(c_double), intent(inout) :: tau"
    assert "rc = mhd_step(gpu_handle, tau, status)" in lines[j:j + 8]
    assert "subroutine gpu_set_tau(tau)" in lines
