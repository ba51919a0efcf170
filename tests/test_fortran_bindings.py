"""The Fortran binding module (lpm-v2_gb300/fortran/lpm_gpu.f90) against the C header: every
`bind(C, name=...)` interface names a function that include/lpm_gpu.h declares, with the same
number of arguments, each of the C parameter's kind and passing.  The image has no Fortran
compiler, so this is the check that the shim a maintainer adds to the reference still
matches the library."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _fortran_interfaces():
    text = (ROOT / "lpm-v2_gb300" / "fortran" / "lpm_gpu.f90").read_text()
    lines = []
    for raw in text.splitlines():
        line = raw.split("!")[0].rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + line.strip().lstrip("&")
        else:
            lines.append(line)
    out = {}
    pat = re.compile(r'function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name="(\w+)"\)', re.I)
    for line in lines:
        m = pat.search(line)
        if m:
            args = [a.strip() for a in m.group(2).split(",") if a.strip()]
            out[m.group(3)] = len(args)
    return out


def _c_prototypes():
    text = (ROOT / "include" / "lpm_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(lpm_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        params = m.group(2).strip()
        n = 0 if params in ("", "void") else len([p for p in params.split(",") if p.strip()])
        out[m.group(1)] = n
    return out


def test_every_fortran_interface_matches_a_c_prototype():
    f = _fortran_interfaces()
    c = _c_prototypes()
    assert len(f) >= 30
    for name, nargs in f.items():
        assert name in c, f"{name} is bound in the Fortran module but not declared in lpm_gpu.h"
        assert nargs == c[name], f"{name}: {nargs} Fortran arguments, {c[name]} C parameters"


def test_the_reference_routines_have_bindings():
    f = _fortran_interfaces()
    for name in ("lpm_bve_velocity", "lpm_plane_velocity", "lpm_pse_sphere_laplacian", "lpm_bve_stream_functions",
                 "lpm_swe_sphere_rhs_integrals", "lpm_beta_plane_velocity", "lpm_bve_solver_create",
                 "lpm_bve_timestep", "lpm_bve_solver_remesh", "lpm_ensemble_create", "lpm_last_error_string"):
        assert name in f


def _fortran_dummies():
    """name -> (result type, [(base, kind, by_value) per dummy argument in order])."""
    text = (ROOT / "lpm-v2_gb300" / "fortran" / "lpm_gpu.f90").read_text()
    lines = []
    for raw in text.splitlines():
        line = raw.split("!")[0].rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + line.strip().lstrip("&")
        else:
            lines.append(line.strip())
    head = re.compile(r'^(integer\(c_int\)|type\(c_ptr\))\s+function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name="(\w+)"\)',
                      re.I)
    decl = re.compile(r"^(integer|real|type)\((c_\w+)\)\s*((?:,\s*[\w()]+)*)\s*::\s*(.+)$", re.I)
    out, cur = {}, None
    for line in lines:
        m = head.match(line)
        if m:
            cur = (m.group(4), m.group(1).lower(), [a.strip() for a in m.group(3).split(",") if a.strip()], {})
            continue
        if cur is None:
            continue
        if re.match(r"^end\s+function", line, re.I):
            name, res, args, types = cur
            out[name] = (res, [types[a.lower()] for a in args])
            cur = None
            continue
        d = decl.match(line)
        if d:
            by_value = "value" in d.group(3).lower()
            for v in re.split(r",\s*(?![^(]*\))", d.group(4)):
                cur[3][re.sub(r"\(.*\)", "", v).strip().lower()] = (d.group(1).lower(), d.group(2).lower(), by_value)
    return out


def _c_params():
    """name -> (return type, [(base type, pointer depth) per parameter])."""
    text = (ROOT / "include" / "lpm_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"([\w\s\*]+?)\b(lpm_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        params = m.group(3).strip()
        plist = []
        if params not in ("", "void"):
            for p in params.split(","):
                p = p.replace("const", " ").strip()
                depth = p.count("*")
                base = p.replace("*", " ").split()[0]
                plist.append((base, depth))
        out[m.group(2)] = (m.group(1).split("\n")[-1].strip(), plist)
    return out


def _allowed(base, depth):
    """The Fortran (base, kind, by_value) forms that bind a C parameter of this type."""
    ptr_value = {("type", "c_ptr", True)}
    if depth == 0:
        return {{"int64_t": ("integer", "c_int64_t", True), "int": ("integer", "c_int", True),
                 "double": ("real", "c_double", True)}[base]}
    if depth == 1:
        if base.startswith("lpm_") or base == "void":
            return ptr_value
        return {("real" if base == "double" else "integer",
                 {"double": "c_double", "int32_t": "c_int32_t", "int64_t": "c_int64_t", "int": "c_int"}[base],
                 False)} | ptr_value
    return {("type", "c_ptr", False)}  # a handle returned through T**


def test_every_fortran_argument_has_the_c_type():
    """Position by position, each dummy argument of the Fortran interfaces has the kind and
    passing (VALUE or by reference) of its C parameter: int64_t <-> integer(c_int64_t), value;
    int <-> integer(c_int), value; double <-> real(c_double), value; T* <-> an array or
    scalar of the matching kind by reference, or type(c_ptr), value; handle** <->
    type(c_ptr) by reference.  A kind mismatch here would pass garbage through the ABI
    without any compiler to catch it in this image."""
    f, c = _fortran_dummies(), _c_params()
    assert len(f) >= 30
    for name, (fres, fargs) in f.items():
        cres, cargs = c[name]
        assert (fres == "type(c_ptr)") == ("char" in cres), f"{name}: result {fres} for C {cres}"
        assert len(fargs) == len(cargs), name
        for k, (fa, ca) in enumerate(zip(fargs, cargs)):
            assert fa in _allowed(*ca), f"{name} argument {k + 1}: Fortran {fa} for C {ca}"
