"""The Fortran binding module (lpm-v2_gb300/fortran/lpm_gpu.f90) against the C header: every
`bind(C, name=...)` interface names a function that include/lpm_gpu.h declares, with the same
number of arguments.  The image has no Fortran compiler, so this is the check that the shim a
maintainer adds to the reference still matches the library."""
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
