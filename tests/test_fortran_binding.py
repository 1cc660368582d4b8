"""The Fortran binding (2clowns-3d_gb300/fortran/clowns_gpu_mod.F90) declares
every function of include/clowns_gpu.h with the header's argument count.

No Fortran compiler exists where these tests run, so the module is checked as
text: each `bind(C, name="...")` interface is matched to the C prototype of
that name, the dummy-argument counts must agree, and the free-form source must
keep within the standard's 132-column line limit."""
import pathlib
import re

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "clowns_gpu.h"
MODULE = ROOT / "2clowns-3d_gb300" / "fortran" / "clowns_gpu_mod.F90"


def c_prototypes():
    hdr = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    hdr = "\n".join(ln for ln in hdr.splitlines() if not ln.lstrip().startswith("#"))
    out = {}
    for m in re.finditer(r"\b([A-Za-z_]\w*)\s*\(([^;{}()]*)\)\s*;", hdr):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return out


def fortran_interfaces():
    src = MODULE.read_text()
    src = re.sub(r"!.*", "", src)                       # comments
    src = re.sub(r"&\s*\n\s*&?", " ", src)              # continuation lines
    out = {}
    pat = r"(?:subroutine|function)\s+\w+\s*\(([^)]*)\)[^\n]*?bind\s*\(\s*C\s*,\s*name\s*=\s*\"(\w+)\"\s*\)"
    for m in re.finditer(pat, src, flags=re.I):
        args = m.group(1).strip()
        out[m.group(2)] = 0 if not args else len(args.split(","))
    return out


def test_every_c_function_has_a_fortran_interface_with_its_arity():
    c = c_prototypes()
    f = fortran_interfaces()
    assert len(c) >= 30
    missing = sorted(set(c) - set(f))
    assert not missing, f"no bind(C) interface for {missing}"
    wrong = {k: (c[k], f[k]) for k in c if f[k] != c[k]}
    assert not wrong, f"argument counts differ (C, Fortran): {wrong}"


def test_fortran_source_lines_fit_free_form():
    long_lines = [i + 1 for i, ln in enumerate(MODULE.read_text().splitlines()) if len(ln) > 132]
    assert not long_lines, long_lines


def test_will_wrapper_reports_the_return_code():
    """pcgpme_will_via_gpu hands PCGPME_WILL's return code to its caller (or stops
    the run with the library's message) instead of dropping it."""
    src = MODULE.read_text()
    body = src[src.index("subroutine pcgpme_will_via_gpu"):src.index("end subroutine pcgpme_will_via_gpu")]
    assert "status = rc" in body and "stop" in body
