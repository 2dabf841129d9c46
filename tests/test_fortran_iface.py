"""The Fortran binding module (include/ps3d_gpu_iface.f90) against the C
header it binds (include/ps3d_gpu.h), checked as text (no Fortran compiler
here): the bind(c) derived types have the C structs' members in the same
order with the same kinds and extents, every bound procedure is declared in
the header, every named constant has the header's value, and every line fits
Fortran's 132 columns."""
import os
import re

INC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
HEADER = open(os.path.join(INC, "ps3d_gpu.h")).read()
FORTRAN = open(os.path.join(INC, "ps3d_gpu_iface.f90")).read()


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def c_struct(name):
    body = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + ";", _strip_c_comments(HEADER)).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        for n in names.split(","):
            m = re.match(r"\s*(\w+)(?:\[(\d+)\])?", n)
            out.append((m.group(1), ctype, int(m.group(2) or 1)))
    return out


def f_type(name):
    body = re.search(r"type, bind\(c\) :: " + name + r"\n(.*?)end type", FORTRAN, re.S).group(1)
    kinds = {"integer(c_int)": "int", "real(c_double)": "double"}
    out = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        ftype, names = [x.strip() for x in line.split("::")]
        for n in names.split(","):
            m = re.match(r"\s*(\w+)(?:\((\d+)\))?", n)
            out.append((m.group(1), kinds[ftype], int(m.group(2) or 1)))
    return out


def test_derived_types_match_the_c_structs():
    for name in ("ps3d_gpu_config", "ps3d_gpu_diag"):
        assert f_type(name) == c_struct(name), name


def test_bound_procedures_are_declared_in_the_header():
    bound = re.findall(r"bind\(c, name='(\w+)'\)", FORTRAN)
    declared = set(re.findall(r"\b(ps3d_(?:gpu|closure)_\w+)\s*\(", HEADER))
    assert len(bound) >= 30
    assert not [b for b in bound if b not in declared]
    # each interface's Fortran name is its C name
    for fname, cname in re.findall(r"function (\w+)\([^)]*\)\s*&?\s*bind\(c, name='(\w+)'\)", FORTRAN):
        assert fname == cname


def test_named_constants_match_the_header():
    defines = dict((k, int(v)) for k, v in re.findall(r"#define (PS3D_\w+) (\d+)", HEADER))
    consts = re.findall(r"(PS3D_\w+) = (\d+)", FORTRAN)
    assert len(consts) >= 30
    for k, v in consts:
        assert defines[k] == int(v), k


def test_lines_fit_free_form_fortran():
    assert max(len(line) for line in FORTRAN.splitlines()) <= 132


STEPPER = open(os.path.join(os.path.dirname(INC), "ps3d_gb300", "fortran", "gpu_stepper.f90")).read()


def test_gpu_stepper_uses_bound_procedures_and_overrides_the_deferred_bindings():
    bound = set(re.findall(r"bind\(c, name='(\w+)'\)", FORTRAN))
    called = set(re.findall(r"\b(ps3d_(?:gpu|closure)_\w+)\(", STEPPER))
    assert called and not (called - bound), called - bound
    # base_stepper's deferred bindings (src/stepper/advance.f90:31-59), with
    # their dummy arguments
    bindings = dict(re.findall(r"procedure :: (\w+) => (\w+)", STEPPER))
    assert {"set_diffusion", "setup", "step"} <= set(bindings)
    args = {k: re.search(r"subroutine " + v + r"\(([^)]*)\)", STEPPER).group(1).replace(" ", "")
            for k, v in bindings.items()}
    assert args["set_diffusion"] == "self,dt,vorch,bf"
    assert args["setup"] == "self"
    assert args["step"] == "self,t,dt"
    assert max(len(line) for line in STEPPER.splitlines()) <= 132
