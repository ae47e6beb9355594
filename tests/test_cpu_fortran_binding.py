"""CPU check of the Fortran binding (mpi-les_gb300/fortran/module_LES_gpu.f95) against
the C header: there is no Fortran compiler here, so the module's bind(C) interfaces are
parsed and held to include/les_gpu.h -- every bound name is declared there, with the
same number of arguments, and every field id parameter has the header's value."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F95 = os.path.join(ROOT, "mpi-les_gb300", "fortran", "module_LES_gpu.f95")
HDR = os.path.join(ROOT, "include", "les_gpu.h")


def _c_functions():
    src = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(les_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return out


def _fortran_interfaces():
    src = open(F95).read()
    out = {}
    pat = r"function\s+(\w+)\s*\(([^)]*)\)\s*&?\s*bind\(C,\s*name='(\w+)'\)"
    for m in re.finditer(pat, src, flags=re.S | re.I):
        args = [a for a in m.group(2).replace("&", " ").split(",") if a.strip()]
        out[m.group(3)] = (m.group(1), len(args))
    return out


def test_every_bound_function_is_declared_with_its_arity():
    c = _c_functions()
    f = _fortran_interfaces()
    assert len(f) >= 20
    for cname, (fname, nargs) in f.items():
        assert cname in c, f"{cname} is bound in the Fortran module but not declared in les_gpu.h"
        assert fname == cname, (fname, cname)
        assert nargs == c[cname], (cname, nargs, c[cname])


def test_field_id_parameters_match_the_header():
    hdr = open(HDR).read()
    ids = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(LES_FIELD_\w+)\s*=\s*(\d+)", hdr)}
    f95 = open(F95).read()
    seen = 0
    for m in re.finditer(r"\b(LES_FIELD_\w+)\s*=\s*(\d+)", f95):
        assert ids.get(m.group(1)) == int(m.group(2)), m.group(0)
        seen += 1
    assert seen >= 20


def test_python_binding_arity_matches_the_header(built_lib):
    """lesgpu's ctypes signatures take as many arguments as les_gpu.h declares."""
    import lesgpu
    lib = lesgpu.load_library()
    c = _c_functions()
    checked = 0
    for name, nargs in c.items():
        fn = getattr(lib, name, None)
        if fn is None or fn.argtypes is None:
            continue
        assert len(fn.argtypes) == nargs, (name, len(fn.argtypes), nargs)
        checked += 1
    assert checked >= 40, checked


def _params_literal():
    """The arguments of the les_params(...) constructor in initialise_LES_gpu."""
    src = open(F95).read()
    m = re.search(r"prm\s*=\s*les_params\((.*)\)\s*$", src, flags=re.M)
    assert m, "initialise_LES_gpu builds no les_params"
    args, depth, cur = [], 0, ""
    for ch in m.group(1):
        if ch == "," and depth == 0:
            args.append(cur.strip())
            cur = ""
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur += ch
    args.append(cur.strip())
    return args, src


def test_drop_in_takes_the_reference_sor_exit_by_default():
    """press.f95:119-121 leaves the SOR loop once sor < pjuge; the drop-in's handle must
    do the same unless the caller asks for fixed iterations (fixed_sor = .true.)."""
    args, src = _params_literal()
    names = ["dt", "ro", "vn", "alpha", "beta", "omega", "pjuge", "nmaxp", "sor_fixed", "sor_ksplit"]
    assert len(args) == len(names), args
    a = dict(zip(names, args))
    assert a["sor_fixed"] == "sor_fixed"
    # the variable starts at 0 and only an explicit fixed_sor = .true. sets it
    body = src[src.index("subroutine initialise_LES_gpu"):src.index("end subroutine", src.index("subroutine initialise_LES_gpu"))]
    assert re.search(r"logical,\s*intent\(in\),\s*optional\s*::\s*fixed_sor", body)
    assert re.search(r"^\s*sor_fixed\s*=\s*0\s*$", body, flags=re.M)
    assert re.search(r"if\s*\(present\(fixed_sor\)\)", body)
    assert re.search(r"if\s*\(fixed_sor\)\s*sor_fixed\s*=\s*1", body)
    assert a["sor_ksplit"] == "0"


def test_drop_in_constants_are_the_references():
    """set.f95:89-95 (dt from the caller, ro, vn, alpha, beta) and press.f95:43-45
    (pjuge, nmaxp, omega), evaluated in FP32 as the reference writes them."""
    import numpy as np
    args, _ = _params_literal()
    f32 = np.float32
    val = {}
    for name, expr in zip(["ro", "vn", "alpha", "beta", "omega", "pjuge", "nmaxp"], args[1:8]):
        e = expr.replace("**", "^")
        if name == "vn":
            assert e.replace(" ", "") == "15.83*10.^(-6.)", expr
            val[name] = f32(f32(15.83) * f32(10.0) ** f32(-6.0))
        else:
            val[name] = f32(float(expr))
    assert args[0] == "dt"
    assert val["ro"] == f32(1.1763)
    assert val["vn"] == f32(15.83) * f32(1e-6)
    assert val["alpha"] == f32(-10.0) and val["beta"] == f32(-1.0)
    assert val["omega"] == f32(1.0)
    assert val["pjuge"] == f32(0.0001)
    assert int(val["nmaxp"]) == 50
