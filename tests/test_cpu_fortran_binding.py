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
