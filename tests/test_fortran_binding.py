"""The Fortran ISO_C_BINDING module (include/pizza_gpu.f90) against the C ABI.

No Fortran compiler is available, so the module is checked by reading it:
every bind(c) interface must name an entry point of include/pizza_gpu.h with
the same number of arguments, interoperable argument types (value vs
reference, int/double/complex/pointer) and return kind; every PZ_* parameter
must equal the header's #define; and type(pz_config) must lay out like the C
struct, whose field offsets come from gcc's offsetof on the header itself.
"""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "pizza_gpu.h")
F90 = os.path.join(ROOT, "include", "pizza_gpu.f90")


def _strip_c_comments(s):
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


def c_functions():
    """name -> (return type, [(type text, name)]) for every pz_* prototype."""
    src = _strip_c_comments(open(HDR).read())
    out = {}
    for m in re.finditer(r"(int|void\s*\*|void|const\s+char\s*\*)\s*(pz_\w+)\s*\(([^;{]*)\)\s*;", src):
        ret = re.sub(r"\s+", "", m.group(1))
        args = []
        body = m.group(3).strip()
        if body and body != "void":
            for a in body.split(","):
                a = " ".join(a.split())
                mm = re.match(r"(.*?)(\w+)$", a)
                args.append((mm.group(1).replace(" ", ""), mm.group(2)))
        out[m.group(2)] = (ret, args)
    return out


def c_defines():
    src = _strip_c_comments(open(HDR).read())
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(PZ_\w+)\s+(-?\d+)", src)}


def c_struct_fields():
    src = _strip_c_comments(open(HDR).read())
    body = re.search(r"typedef\s+struct\s+pz_config\s*\{(.*?)\}\s*pz_config;", src, re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        typ, names = decl.split(" ", 1)
        fields += [(typ, n.strip()) for n in names.split(",")]
    return fields


def _f90_lines():
    """Source lines with comments removed and & continuations joined."""
    raw = open(F90).read().split("\n")
    lines, cur = [], ""
    for ln in raw:
        ln = ln.split("!")[0].rstrip()
        if cur:
            ln = cur + " " + ln.lstrip()
            cur = ""
        if ln.endswith("&"):
            cur = ln[:-1]
            continue
        if ln.strip():
            lines.append(ln.strip())
    return lines


def f90_interfaces():
    """bind name -> (kind 'function'/'subroutine', result type, [(arg, type, attrs)])."""
    lines = _f90_lines()
    out = {}
    i = 0
    while i < len(lines):
        m = re.match(r"(?:(integer\(c_int\)|type\(c_ptr\))\s+)?(function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*"
                     r"bind\(c,\s*name='(\w+)'\)", lines[i], re.I)
        if not m:
            i += 1
            continue
        res, kind, fname, arglist, bname = m.groups()
        argnames = [a.strip().lower() for a in arglist.split(",") if a.strip()]
        decl = {}
        i += 1
        while not re.match(r"end\s+(function|subroutine)", lines[i], re.I):
            d = re.match(r"(integer\(c_int\)|real\(c_double\)|complex\(c_double_complex\)|type\(\w+\))\s*"
                         r"((?:,\s*[\w()]+(?:\([^)]*\))?)*)\s*::\s*(.*)", lines[i], re.I)
            if d:
                typ = d.group(1).lower()
                attrs = {a.strip().lower() for a in d.group(2).split(",") if a.strip()}
                for v in re.split(r",\s*(?![^()]*\))", d.group(3)):
                    vm = re.match(r"(\w+)\s*(\(.*\))?", v.strip())
                    decl[vm.group(1).lower()] = (typ, attrs, vm.group(2) or "")
            i += 1
        out[bname] = (kind.lower(), (res or "").lower(), fname.lower(),
                      [(a, *decl[a]) for a in argnames])
        i += 1
    return out


def f90_parameters():
    out = {}
    for ln in _f90_lines():
        m = re.match(r"integer\(c_int\),\s*parameter\s*::\s*(.*)", ln, re.I)
        if m:
            for item in m.group(1).split(","):
                k, v = item.split("=")
                out[k.strip()] = int(v)
    return out


def f90_struct_fields():
    lines = _f90_lines()
    s = lines.index("type, bind(c) :: pz_config")
    fields = []
    for ln in lines[s + 1:]:
        if ln.startswith("end type"):
            break
        typ, names = ln.split("::")
        fields += [(typ.strip().lower(), n.strip()) for n in names.split(",")]
    return fields


def _compatible(ctype, ftype, attrs):
    """Whether a C parameter type and a Fortran dummy interoperate."""
    by_value = "value" in attrs
    if ctype == "int":
        return ftype == "integer(c_int)" and by_value
    if ctype == "double":
        return ftype == "real(c_double)" and by_value
    if ctype.endswith("**"):
        return ftype == "type(c_ptr)" and not by_value
    if ctype in ("pz_handle*",):
        return ftype == "type(c_ptr)" and by_value
    if ctype.endswith("*"):
        base = ctype.replace("const", "")[:-1]
        if ftype == "type(c_ptr)":
            return by_value                      # an address passed as a value (device pointers)
        if by_value:
            return False
        return {"int": ftype == "integer(c_int)",
                "double": ftype in ("real(c_double)", "complex(c_double_complex)"),
                "pz_config": ftype == "type(pz_config)"}.get(base, False)
    return False


def test_every_entry_point_has_a_fortran_interface():
    cf = c_functions()
    fi = f90_interfaces()
    assert set(cf) == set(fi), (sorted(set(cf) - set(fi)), sorted(set(fi) - set(cf)))


@pytest.mark.parametrize("name", sorted(c_functions()))
def test_interface_matches_prototype(name):
    ret, cargs = c_functions()[name]
    kind, res, fname, fargs = f90_interfaces()[name]
    assert fname == name.lower()
    if ret == "void":
        assert kind == "subroutine"
    elif ret == "int":
        assert kind == "function" and res == "integer(c_int)"
    else:                                                   # void*, const char*
        assert kind == "function" and res == "type(c_ptr)"
    assert len(cargs) == len(fargs), (cargs, fargs)
    for (ct, cn), (fn, ft, attrs, dims) in zip(cargs, fargs):
        assert cn.lower() == fn, (name, cn, fn)
        assert _compatible(ct, ft, attrs), (name, cn, ct, ft, attrs)
        if "optional" in attrs:
            assert ct.endswith("*") and "value" not in attrs, (name, cn)


def test_series_rows_are_pz_series_cols_wide():
    defs = c_defines()
    for name in ("pz_get_series", "pz_latest_rows"):
        _, _, _, fargs = f90_interfaces()[name]
        dims = {a: d for a, _, _, d in fargs}
        assert dims["rows"].replace(" ", "") == f"({defs['PZ_SERIES_COLS']},*)", (name, dims["rows"])


def test_parameters_equal_header_defines():
    defs = c_defines()
    par = f90_parameters()
    for k, v in par.items():
        assert k in defs, k
        assert defs[k] == v, (k, defs[k], v)
    scheme_like = [k for k in defs if k not in par]
    assert not scheme_like, scheme_like


def _layout(fields, size_of):
    off, out, align = 0, [], 1
    for typ, name in fields:
        sz = size_of(typ)
        off = (off + sz - 1) // sz * sz
        out.append((name, off, sz))
        off += sz
        align = max(align, sz)
    return out, (off + align - 1) // align * align


def test_struct_layout_matches_c():
    cfields = c_struct_fields()
    ffields = f90_struct_fields()
    assert [n for _, n in cfields] == [n for _, n in ffields]
    csz = {"int": 4, "double": 8}
    fsz = {"integer(c_int)": 4, "real(c_double)": 8}
    for (ct, n), (ft, _) in zip(cfields, ffields):
        assert csz[ct] == fsz[ft], n
    flay, fsize = _layout(ffields, fsz.__getitem__)
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler to read the struct offsets")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "off.c")
        with open(c, "w") as f:
            f.write('#include <stdio.h>\n#include <stddef.h>\n#include "pizza_gpu.h"\nint main(void){\n')
            for _, n in cfields:
                f.write(f'printf("{n} %zu %zu\\n", offsetof(pz_config, {n}), sizeof(((pz_config*)0)->{n}));\n')
            f.write('printf("__size %zu 0\\n", sizeof(pz_config));\nreturn 0;}\n')
        exe = os.path.join(d, "off")
        subprocess.run([gcc, "-I", os.path.dirname(HDR), c, "-o", exe], check=True)
        got = {}
        for ln in subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n"):
            if ln:
                k, o, s = ln.split()
                got[k] = (int(o), int(s))
    for name, off, sz in flay:
        assert got[name] == (off, sz), (name, got[name], (off, sz))
    assert got["__size"][0] == fsize
    # the Python binding's ctypes mirror lays out the same way
    from pizza_gb300 import _CConfig
    for name, off, sz in flay:
        assert getattr(_CConfig, name).offset == off, name
    import ctypes
    assert ctypes.sizeof(_CConfig) == fsize
