"""The Fortran side of the boundary (integration/bgk_gpu.F90, integration/bgk_gpu_loop.F90)
checked against the C header without a Fortran compiler (there is none on either machine).

- every `bind(c, name=...)` interface names an entry point of include/bgk2d_gb300.h, with as
  many dummy arguments as the C prototype has parameters, each of a kind that passes the C
  parameter: `value` scalars for C scalars of the same width, arrays and by-reference scalars
  for C pointers, `type(c_ptr), value` for a C pointer;
- every named constant equals the header's #define of the same name;
- the fields of `type, bind(c) :: bgk_case_desc`, laid out by the C rules for their
  interoperable kinds, have the offsets and size that the C compiler gives the struct (the
  ctypes mirror, whose offsets tests/test_abi.py measures with gcc);
- the loop module calls only entry points that the binding module declares.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F_BIND = os.path.join(ROOT, "integration", "bgk_gpu.F90")
F_LOOP = os.path.join(ROOT, "integration", "bgk_gpu_loop.F90")
HEADER = os.path.join(ROOT, "include", "bgk2d_gb300.h")

# interoperable kind -> (C base type, size in bytes)
F_KIND = {"integer(c_int)": ("int32", 4), "integer(c_int64_t)": ("int64", 8), "integer(c_size_t)": ("size_t", 8),
          "real(c_double)": ("double", 8), "real(c_float)": ("float", 4), "type(c_ptr)": ("ptr", 8),
          "character(kind=c_char)": ("char", 1), "type(bgk_case_desc)": ("bgk_case_desc", None)}
C_BASE = {"int32_t": "int32", "int": "int32", "int64_t": "int64", "size_t": "size_t", "double": "double",
          "float": "float", "char": "char", "void": "void", "bgk_handle": "bgk_handle",
          "bgk_case_desc": "bgk_case_desc", "bgk_batch": "bgk_batch", "bgk_server": "bgk_server"}


def _fortran_lines(path):
    """Source lines with comments removed and `&` continuations joined."""
    out, buf = [], ""
    for raw in open(path):
        line = raw.split("!")[0].rstrip()
        if not line.strip():
            continue
        if line.endswith("&"):
            buf += line[:-1] + " "
            continue
        out.append((buf + line).strip())
        buf = ""
    return out


def _header_prototypes():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = {}
    for name, params in re.findall(r"^(?:int|const char \*)\s*(bgk_\w+)\s*\(([^)]*)\)\s*;", text, flags=re.M):
        plist = [p.strip() for p in params.replace("\n", " ").split(",") if p.strip() and p.strip() != "void"]
        protos[name] = plist
    return protos


def _c_param(p):
    """'const void *const pops[9]' -> ('void', 2): base type and levels of pointer."""
    levels = p.count("*") + p.count("[")
    words = re.sub(r"\[.*?\]|\*", " ", p).split()
    words = [w for w in words if w not in ("const", "unsigned")]
    return C_BASE[words[0]], levels


def _interfaces():
    """{name: [(dummy, kind, is_value, is_array)]} from the interface block."""
    lines = _fortran_lines(F_BIND)
    out, cur, args = {}, None, []
    for ln in lines:
        m = re.match(r"integer\(c_int\) function (\w+)\(([^)]*)\) bind\(c, name=\"(\w+)\"\)", ln)
        if m:
            assert m.group(1) == m.group(3), ln
            cur, args = m.group(1), [a.strip() for a in m.group(2).split(",") if a.strip()]
            out[cur] = {a: None for a in args}
            continue
        if cur and ln.startswith("end function"):
            assert all(v is not None for v in out[cur].values()), (cur, out[cur])
            out[cur] = [(a,) + out[cur][a] for a in args]
            cur = None
            continue
        if cur and "::" in ln and not ln.startswith("import"):
            decl, names = ln.split("::")
            attrs = [x.strip() for x in re.split(r",(?![^(]*\))", decl)]
            kind = attrs[0]
            is_value = "value" in attrs
            for nm in re.split(r",(?![^(]*\))", names):
                nm = nm.strip()
                base = nm.split("(")[0]
                out[cur][base] = (kind, is_value, "(" in nm)
    return out


def test_every_interface_binds_a_header_entry_point_with_matching_arguments():
    protos = _header_prototypes()
    ifaces = _interfaces()
    assert len(ifaces) >= 18
    for name, dummies in ifaces.items():
        assert name in protos, f"{name} is not declared in include/bgk2d_gb300.h"
        cparams = protos[name]
        assert len(dummies) == len(cparams), (name, dummies, cparams)
        for (dummy, kind, is_value, is_array), cp in zip(dummies, cparams):
            fbase, _ = F_KIND[kind]
            cbase, levels = _c_param(cp)
            where = f"{name}({dummy}) vs '{cp}'"
            if fbase == "ptr":
                # c_ptr by value is one C pointer; an array of c_ptr or a c_ptr returned through
                # the argument is a pointer to pointers
                assert levels == (1 if is_value and not is_array else 2), where
            elif is_value:
                assert not is_array and levels == 0 and cbase == fbase, where
            else:  # arrays and by-reference scalars: a pointer to the same type
                assert levels == 1 and cbase == fbase, where


def test_named_constants_equal_the_header_defines():
    text = open(HEADER).read()
    defines = {k: int(v) for k, v in re.findall(r"^#define (BGK_\w+) (-?\d+)", text, flags=re.M)}
    seen = 0
    for ln in _fortran_lines(F_BIND):
        if ln.startswith("integer(c_int), parameter ::"):
            for name, val in re.findall(r"(BGK_\w+)\s*=\s*(-?\d+)", ln):
                assert defines.get(name) == int(val), name
                seen += 1
    assert seen >= 30


def _fortran_struct_layout():
    """(field, offset) list and size of the bind(c) type under the C layout rules."""
    lines = _fortran_lines(F_BIND)
    i = lines.index("type, bind(c) :: bgk_case_desc")
    fields, off, align_max = [], 0, 1
    for ln in lines[i + 1:]:
        if ln.startswith("end type"):
            break
        kind, names = [x.strip() for x in ln.split("::")]
        _, size = F_KIND[kind]
        for nm in re.split(r",(?![^(]*\))", names):
            nm = nm.strip()
            count = 1
            m = re.match(r"(\w+)\(([\d,]+)\)", nm)
            if m:
                nm = m.group(1)
                for d in m.group(2).split(","):
                    count *= int(d)
            off = (off + size - 1) // size * size
            fields.append((nm, off))
            off += size * count
            align_max = max(align_max, size)
    return fields, (off + align_max - 1) // align_max * align_max


def test_case_desc_mirror_has_the_c_layout():
    from bgk2d_gpu_gb300 import _lib
    import ctypes
    fields, size = _fortran_struct_layout()
    C = _lib.CaseDesc
    assert [f for f, _ in fields] == [f for f, *_ in C._fields_]
    for f, off in fields:
        assert getattr(C, f).offset == off, f
    assert ctypes.sizeof(C) == size


def test_loop_module_calls_only_bound_entry_points():
    ifaces = set(_interfaces())
    text = " ".join(_fortran_lines(F_LOOP))
    called = set(re.findall(r"\b(bgk_\w+)\s*\(", text))
    helpers = {"bgk_check", "bgk_pops", "bgk_gpu_start", "bgk_gpu_next_stop", "bgk_gpu_time_loop", "bgk_gpu_stop"}
    unknown = called - ifaces - helpers
    assert not unknown, unknown
    assert {"bgk_create", "bgk_upload", "bgk_step", "bgk_download", "bgk_destroy"} <= called


def test_loop_stops_cover_every_step_where_diagnostic_acts():
    """The stops of bgk_gpu_time_loop (bgk_gpu_next_stop, restated here) visit every step at which
    SRC/diagnostic.F90 or the isignal profile does something, and the last step."""
    def next_stop(it, itfin, every):
        return min([itfin] + [(it // e + 1) * e for e in every])
    for itstart, itfin, every in ((0, 1000, (500, 100, 1000, 50)), (37, 2111, (700, 300, 10 ** 6, 250)),
                                  (0, 10, (3, 4, 5, 7))):
        stops, it = [], itstart
        while it < itfin:
            it = next_stop(it, itfin, every)
            stops.append(it)
        acts = [t for t in range(itstart + 1, itfin + 1) if any(t % e == 0 for e in every)]
        assert set(acts) <= set(stops) and stops[-1] == itfin and stops == sorted(set(stops))
