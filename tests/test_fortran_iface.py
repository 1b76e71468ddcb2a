"""include/p2m_iface.f90 (the ISO_C_BINDING module a Fortran host such as pks2map.f90 uses)
against the C headers, without a Fortran compiler: the bind(C) derived types have the C
structs' fields in the same order with interoperable kinds and the same array sizes,
every interface binds a function the headers declare and the library exports, with the
same number of arguments, scalars passed by value and pointers by reference (or as
type(c_ptr), value), and the integer parameters equal the C enumerators."""
import os
import re

import pytest

import matt_young_mapmaking_gb300 as p2m

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "include", "p2m_iface.f90")
HEADERS = [os.path.join(ROOT, "include", h) for h in ("p2m.h", "p2m_tools.h")]

C_TO_F = {"int32_t": "integer(c_int)", "int": "integer(c_int)",
          "int64_t": "integer(c_long_long)", "float": "real(c_float)",
          "double": "real(c_double)"}
MAXMAPS = 8


def _strip_c_comments(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def _fortran_lines():
    """the module's statements, comments dropped and & continuations joined"""
    out, cur = [], ""
    with open(F90) as f:
        for raw in f:
            line = raw.split("!", 1)[0].rstrip()
            if not line.strip():
                continue
            if cur:
                line = cur + " " + line.strip().lstrip("&").strip()
                cur = ""
            if line.endswith("&"):
                cur = line[:-1].rstrip()
                continue
            out.append(line.strip())
    return out


def c_struct(name):
    text = _strip_c_comments("".join(open(h).read() for h in HEADERS))
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, rest = decl.split(None, 1)
        for part in rest.split(","):
            part = part.strip()
            dm = re.match(r"(\w+)(?:\[(\w+)\])?$", part)
            assert dm, part
            dim = dm.group(2)
            fields.append((dm.group(1), C_TO_F[ctype], MAXMAPS if dim == "P2M_MAXMAPS" else
                           (int(dim) if dim else None)))
    return fields


def f_type(name):
    lines = _fortran_lines()
    i = lines.index("type, bind(C) :: %s" % name)
    fields = []
    for line in lines[i + 1:]:
        if line.startswith("end type"):
            break
        kind, names = [x.strip() for x in line.split("::")]
        for nm in names.split(","):
            nm = nm.strip()
            dm = re.match(r"(\w+)(?:\((\w+)\))?$", nm)
            dim = dm.group(2)
            fields.append((dm.group(1), kind, MAXMAPS if dim == "P2M_MAXMAPS" else
                           (int(dim) if dim else None)))
    return fields


@pytest.mark.parametrize("name", ["p2m_config", "p2m_stats", "p2m_map_stats"])
def test_bind_c_types_match_c_structs(name):
    assert f_type(name) == c_struct(name)


def c_prototypes():
    text = _strip_c_comments("".join(open(h).read() for h in HEADERS))
    protos = {}
    for m in re.finditer(r"(?:^|\n)\s*([\w ]+?[\s\*]+)(p2m_\w+)\s*\(([^;{]*?)\)\s*;", text):
        args = [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]
        protos[m.group(2)] = args
    return protos


def f_interfaces():
    lines = _fortran_lines()
    funcs, cur = {}, None
    for line in lines:
        m = re.match(r"(?:[\w(), ]+ )?(?:function|subroutine) (\w+)\(([^)]*)\).*bind\(C, "
                     r"name=\"(\w+)\"\)", line)
        if m:
            cur = {"fname": m.group(1), "args": [a.strip() for a in m.group(2).split(",")
                                                 if a.strip()], "decl": {}}
            funcs[m.group(3)] = cur
            continue
        if line.startswith("end function") or line.startswith("end subroutine"):
            cur = None
            continue
        if cur is not None and "::" in line and not line.startswith("import"):
            attrs, names = [x.strip() for x in line.split("::")]
            for nm in names.split(","):
                cur["decl"][re.match(r"(\w+)", nm.strip()).group(1)] = attrs
    return funcs


def test_interfaces_match_c_prototypes_and_exports():
    protos = c_prototypes()
    funcs = f_interfaces()
    exported = set(p2m.exported_symbols())
    assert len(funcs) >= 18
    for cname, f in funcs.items():
        assert cname in protos, "%s is not declared in the C headers" % cname
        assert cname in exported, "%s is not exported by the library" % cname
        cargs = protos[cname]
        assert len(cargs) == len(f["args"]), "%s: %d C arguments, %d Fortran" % (
            cname, len(cargs), len(f["args"]))
        for carg, farg in zip(cargs, f["args"]):
            attrs = f["decl"][farg]
            is_ptr = "*" in carg or "[" in carg
            if is_ptr:
                # a C pointer: a Fortran argument by reference, or type(c_ptr) by value
                assert ("value" not in attrs) or attrs.startswith("type(c_ptr)"), (cname, farg)
            else:
                ctype = carg.split()[0]
                assert "value" in attrs, "%s: scalar %s must be passed by value" % (cname, farg)
                assert attrs.startswith(C_TO_F[ctype]), (cname, farg, attrs, ctype)


def test_parameters_equal_c_enumerators():
    text = _strip_c_comments(open(HEADERS[0]).read())
    cvals = {m.group(1): int(m.group(2))
             for m in re.finditer(r"\b(P2M_\w+)\s*=\s*(\d+)", text)}
    cvals.update({m.group(1): int(m.group(2))
                  for m in re.finditer(r"#define (P2M_MAX\w+) (\d+)", text)})
    fvals = {}
    for line in _fortran_lines():
        if "parameter ::" in line:
            for m in re.finditer(r"(P2M_\w+) = (\d+)", line.split("::", 1)[1]):
                fvals[m.group(1)] = int(m.group(2))
    assert len(fvals) >= 20
    for k, v in fvals.items():
        assert cvals.get(k) == v, "%s: Fortran %d, C %s" % (k, v, cvals.get(k))
