"""The ISO_C_BINDING module that a maintainer adds to the reference
(``module lbm_gpu``) against the C ABI (include/lbm.h).

No Fortran compiler exists on either machine, so the module cannot be
compiled here.  These tests hold its text to the C declarations by the
interoperability rules of Fortran 2003 (ISO/IEC 1539-1, 15.3): a dummy with
VALUE is passed as the C value; without VALUE it is passed by reference
(one more level of pointer), an assumed-size array ``x(*)`` as a pointer to
its first element; ``type(c_ptr)`` is a C object pointer, ``integer(c_int)``
an ``int``, ``integer(c_int32_t)`` an ``int32_t``, ``real(c_double)`` a
``double``; a BIND(C) derived type matches the C struct whose members have
the same types in the same order.  A dummy declared INTENT(IN) must not
stand for a C pointer the callee writes through.  The release-block snippet
and the list of per-subroutine entries of the same shape are checked too.
No GPU is needed.
"""

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

F_KINDS = {"integer(c_int)": "int", "integer(c_int32_t)": "int32_t",
           "integer(c_int64_t)": "int64_t", "real(c_double)": "double",
           "type(c_ptr)": "ptr", "type(lbm_config)": "lbm_config"}
C_INTS = {"int", "int32_t"}


def fortran_module() -> str:
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```fortran\n(.*?)```", text, re.S)
    mods = [b for b in blocks if b.lstrip().startswith("module lbm_gpu")]
    assert len(mods) == 1
    return mods[0]


def fortran_snippets() -> list:
    text = (ROOT / "INTEGRATION.md").read_text()
    return re.findall(r"```fortran\n(.*?)```", text, re.S)


def parse_module(src: str):
    """(derived type fields, interface functions) of the module text."""
    fields, funcs = [], {}
    lines = [ln.split("!")[0].rstrip() for ln in src.splitlines()]
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        if ln.startswith("type, bind(C) :: lbm_config"):
            i += 1
            while not lines[i].strip().startswith("end type"):
                kind, names = [s.strip() for s in lines[i].split("::")]
                for nm in re.findall(r"(\w+)(?:\((\d+)\))?", names):
                    fields.append((nm[0], F_KINDS[kind], int(nm[1] or 1)))
                i += 1
        m = re.match(r"integer\(c_int\) function (\w+)\(([^)]*)\) bind\(C(?:, name=\"(\w+)\")?\)", ln)
        if m:
            fname, args, cname = m.group(1), [a.strip() for a in m.group(2).split(",") if a.strip()], m.group(3)
            decl = {}
            i += 1
            while not lines[i].strip().startswith("end function"):
                for st in lines[i].split(";"):
                    st = st.strip()
                    if not st or st == "import":
                        continue
                    spec, names = [s.strip() for s in st.split("::")]
                    parts = [p.strip() for p in re.split(r",(?![^(]*\))", spec)]
                    kind, attrs = F_KINDS[parts[0]], set(parts[1:])
                    for nm in [n.strip() for n in names.split(",")]:
                        arr = nm.endswith("(*)")
                        decl[nm.replace("(*)", "")] = (kind, "value" in attrs, arr,
                                                       "intent(in)" in attrs)
                i += 1
            assert set(decl) == set(args), (fname, args, decl)
            funcs[cname or fname] = [decl[a] for a in args]
        i += 1
    return fields, funcs


def c_header():
    src = (ROOT / "include" / "lbm.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|int64_t)\s+(lbm_\w+)\s*\(([^)]*)\)\s*;", src):
        params = []
        for p in [q.strip() for q in m.group(2).split(",") if q.strip() and q.strip() != "void"]:
            const = p.startswith("const ")
            p = p.replace("const ", "")
            arr = re.search(r"\[\d*\]$", p)
            p = re.sub(r"\[\d*\]$", "", p)
            depth = p.count("*") + (1 if arr else 0)
            base = p.replace("*", " ").split()[0]
            params.append((base, depth, const))
        protos[m.group(1)] = params
    body = re.search(r"typedef struct lbm_config \{(.*?)\} lbm_config;", src, re.S).group(1)
    fields = []
    for st in [s.strip() for s in body.split(";") if s.strip()]:
        typ, names = st.split(None, 1)
        for nm in [n.strip() for n in names.split(",")]:
            m = re.match(r"(\w+)(?:\[(\d+)\])?", nm)
            fields.append((m.group(1), typ, int(m.group(2) or 1)))
    return protos, fields


def expected(kind, value, arr):
    """The C (base, pointer depth) a Fortran dummy stands for."""
    if kind == "ptr":
        return ("*", 1 if value else 2)
    depth = 0 if (value and not arr) else 1
    return (kind, depth)


def test_derived_type_matches_the_c_struct():
    ffields, _ = parse_module(fortran_module())
    _, cfields = c_header()
    assert [(n, k, c) for n, k, c in ffields] == [(n, t, c) for n, t, c in cfields]


def test_interfaces_match_the_c_prototypes():
    _, funcs = parse_module(fortran_module())
    protos, _ = c_header()
    assert len(funcs) >= 10
    for name, fargs in funcs.items():
        assert name in protos, name
        cargs = protos[name]
        assert len(fargs) == len(cargs), name
        for (kind, value, arr, intent_in), (base, depth, const) in zip(fargs, cargs):
            eb, ed = expected(kind, value, arr)
            assert depth == ed, (name, kind, base, depth)
            if eb == "int":
                assert base in C_INTS, (name, base)
            elif eb != "*":
                assert base == eb, (name, eb, base)
            if intent_in and depth >= 1 and kind != "ptr":
                assert const, (name, "intent(in) on a pointer the C side writes through")
            if depth >= 1 and kind != "ptr" and not const:
                assert not intent_in, name


def test_per_subroutine_entries_have_the_call_shape():
    """The entries the text binds with the interface of lbm_call: int f(lbm_ctx*)."""
    text = (ROOT / "INTEGRATION.md").read_text()
    m = re.search(r"One interface per entry with the same shape as `lbm_call` \((.*?)\)", text, re.S)
    names = re.findall(r"`(lbm_\w+)`", m.group(1))
    assert len(names) == 11
    protos, _ = c_header()
    for n in names:
        assert protos[n] == [("lbm_ctx", 1, False)], n


@pytest.mark.parametrize("call,name", [
    ("lbm_release_particles(lbm_ctx, npart, ypglb)", "lbm_release_particles"),
    ("lbm_collision_mrt(lbm_ctx)", "lbm_collision_mrt"),
])
def test_snippets_call_declared_entries(call, name):
    assert any(call in s for s in fortran_snippets())
    _, funcs = parse_module(fortran_module())
    assert name in funcs or name in c_header()[0]
    nargs = call.count(",") + 1
    assert len(c_header()[0][name]) == nargs
