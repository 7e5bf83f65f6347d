"""Program units and statements of the Fortran-subset translator.

Turns the statement list of ``fparse.read_statements`` into program units
(modules, subroutines, functions) with declarations and a nested statement
tree.  Test infrastructure: it exists to run the reference's own source on
the CPU and pin the oracle against it.
"""

from __future__ import annotations

import re
from dataclasses import dataclass, field

from .fparse import (Ctor, FortranError, Kw, Name, Ref, Slice, Stmt, find_top, matching_paren,
                     parse_expr, split_top)

TYPE_WORDS = ("integer", "real", "logical", "complex", "character", "double precision",
              "doubleprecision", "double complex")


@dataclass
class Decl:
    name: str
    base: str                  # int | int8 | real | complex | logical | char
    dims: list = None          # list of (lo, hi) expr pairs, or ":" entries, None if scalar
    attrs: set = field(default_factory=set)
    init: object = None        # parameter value / initialiser expr
    where: str = ""


@dataclass
class Unit:
    kind: str                  # module | subroutine | function
    name: str
    args: list
    file: str
    decls: dict = field(default_factory=dict)     # name -> Decl (insertion ordered)
    uses: list = field(default_factory=list)
    body: list = field(default_factory=list)
    result: str = ""
    result_type: str = ""
    implicit_none: bool = False


# statement tree nodes
@dataclass
class Assign:
    lhs: object
    rhs: object
    where: str


@dataclass
class Call:
    name: str
    args: list
    where: str


@dataclass
class If:
    branches: list             # [(cond, [stmts])]; cond None for else
    where: str


@dataclass
class Do:
    var: str
    lo: object
    hi: object
    step: object
    body: list
    where: str


@dataclass
class DoWhile:
    cond: object               # None: endless loop
    body: list
    where: str


@dataclass
class Select:
    expr: object
    cases: list                # [(list of values/Slice, or None for default, [stmts])]
    where: str


@dataclass
class Where:
    branches: list             # [(mask or None, [Assign])]
    where: str


@dataclass
class Simple:
    what: str                  # exit | cycle | return | stop | continue | ignore
    where: str
    arg: object = None


@dataclass
class Alloc:
    dealloc: bool
    items: list                # Ref (allocate) or Name (deallocate)
    where: str


@dataclass
class Goto:
    label: str
    where: str


@dataclass
class Label:
    label: str
    where: str


def _base_type(spec: str, where: str) -> str:
    s = spec.replace(" ", "")
    if s.startswith("doubleprecision"):
        return "real"
    if s.startswith("doublecomplex"):
        return "complex"
    if s.startswith("integer"):
        m = re.match(r"integer(\*(\d+)|\((kind=)?(\d+)\))?$", s)
        if not m:
            raise FortranError(f"{where}: integer spec {spec!r}")
        kind = m.group(2) or m.group(4) or "4"
        return "int8" if kind == "8" else "int"
    if s.startswith("real"):
        return "real"          # default real promoted to 8 bytes (-r8)
    if s.startswith("complex"):
        return "complex"
    if s.startswith("logical"):
        return "logical"
    if s.startswith("character"):
        return "char"
    raise FortranError(f"{where}: unknown type {spec!r}")


def _dims(text: str, where: str) -> list:
    out = []
    for d in split_top(text):
        if d == ":" or d == "*":
            out.append(d)
        elif find_top(d, ":") >= 0:
            i = find_top(d, ":")
            out.append((parse_expr(d[:i], where), parse_expr(d[i + 1:], where)))
        else:
            out.append((None, parse_expr(d, where)))
    return out


def _is_type_stmt(t: str) -> bool:
    for w in TYPE_WORDS:
        if t.startswith(w):
            rest = t[len(w):].lstrip()
            if rest == "" or rest[0] in ",:(*" or re.match(r"[a-z_]", rest) or rest.startswith("::"):
                # exclude "real(x) = ..." style assignments (never used) and function headers
                if re.match(r"^[a-z ]*function\b", rest) or " function " in (" " + rest):
                    return False
                return True
    return False


def parse_decl(unit: Unit, st: Stmt):
    t = st.text
    where = st.where()
    # split type spec from the rest
    m = re.match(r"^(double\s*precision|double\s*complex|integer|real|logical|complex|character)", t)
    spec = m.group(0)
    rest = t[m.end():]
    if rest.startswith("*"):
        m2 = re.match(r"^\*\s*(\d+|\(\s*\*\s*\))", rest)
        spec += rest[:m2.end()]
        rest = rest[m2.end():]
    elif rest.lstrip().startswith("("):
        r = rest.lstrip()
        j = matching_paren(r, 0)
        kind_txt = r[:j + 1]
        rest = r[j + 1:]
        if not spec.startswith("character"):
            spec += kind_txt
    base = _base_type(spec, where)
    attrs = set()
    dims_attr = None
    if find_top(rest, ":") >= 0 and "::" in rest:
        i = rest.index("::")
        attr_txt, ents = rest[:i], rest[i + 2:]
        for a in split_top(attr_txt.strip().lstrip(",")):
            a = a.strip()
            if not a:
                continue
            if a.startswith("dimension"):
                dims_attr = _dims(a[a.index("(") + 1:a.rindex(")")], where)
            elif a.startswith("intent"):
                attrs.add("intent")
            elif a in ("parameter", "allocatable", "save", "target", "pointer", "optional",
                       "external"):
                attrs.add(a)
            else:
                raise FortranError(f"{where}: attribute {a!r}")
    else:
        ents = rest.lstrip(",")
    for e in split_top(ents):
        e = e.strip()
        if not e:
            continue
        init = None
        i = find_top(e, "=")
        if i >= 0:
            init = parse_expr(e[i + 1:], where)
            e = e[:i].strip()
        m = re.match(r"^([a-z_][a-z0-9_]*)\s*(\*\s*\d+)?\s*(\((.*)\))?$", e)
        if not m:
            raise FortranError(f"{where}: entity {e!r}")
        name = m.group(1)
        dims = _dims(m.group(4), where) if m.group(3) else dims_attr
        d = unit.decls.get(name)
        if d is None:
            unit.decls[name] = Decl(name, base, dims, set(attrs), init, where)
        else:  # e.g. dimension given earlier, or a function result typed here
            d.base = base
            d.dims = dims if dims is not None else d.dims
            d.attrs |= attrs
            d.init = init if init is not None else d.init


def parse_parameter_stmt(unit: Unit, st: Stmt):
    inner = st.text[st.text.index("(") + 1:st.text.rindex(")")]
    for e in split_top(inner):
        i = find_top(e, "=")
        name = e[:i].strip()
        val = parse_expr(e[i + 1:], st.where())
        d = unit.decls.get(name)
        if d is None:
            # implicit typing
            base = "int" if name[0] in "ijklmn" else "real"
            d = unit.decls[name] = Decl(name, base, None, set(), None, st.where())
        d.attrs.add("parameter")
        d.init = val


class UnitParser:
    def __init__(self, stmts: list):
        self.stmts = stmts
        self.i = 0

    def units(self) -> list:
        out = []
        while self.i < len(self.stmts):
            st = self.stmts[self.i]
            t = st.text
            m = re.match(r"^module\s+([a-z_][a-z0-9_]*)$", t)
            if m:
                out.append(self.unit("module", m.group(1), [], st))
                continue
            m = re.match(r"^(recursive\s+)?subroutine\s+([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", t)
            if m:
                args = [a.strip() for a in split_top(m.group(4))] if m.group(4) else []
                out.append(self.unit("subroutine", m.group(2), [a for a in args if a], st))
                continue
            m = re.match(r"^(([a-z ]+(\([^)]*\))?)\s+)?function\s+([a-z_][a-z0-9_]*)\s*\((.*)\)"
                         r"(\s*result\s*\((\w+)\))?$", t)
            if m:
                args = [a.strip() for a in split_top(m.group(5))] if m.group(5).strip() else []
                u = self.unit("function", m.group(4), args, st, prefix=(m.group(2) or "").strip(),
                              result=m.group(7))
                out.append(u)
                continue
            m = re.match(r"^program\s+", t)
            if m:
                # skip the main program (the translator's driver replaces it)
                while not re.match(r"^end(\s*program.*)?$", self.stmts[self.i].text):
                    self.i += 1
                self.i += 1
                continue
            raise FortranError(f"{st.where()}: unexpected statement outside a unit: {t!r}")
        return out

    def unit(self, kind, name, args, st, prefix="", result=None) -> Unit:
        u = Unit(kind, name, args, st.file)
        if kind == "function":
            u.result = result or name
            if prefix:
                u.result_type = _base_type(prefix, st.where())
        self.i += 1
        # specification part
        while self.i < len(self.stmts):
            s = self.stmts[self.i]
            t = s.text
            if t.startswith("use "):
                u.uses.append(t[4:].split(",")[0].strip())
            elif t == "implicit none":
                u.implicit_none = True
            elif _is_type_stmt(t):
                parse_decl(u, s)
            elif re.match(r"^parameter\s*\(", t):
                parse_parameter_stmt(u, s)
            elif re.match(r"^(save|external|intrinsic)\b", t):
                pass
            elif t.startswith("data "):
                raise FortranError(f"{s.where()}: DATA statements are not supported")
            elif t.startswith("contains"):
                raise FortranError(f"{s.where()}: CONTAINS is not supported")
            else:
                break
            self.i += 1
        if kind == "module":
            end = self.stmts[self.i]
            if not re.match(r"^end(\s*module.*)?$", end.text):
                raise FortranError(f"{end.where()}: executable statement in module")
            self.i += 1
            return u
        body, term = self.block(("end",))
        u.body = body
        return u

    # ---------------------------------------------------------------------
    def block(self, terminators):
        """Parse statements until one whose text starts a terminator; return
        (stmts, terminating Stmt)."""
        out = []
        while self.i < len(self.stmts):
            st = self.stmts[self.i]
            t = st.text
            w = st.where()
            if st.label:
                out.append(Label(st.label, w))
            if self._is_term(t, terminators):
                self.i += 1
                return out, st
            self.i += 1
            out.extend(self.statement(st))
        raise FortranError(f"unterminated block, expected {terminators}")

    @staticmethod
    def _is_term(t, terms) -> bool:
        for term in terms:
            if term == "end":
                if re.match(r"^end(\s*(subroutine|function|program)\b.*)?$", t):
                    return True
            elif term == "enddo":
                if re.match(r"^end\s*do$", t):
                    return True
            elif term == "endif":
                if re.match(r"^end\s*if$", t):
                    return True
            elif term == "else":
                if re.match(r"^else(\s*if\b.*)?$", t) or t == "else":
                    return True
            elif term == "endselect":
                if re.match(r"^end\s*select$", t):
                    return True
            elif term == "case":
                if re.match(r"^case\b", t):
                    return True
            elif term == "endwhere":
                if re.match(r"^end\s*where$", t):
                    return True
            elif term == "elsewhere":
                if re.match(r"^else\s*where(\s*\(.*\))?$", t):
                    return True
            elif term == "continue_label":
                pass
        return False

    def statement(self, st: Stmt) -> list:
        t = st.text
        w = st.where()
        # block IF
        m = re.match(r"^if\s*\(", t)
        if m:
            j = matching_paren(t, t.index("("))
            cond = parse_expr(t[t.index("(") + 1:j], w)
            rest = t[j + 1:].strip()
            if rest == "then":
                return [self.if_block(cond, w)]
            if not rest:
                raise FortranError(f"{w}: empty IF")
            inner = self.statement(Stmt(rest, st.file, st.line))
            return [If([(cond, inner)], w)]
        m = re.match(r"^do\s*(\d+\s+)?(.*)$", t)
        if m and (t == "do" or re.match(r"^do\s+(while\b|[a-z_])", t) or t.startswith("do while")):
            if m.group(1):
                raise FortranError(f"{w}: labelled DO is not supported")
            rest = m.group(2).strip()
            if rest == "":
                body, _ = self.block(("enddo",))
                return [DoWhile(None, body, w)]
            mw = re.match(r"^while\s*\((.*)\)$", rest)
            if mw:
                cond = parse_expr(mw.group(1), w)
                body, _ = self.block(("enddo",))
                return [DoWhile(cond, body, w)]
            i = find_top(rest, "=")
            var = rest[:i].strip()
            parts = split_top(rest[i + 1:])
            lo = parse_expr(parts[0], w)
            hi = parse_expr(parts[1], w)
            step = parse_expr(parts[2], w) if len(parts) > 2 else None
            body, _ = self.block(("enddo",))
            return [Do(var, lo, hi, step, body, w)]
        m = re.match(r"^select\s*case\s*\((.*)\)$", t)
        if m:
            return [self.select_block(parse_expr(m.group(1), w), w)]
        m = re.match(r"^where\s*\(", t)
        if m:
            j = matching_paren(t, t.index("("))
            mask = parse_expr(t[t.index("(") + 1:j], w)
            rest = t[j + 1:].strip()
            if rest:
                return [Where([(mask, self.statement(Stmt(rest, st.file, st.line)))], w)]
            return [self.where_block(mask, w)]
        if re.match(r"^call\s", t):
            rest = t[5:].strip()
            if "(" in rest:
                k = rest.index("(")
                name = rest[:k].strip()
                j = matching_paren(rest, k)
                args = split_top(rest[k + 1:j]) if rest[k + 1:j].strip() else []
                return [Call(name, [self._arg(a, w) for a in args], w)]
            return [Call(rest, [], w)]
        if t in ("exit", "cycle", "return", "continue"):
            return [Simple(t, w)]
        if t.startswith("stop"):
            return [Simple("stop", w, t[4:].strip())]
        m = re.match(r"^go\s*to\s+(\d+)$", t)
        if m:
            return [Goto(m.group(1), w)]
        if re.match(r"^(write|print|read|open|close|format|flush|rewind|inquire)\b", t):
            return [Simple("ignore", w, t)]
        m = re.match(r"^(de)?allocate\s*\((.*)\)$", t)
        if m:
            items = [parse_expr(a, w) for a in split_top(m.group(2)) if not a.startswith("stat")]
            return [Alloc(bool(m.group(1)), items, w)]
        i = find_top(t, "=")
        if i > 0 and t[i - 1] not in "<>/=" and t[i + 1:i + 2] != "=":
            lhs = parse_expr(t[:i], w)
            rhs = parse_expr(t[i + 1:], w)
            return [Assign(lhs, rhs, w)]
        raise FortranError(f"{w}: unsupported statement {t!r}")

    @staticmethod
    def _arg(a: str, w):
        i = find_top(a, "=")
        if i > 0 and a[i + 1:i + 2] != "=" and a[i - 1] not in "<>/=" and re.match(r"^\s*[a-z_]\w*\s*$", a[:i]):
            return Kw(a[:i].strip(), parse_expr(a[i + 1:], w))
        return parse_expr(a, w)

    def if_block(self, cond, w):
        branches = []
        body, term = self.block(("else", "endif"))
        branches.append((cond, body))
        while True:
            t = term.text
            if re.match(r"^end\s*if$", t):
                return If(branches, w)
            m = re.match(r"^else\s*if\s*\(", t)
            if m:
                j = matching_paren(t, t.index("("))
                c = parse_expr(t[t.index("(") + 1:j], term.where())
                body, term = self.block(("else", "endif"))
                branches.append((c, body))
                continue
            if t == "else":
                body, term = self.block(("endif",))
                branches.append((None, body))
                continue
            raise FortranError(f"{term.where()}: bad IF terminator {t!r}")

    def select_block(self, e, w):
        cases = []
        # skip to the first CASE
        body, term = self.block(("case", "endselect"))
        if body:
            raise FortranError(f"{w}: statements before the first CASE")
        while True:
            t = term.text
            if re.match(r"^end\s*select$", t):
                return Select(e, cases, w)
            if re.match(r"^case\s+default$", t):
                vals = None
            else:
                m = re.match(r"^case\s*\((.*)\)$", t)
                vals = []
                for a in split_top(m.group(1)):
                    if find_top(a, ":") >= 0:
                        i = find_top(a, ":")
                        lo = parse_expr(a[:i], w) if a[:i].strip() else None
                        hi = parse_expr(a[i + 1:], w) if a[i + 1:].strip() else None
                        vals.append(Slice(lo, hi))
                    else:
                        vals.append(parse_expr(a, w))
            body, term = self.block(("case", "endselect"))
            cases.append((vals, body))

    def where_block(self, mask, w):
        branches = []
        body, term = self.block(("elsewhere", "endwhere"))
        branches.append((mask, body))
        while True:
            t = term.text
            if re.match(r"^end\s*where$", t):
                return Where(branches, w)
            m = re.match(r"^else\s*where\s*(\((.*)\))?$", t)
            c = parse_expr(m.group(2), w) if m.group(1) else None
            body, term = self.block(("elsewhere", "endwhere"))
            branches.append((c, body))


def parse_units(text: str, fname: str, patches=()) -> list:
    from .fparse import read_statements
    return UnitParser(read_statements(text, fname, patches)).units()
