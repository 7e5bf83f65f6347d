"""Front end of the Fortran-subset translator (test infrastructure).

Reads the free-form Fortran 90 of the reference's hot-path programs and
builds an abstract syntax tree per program unit: statements are split and
continuation lines joined, comments dropped, keywords and names lower-cased
(Fortran is case-insensitive), expressions parsed with Fortran's operator
precedence.  Only the subset those programs use is supported; anything else
raises ``FortranError`` with the file and line, so a silent
mistranslation cannot pass for the reference.
"""

from __future__ import annotations

import re
from dataclasses import dataclass, field


class FortranError(Exception):
    pass


# ----------------------------------------------------------------------------
# source lines -> statements

@dataclass
class Stmt:
    text: str          # lower-cased outside string literals, no comment
    file: str
    line: int
    label: str = ""

    def where(self) -> str:
        return f"{self.file}:{self.line}"


def _strip_comment(line: str) -> str:
    out = []
    q = None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def _lower_outside_strings(s: str) -> str:
    out = []
    q = None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


def _split_semicolons(s: str) -> list:
    parts, cur, q = [], [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == ";":
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


def read_statements(text: str, fname: str, patches=()) -> list:
    """Free-form source -> list of Stmt.  `patches` is a sequence of
    (old, new) literal replacements applied to the raw text first."""
    for old, new in patches:
        if old not in text:
            raise FortranError(f"{fname}: patch target not found: {old!r}")
        text = text.replace(old, new)
    lines = text.split("\n")
    stmts = []
    buf, start = "", 0
    for i, raw in enumerate(lines, 1):
        ln = _strip_comment(raw).rstrip()
        if not ln.strip():
            if buf:
                continue  # blank/comment line inside a continuation
            continue
        s = ln.strip()
        if buf:
            if s.startswith("&"):
                s = s[1:]
            buf += " " + s
        else:
            buf, start = s, i
        if buf.endswith("&"):
            buf = buf[:-1]
            continue
        for part in _split_semicolons(buf):
            part = part.strip()
            if part:
                label = ""
                m = re.match(r"^(\d+)\s+(.*)$", part)
                if m:
                    label, part = m.group(1), m.group(2)
                stmts.append(Stmt(_lower_outside_strings(part), fname, start, label))
        buf = ""
    if buf:
        raise FortranError(f"{fname}: dangling continuation at end of file")
    return stmts


# ----------------------------------------------------------------------------
# expressions

@dataclass
class Num:
    text: str
    kind: str  # "int" | "real"


@dataclass
class Str:
    value: str


@dataclass
class Logic:
    value: bool


@dataclass
class Name:
    name: str


@dataclass
class Slice:
    lo: object = None
    hi: object = None
    step: object = None


@dataclass
class Kw:
    name: str
    value: object


@dataclass
class Ref:
    """name(args): array element/section or function call (resolved later)."""
    name: str
    args: list


@dataclass
class Bin:
    op: str
    a: object
    b: object


@dataclass
class Un:
    op: str
    a: object


@dataclass
class Ctor:
    items: list


_TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<real>(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)(_\w+)? | (\d+\.\d*|\.\d+)(_\w+)?)
  | (?P<int>\d+(_\w+)?)
  | (?P<dotop>\.(eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.)
  | (?P<str>'([^']|'')*'|"([^"]|"")*")
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|//|==|/=|<=|>=|\(/|/\)|[-+*/<>(),:=%])
""", re.X)


def tokenize(s: str, where: str) -> list:
    toks = []
    pos = 0
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise FortranError(f"{where}: cannot tokenize at {s[pos:pos + 20]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        val = m.group(kind)
        if kind == "real":
            # a real literal directly followed by a dot-operator: "1.and." is 1 .and.
            pass
        toks.append((kind, val))
    # fix "1.eq.x" lexed as real "1." + name "eq" ...: re-lex digit-dot-op cases
    fixed = []
    for kind, val in toks:
        fixed.append((kind, val))
    return fixed


_DOTMAP = {".eq.": "==", ".ne.": "/=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
           ".and.": ".and.", ".or.": ".or.", ".not.": ".not.", ".eqv.": ".eqv.",
           ".neqv.": ".neqv."}


class ExprParser:
    """Recursive descent over Fortran's precedence:
    .eqv. < .or. < .and. < .not. < relational < // < + - (binary) <
    unary + - < * / < ** (right associative)."""

    def __init__(self, text: str, where: str):
        self.where = where
        text = self._separate_dot_ops(text)
        self.toks = tokenize(text, where)
        self.i = 0

    @staticmethod
    def _separate_dot_ops(text: str) -> str:
        # "1.eq.2" -> "1 .eq. 2": a digit followed by a dot-operator
        return re.sub(r"(\d)\.(eq|ne|lt|le|gt|ge|and|or|eqv|neqv)\.", r"\1 .\2.", text)

    def peek(self, k=0):
        j = self.i + k
        return self.toks[j] if j < len(self.toks) else (None, None)

    def take(self):
        t = self.peek()
        self.i += 1
        return t

    def expect(self, val):
        k, v = self.take()
        if v != val:
            raise FortranError(f"{self.where}: expected {val!r}, got {v!r}")

    def at(self, val) -> bool:
        return self.peek()[1] == val

    def done(self) -> bool:
        return self.i >= len(self.toks)

    def parse(self):
        e = self.expr()
        if not self.done():
            raise FortranError(f"{self.where}: trailing tokens {self.toks[self.i:]}")
        return e

    def expr(self):
        a = self.or_expr()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.take()[1]
            a = Bin(op, a, self.or_expr())
        return a

    def or_expr(self):
        a = self.and_expr()
        while self.at(".or."):
            self.take()
            a = Bin(".or.", a, self.and_expr())
        return a

    def and_expr(self):
        a = self.not_expr()
        while self.at(".and."):
            self.take()
            a = Bin(".and.", a, self.not_expr())
        return a

    def not_expr(self):
        if self.at(".not."):
            self.take()
            return Un(".not.", self.not_expr())
        return self.rel_expr()

    def rel_expr(self):
        a = self.concat_expr()
        k, v = self.peek()
        v = _DOTMAP.get(v, v)
        if v in ("==", "/=", "<", "<=", ">", ">="):
            self.take()
            return Bin(v, a, self.concat_expr())
        return a

    def concat_expr(self):
        a = self.add_expr()
        while self.at("//"):
            self.take()
            a = Bin("//", a, self.add_expr())
        return a

    def add_expr(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.mul_expr()
            a = Un(op, a) if op == "-" else a
        else:
            a = self.mul_expr()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = Bin(op, a, self.mul_expr())
        return a

    def mul_expr(self):
        a = self.pow_expr()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = Bin(op, a, self.pow_expr())
        return a

    def pow_expr(self):
        a = self.primary()
        if self.at("**"):
            self.take()
            if self.peek()[1] in ("+", "-"):  # x**-1
                op = self.take()[1]
                b = self.pow_expr()
                b = Un(op, b) if op == "-" else b
            else:
                b = self.pow_expr()
            return Bin("**", a, b)
        return a

    def primary(self):
        k, v = self.take()
        if k == "int":
            return Num(v.split("_")[0], "int")
        if k == "real":
            return Num(v.split("_")[0], "real")
        if k == "str":
            q = v[0]
            return Str(v[1:-1].replace(q + q, q))
        if k == "dotop":
            if v in (".true.", ".false."):
                return Logic(v == ".true.")
            raise FortranError(f"{self.where}: unexpected {v}")
        if v == "(/":
            items = []
            if not self.at("/)"):
                items.append(self.expr())
                while self.at(","):
                    self.take()
                    items.append(self.expr())
            self.expect("/)")
            return Ctor(items)
        if v == "(":
            e = self.expr()
            if self.at(","):  # complex constant (a, b)
                self.take()
                b = self.expr()
                self.expect(")")
                return Ref("cmplx", [e, b])
            self.expect(")")
            return e
        if k == "name":
            if self.at("("):
                self.take()
                args = self.arglist()
                return Ref(v, args)
            return Name(v)
        raise FortranError(f"{self.where}: unexpected token {v!r}")

    def arglist(self):
        args = []
        if self.at(")"):
            self.take()
            return args
        while True:
            args.append(self.arg())
            if self.at(","):
                self.take()
                continue
            self.expect(")")
            return args

    def arg(self):
        # keyword argument name = expr
        k, v = self.peek()
        if k == "name" and self.peek(1)[1] == "=":
            self.take()
            self.take()
            return Kw(v, self.expr())
        # slice forms  :  a:  :b  a:b  a:b:s
        lo = hi = st = None
        if self.at(":"):
            self.take()
            if not (self.at(",") or self.at(")") or self.at(":")):
                hi = self.expr()
            if self.at(":"):
                self.take()
                st = self.expr()
            return Slice(lo, hi, st)
        e = self.expr()
        if self.at(":"):
            self.take()
            lo = e
            if not (self.at(",") or self.at(")") or self.at(":")):
                hi = self.expr()
            if self.at(":"):
                self.take()
                st = self.expr()
            return Slice(lo, hi, st)
        return e


def parse_expr(text: str, where: str):
    return ExprParser(text, where).parse()


def split_top(text: str, sep: str = ",") -> list:
    """Split at top-level separators (outside parentheses and strings)."""
    parts, cur, depth, q = [], [], 0, None
    i = 0
    while i < len(text):
        ch = text[i]
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == "(":
            depth += 1
            cur.append(ch)
        elif ch == ")":
            depth -= 1
            cur.append(ch)
        elif ch == sep and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
        i += 1
    parts.append("".join(cur).strip())
    return parts


def find_top(text: str, ch: str) -> int:
    """Index of the first top-level `ch` (outside parentheses/strings), -1 if none."""
    depth, q = 0, None
    for i, c in enumerate(text):
        if q:
            if c == q:
                q = None
        elif c in "'\"":
            q = c
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        elif c == ch and depth == 0:
            return i
    return -1


def matching_paren(text: str, start: int) -> int:
    """Index of the ')' matching the '(' at `start`."""
    depth, q = 0, None
    for i in range(start, len(text)):
        c = text[i]
        if q:
            if c == q:
                q = None
        elif c in "'\"":
            q = c
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return i
    raise FortranError(f"unbalanced parentheses in {text!r}")
