"""Code generator of the Fortran-subset translator (test infrastructure).

Emits one C++ translation unit per program: the module variables as
globals (with an initialiser that applies parameter overrides), every
reachable subroutine and function, a table that exposes module variables by
name, and a dispatcher for argument-free subroutines.  Semantics kept from
Fortran:

* default REAL is 8 bytes (the reference was built with default reals
  promoted to 8 bytes); real literals are double;
* expressions are emitted fully parenthesised in source order, and the
  generated code is compiled without floating-point contraction;
* x**n with integer n is a left-to-right product; integer division
  truncates; array assignments evaluate the right-hand side before storing
  when it references the array being assigned;
* arguments pass by reference; explicit-shape dummies view the caller's
  memory with their own bounds (sequence association); array sections
  that are not contiguous pass through copy-in/copy-out temporaries;
* element addresses follow Fortran's linear address arithmetic, and a
  reference outside the array's allocation raises an error instead of
  touching other memory.
"""

from __future__ import annotations

from .fparse import Bin, Ctor, FortranError, Kw, Logic, Name, Num, Ref, Slice, Str, Un
from .funits import (Alloc, Assign, Call, Decl, Do, DoWhile, Goto, If, Label, Select, Simple,
                     Unit, Where)

CTYPE = {"int": "int32_t", "int8": "int64_t", "real": "double", "complex": "frt::cplx",
         "logical": "bool", "char": "std::string"}

MPI_CONST = {
    "mpi_comm_world": ("int", "frt::mpi::COMM_WORLD"), "mpi_real8": ("int", "frt::mpi::REAL8"),
    "mpi_integer": ("int", "frt::mpi::INTEGER"), "mpi_real": ("int", "frt::mpi::REAL"),
    "mpi_double_precision": ("int", "frt::mpi::DOUBLE_PRECISION"),
    "mpi_logical": ("int", "frt::mpi::LOGICAL"), "mpi_sum": ("int", "frt::mpi::SUM"),
    "mpi_max": ("int", "frt::mpi::MAX"), "mpi_min": ("int", "frt::mpi::MIN"),
    "mpi_prod": ("int", "frt::mpi::PROD"),
    "mpi_status_size": ("int", "frt::mpi::STATUS_SIZE"),
    "mpi_any_source": ("int", "frt::mpi::ANY_SOURCE"),
    "mpi_double_complex": ("int", "frt::mpi::DOUBLE_COMPLEX"),
    "mpi_complex16": ("int", "frt::mpi::COMPLEX16"),
}

# run-time procedures: argument passing per position
#   buf: address (void*), val: int by value, ref: reference, ptr: typed pointer
RUNTIME_CALLS = {
    "mpi_init": ["ref"], "mpi_finalize": ["ref"], "mpi_comm_rank": ["val", "ref", "ref"],
    "mpi_comm_size": ["val", "ref", "ref"], "mpi_barrier": ["val", "ref"],
    "mpi_bcast": ["buf", "val", "val", "val", "val", "ref"],
    "mpi_allreduce": ["buf", "buf", "val", "val", "val", "val", "ref"],
    "mpi_reduce": ["buf", "buf", "val", "val", "val", "val", "val", "ref"],
    "mpi_isend": ["buf", "val", "val", "val", "val", "val", "ref", "ref"],
    "mpi_irecv": ["buf", "val", "val", "val", "val", "val", "ref", "ref"],
    "mpi_send": ["buf", "val", "val", "val", "val", "val", "ref"],
    "mpi_recv": ["buf", "val", "val", "val", "val", "val", "buf", "ref"],
    "mpi_sendrecv": ["buf", "val", "val", "val", "val", "buf", "val", "val", "val", "val", "val",
                     "buf", "ref"],
    "mpi_waitall": ["val", "ptr", "buf", "ref"], "mpi_wait": ["ref", "buf", "ref"],
    "fftw_f77_create_plan_": ["ref", "val", "val", "val"],
    "rfftwnd_f77_create_plan_": ["ref", "val", "val", "val", "val"],
    "fftw_f77_destroy_plan_": ["ref"], "rfftwnd_f77_destroy_plan_": ["ref"],
    "fftw_f77_one_": ["ref", "ptr", "ptr"],
    "rfftwnd_f77_one_real_to_complex_": ["ref", "ptr", "val"],
    "rfftwnd_f77_one_complex_to_real_": ["ref", "ptr", "val"],
    "srand": ["val"],
}

ELEMENTAL = {"abs", "sqrt", "dsqrt", "exp", "dexp", "log", "alog", "dlog", "sin", "cos", "tan",
             "dsin", "dcos", "atan", "datan", "atan2", "asin", "acos", "real", "dble", "dfloat",
             "float", "int", "nint", "mod", "max", "min", "amax1", "amin1", "max0", "min0",
             "dmax1", "dmin1", "sign", "cmplx", "dcmplx", "aimag", "conjg", "floor", "idint",
             "ifix"}
REDUCTIONS = {"sum", "maxval", "minval", "count"}
OTHER_INTRINSICS = {"cshift", "size", "trim", "mpi_wtime", "lbound", "ubound", "rand", "irand"}

CPP_KEYWORDS = set()


class Sym:
    def __init__(self, decl: Decl, kind: str, cname: str):
        self.decl = decl
        self.kind = kind          # var | param | dummy | module | result
        self.cname = cname

    @property
    def base(self):
        return self.decl.base

    @property
    def rank(self):
        return len(self.decl.dims) if self.decl.dims else 0


class Gen:
    def __init__(self, units: list, program: str):
        self.program = program
        self.units = {}
        self.modules = {}
        for u in units:
            if u.kind == "module":
                self.modules[u.name] = u
            else:
                if u.name in self.units:
                    raise FortranError(f"duplicate procedure {u.name}")
                self.units[u.name] = u
        self.tmp = 0
        self.out = []

    # ------------------------------------------------------------------
    # symbols
    def scope_of(self, u: Unit) -> dict:
        sc = {}
        for m in u.uses:
            if m == "mpi":
                continue
            if m not in self.modules:
                raise FortranError(f"{u.file}: module {m} is not available")
            for name, d in self.modules[m].decls.items():
                kind = "mparam" if "parameter" in d.attrs else "module"
                sc[name] = Sym(d, kind, f"F_{name}")
        for name, d in u.decls.items():
            if name in u.args:
                sc[name] = Sym(d, "dummy", f"F_{name}")
            elif u.kind == "function" and name == u.result:
                sc[name] = Sym(d, "result", f"F_{name}_r")
            elif "parameter" in d.attrs:
                sc[name] = Sym(d, "param", f"F_{name}")
            else:
                if name in self.units and d.dims is None and name != u.name:
                    continue  # a typed external function
                sc[name] = Sym(d, "var", f"F_{name}")
        for a in u.args:
            if a not in sc:
                if u.implicit_none:
                    raise FortranError(f"{u.file}: {u.name}: dummy {a} has no declaration")
                base = "int" if a[0] in "ijklmn" else "real"
                d = Decl(a, base)
                u.decls[a] = d
                sc[a] = Sym(d, "dummy", f"F_{a}")
        if u.kind == "function" and u.result not in sc:
            base = u.result_type or ("int" if u.result[0] in "ijklmn" else "real")
            d = Decl(u.result, base)
            sc[u.result] = Sym(d, "result", f"F_{u.result}_r")
        self._implicit_none = u.implicit_none
        return sc

    def lookup(self, name: str):
        s = self.sc.get(name)
        if s is not None:
            return s
        if name in MPI_CONST:
            return None
        if self._implicit_none:
            return None
        # implicit typing of an undeclared local
        base = "int" if name[0] in "ijklmn" else "real"
        d = Decl(name, base)
        s = Sym(d, "var", f"F_{name}")
        self.sc[name] = s
        self.implicit_locals.append(s)
        return s

    def is_array(self, name: str) -> bool:
        s = self.sc.get(name)
        return s is not None and s.rank > 0

    # ------------------------------------------------------------------
    # typing: (base, rank)
    def etype(self, e):
        if isinstance(e, Num):
            return ("int" if e.kind == "int" else "real", 0)
        if isinstance(e, Str):
            return ("char", 0)
        if isinstance(e, Logic):
            return ("logical", 0)
        if isinstance(e, Name):
            if e.name in MPI_CONST:
                return (MPI_CONST[e.name][0], 0)
            s = self.lookup(e.name)
            if s is None:
                raise FortranError(f"{self.where}: unknown name {e.name}")
            return (s.base, s.rank)
        if isinstance(e, Un):
            b, r = self.etype(e.a)
            return ("logical", r) if e.op == ".not." else (b, r)
        if isinstance(e, Bin):
            ba, ra = self.etype(e.a)
            bb, rb = self.etype(e.b)
            r = max(ra, rb)
            if e.op in ("==", "/=", "<", "<=", ">", ">=", ".and.", ".or.", ".eqv.", ".neqv."):
                return ("logical", r)
            if e.op == "//":
                return ("char", 0)
            return (self.promote(ba, bb), r)
        if isinstance(e, Ref):
            if self.is_array(e.name):
                s = self.sc[e.name]
                r = sum(1 for a in e.args if isinstance(a, Slice))
                return (s.base, r)
            return self.call_type(e)
        if isinstance(e, Ctor):
            b = self.etype(e.items[0])[0] if e.items else "real"
            for it in e.items[1:]:
                b = self.promote(b, self.etype(it)[0])
            return (b, 1)
        raise FortranError(f"{self.where}: cannot type {e}")

    @staticmethod
    def promote(a, b):
        order = ["logical", "int", "int8", "real", "complex"]
        if a == "char" or b == "char":
            return "char"
        return a if order.index(a) >= order.index(b) else b

    def args_pos(self, e: Ref):
        return [a.value if isinstance(a, Kw) else a for a in e.args]

    def call_type(self, e: Ref):
        n = e.name
        args = self.args_pos(e)
        ranks = [self.etype(a)[1] for a in args if not isinstance(a, Slice)]
        r = max(ranks) if ranks else 0
        if n in ("real", "dble", "dfloat", "float", "sqrt", "dsqrt", "exp", "dexp", "log",
                 "alog", "dlog", "sin", "cos", "tan", "dsin", "dcos", "atan", "datan", "atan2",
                 "asin", "acos", "aimag", "amax1", "amin1", "dmax1", "dmin1"):
            if n in ("sqrt", "exp", "log") and self.etype(args[0])[0] == "complex":
                return ("complex", r)
            return ("real", r)
        if n in ("int", "nint", "floor", "idint", "ifix", "max0", "min0"):
            return ("int", r)
        if n in ("abs", "mod", "sign", "max", "min"):
            b = self.etype(args[0])[0]
            for a in args[1:]:
                b = self.promote(b, self.etype(a)[0])
            if n == "abs" and b == "complex":
                b = "real"
            return (b, r)
        if n in ("cmplx", "dcmplx", "conjg"):
            return ("complex", r)
        if n == "count":
            return ("int", 0)
        if n in REDUCTIONS:
            return (self.etype(args[0])[0], 0)
        if n == "cshift":
            return self.etype(args[0])
        if n in ("size", "lbound", "ubound"):
            return ("int", 0)
        if n == "trim":
            return ("char", 0)
        if n == "mpi_wtime":
            return ("real", 0)
        if n in self.units and self.units[n].kind == "function":
            u = self.units[n]
            sc = self.scope_of_cached(u)
            return (sc[u.result].base, 0)
        s = self.sc.get(n)
        if s is not None and s.rank == 0 and n in self.units:
            return (s.base, 0)
        raise FortranError(f"{self.where}: unknown function {n}")

    def scope_of_cached(self, u):
        if not hasattr(u, "_scope"):
            save = (self.sc, self._implicit_none, self.implicit_locals)
            self.implicit_locals = []
            u._scope = self.scope_of(u)
            self.sc, self._implicit_none, self.implicit_locals = save
        return u._scope

    # ------------------------------------------------------------------
    # scalar expressions
    def num(self, e: Num) -> str:
        t = e.text
        if e.kind == "int":
            return t
        t = t.replace("d", "e")
        if t.startswith("."):
            t = "0" + t
        if "." not in t and "e" in t:
            t = t.replace("e", ".e", 1)
        return t

    def cexpr(self, e, idx=None) -> str:
        """C++ for expression e; idx: loop variables when e is array-valued
        (elemental context)."""
        if isinstance(e, Num):
            return self.num(e)
        if isinstance(e, Str):
            return "std::string(" + '"' + e.value.replace("\\", "\\\\").replace('"', '\\"') + '")'
        if isinstance(e, Logic):
            return "true" if e.value else "false"
        if isinstance(e, Name):
            if e.name in MPI_CONST:
                return MPI_CONST[e.name][1]
            s = self.lookup(e.name)
            if s is None:
                raise FortranError(f"{self.where}: unknown name {e.name}")
            if s.rank > 0:
                if idx is None:
                    raise FortranError(f"{self.where}: array {e.name} in scalar context")
                subs = ", ".join(f"{s.cname}.lb[{d}] + {idx[d]}" for d in range(s.rank))
                return f"{s.cname}({subs})"
            return s.cname
        if isinstance(e, Un):
            a = self.cexpr(e.a, idx)
            if e.op == "-":
                return f"(-{a})"
            if e.op == ".not.":
                return f"(!{a})"
            return a
        if isinstance(e, Bin):
            return self.cbin(e, idx)
        if isinstance(e, Ref):
            if self.is_array(e.name):
                return self.caref(e, idx)
            return self.ccall(e, idx)
        raise FortranError(f"{self.where}: cannot emit {e}")

    def cbin(self, e: Bin, idx) -> str:
        a = self.cexpr(e.a, idx)
        op = e.op
        if op == "**":
            ta = self.etype(e.a)[0]
            tb = self.etype(e.b)[0]
            b = self.cexpr(e.b, idx)
            if tb in ("int", "int8"):
                if ta in ("int", "int8"):
                    return f"frt::ipow({a}, {b})"
                if ta == "complex":
                    return f"std::pow({a}, (double)({b}))"
                return f"frt::rpowi({a}, {b})"
            return f"std::pow({a}, {b})"
        b = self.cexpr(e.b, idx)
        m = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=",
             ".and.": "&&", ".or.": "||", ".eqv.": "==", ".neqv.": "!=", "//": "+",
             "+": "+", "-": "-", "*": "*", "/": "/"}
        if op not in m:
            raise FortranError(f"{self.where}: operator {op}")
        ta, tb = self.etype(e.a)[0], self.etype(e.b)[0]
        if op in ("+", "-", "*", "/") and "complex" in (ta, tb):
            if ta in ("int", "int8"):
                a = f"(double)({a})"
            if tb in ("int", "int8"):
                b = f"(double)({b})"
        return f"({a} {m[op]} {b})"

    def caref(self, e: Ref, idx) -> str:
        s = self.sc[e.name]
        if len(e.args) != s.rank:
            raise FortranError(f"{self.where}: {e.name} has rank {s.rank}, {len(e.args)} subscripts")
        subs = []
        k = 0
        for d, a in enumerate(e.args):
            if isinstance(a, Slice):
                if idx is None:
                    raise FortranError(f"{self.where}: section of {e.name} in scalar context")
                lo = self.cexpr(a.lo) if a.lo is not None else f"{s.cname}.lb[{d}]"
                st = self.cexpr(a.step) if a.step is not None else "1"
                subs.append(f"({lo}) + ({st}) * {idx[k]}")
                k += 1
            else:
                if self.etype(a)[1] != 0:
                    raise FortranError(f"{self.where}: vector subscript of {e.name}")
                subs.append(self.cexpr(a))
        return f"{s.cname}({', '.join(subs)})"

    def extents(self, e) -> list:
        """C++ extent expressions of an array-valued expression."""
        if isinstance(e, Name):
            s = self.sc[e.name]
            return [f"{s.cname}.extent({d + 1})" for d in range(s.rank)]
        if isinstance(e, Ref) and self.is_array(e.name):
            s = self.sc[e.name]
            out = []
            for d, a in enumerate(e.args):
                if isinstance(a, Slice):
                    lo = self.cexpr(a.lo) if a.lo is not None else f"{s.cname}.lb[{d}]"
                    hi = self.cexpr(a.hi) if a.hi is not None else f"{s.cname}.ub[{d}]"
                    st = self.cexpr(a.step) if a.step is not None else "1"
                    out.append(f"std::max<int64_t>(0, (({hi}) - ({lo}) + ({st})) / ({st}))")
            return out
        if isinstance(e, Bin):
            if self.etype(e.a)[1]:
                return self.extents(e.a)
            return self.extents(e.b)
        if isinstance(e, Un):
            return self.extents(e.a)
        if isinstance(e, Ref):
            for a in self.args_pos(e):
                if not isinstance(a, Slice) and self.etype(a)[1]:
                    return self.extents(a)
        raise FortranError(f"{self.where}: no shape for {e}")

    # ------------------------------------------------------------------
    # intrinsic and function calls in expressions
    def ccall(self, e: Ref, idx) -> str:
        n = e.name
        args = self.args_pos(e)
        kws = {a.name: a.value for a in e.args if isinstance(a, Kw)}
        A = lambda i: self.cexpr(args[i], idx)  # noqa: E731
        T = lambda i: self.etype(args[i])[0]  # noqa: E731
        if n in ("sqrt", "dsqrt"):
            return f"std::sqrt({A(0)})"
        if n in ("exp", "dexp"):
            return f"std::exp({A(0)})"
        if n in ("log", "alog", "dlog"):
            return f"std::log({A(0)})"
        if n in ("sin", "dsin", "cos", "dcos", "tan", "asin", "acos"):
            return f"std::{n.lstrip('d') if n.startswith('d') else n}({A(0)})"
        if n in ("atan", "datan"):
            return f"std::atan({A(0)})"
        if n == "atan2":
            return f"std::atan2({A(0)}, {A(1)})"
        if n == "abs":
            return f"std::abs({A(0)})"
        if n in ("real", "dble", "dfloat", "float"):
            if T(0) == "complex":
                return f"({A(0)}).real()"
            return f"(double)({A(0)})"
        if n == "aimag":
            return f"({A(0)}).imag()"
        if n == "conjg":
            return f"std::conj({A(0)})"
        if n in ("cmplx", "dcmplx"):
            im = A(1) if len(args) > 1 else "0.0"
            return f"frt::cplx((double)({A(0)}), (double)({im}))"
        if n in ("int", "idint", "ifix"):
            if T(0) in ("int", "int8"):
                return f"(int32_t)({A(0)})"
            return f"frt::fint({A(0)})"
        if n == "nint":
            return f"frt::nint({A(0)})"
        if n == "floor":
            return f"(int32_t)std::floor({A(0)})"
        if n == "mod":
            if T(0) in ("int", "int8") and T(1) in ("int", "int8"):
                return f"frt::imod({A(0)}, {A(1)})"
            return f"frt::rmod({A(0)}, {A(1)})"
        if n == "sign":
            return f"frt::sign({A(0)}, {A(1)})"
        if n in ("max", "amax1", "max0", "dmax1"):
            return f"frt::fmaxn({', '.join(A(i) for i in range(len(args)))})"
        if n in ("min", "amin1", "min0", "dmin1"):
            return f"frt::fminn({', '.join(A(i) for i in range(len(args)))})"
        if n == "trim":
            return f"frt::trim({A(0)})"
        if n == "mpi_wtime":
            return "frt::mpi_wtime()"
        if n == "size":
            s = self.sc[args[0].name]
            if len(args) > 1:
                return f"{s.cname}.extent({self.cexpr(args[1])})"
            return f"{s.cname}.size()"
        if n in ("lbound", "ubound"):
            s = self.sc[args[0].name]
            return f"{s.cname}.{n}({self.cexpr(args[1])})"
        if n == "cshift":
            if idx is None:
                raise FortranError(f"{self.where}: cshift in scalar context")
            arr = args[0]
            shift = kws.get("shift", args[1] if len(args) > 1 else None)
            dim = kws.get("dim", args[2] if len(args) > 2 else Num("1", "int"))
            if not isinstance(dim, Num):
                raise FortranError(f"{self.where}: cshift dim must be a constant")
            d = int(dim.text) - 1
            ext = self.extents(arr)[d]
            sh = list(idx)
            sh[d] = f"frt::cshift_index({idx[d]}, {self.cexpr(shift)}, {ext})"
            return self.cexpr(arr, sh)
        if n in REDUCTIONS:
            return self.creduce(n, args[0], kws.get("mask"))
        if n in ("rand", "irand"):
            return f"frt::{n}()"
        if n in self.units:
            return self.cuser_call(e, expr=True)
        raise FortranError(f"{self.where}: unknown function {n}")

    def creduce(self, n, arr, mask) -> str:
        base, rank = self.etype(arr)
        if rank == 0:
            raise FortranError(f"{self.where}: {n} of a scalar")
        if n == "count":
            mask, base = arr, "int"
        ct = CTYPE[base]
        ext = self.extents(arr)
        iv = [f"_r{self.new_tmp()}" for _ in range(rank)]
        init = {"sum": f"{ct}(0)", "maxval": f"-std::numeric_limits<{ct}>::max()",
                "minval": f"std::numeric_limits<{ct}>::max()", "count": "0"}[n]
        loops = ""
        for d in reversed(range(rank)):
            loops += f"for (int64_t {iv[d]} = 0; {iv[d]} < {ext[d]}; ++{iv[d]}) "
        el = self.cexpr(arr, iv) if n != "count" else "1"
        upd = {"sum": f"_s = _s + {el};", "maxval": f"{{ {ct} _v = {el}; if (_v > _s) _s = _v; }}",
               "minval": f"{{ {ct} _v = {el}; if (_v < _s) _s = _v; }}",
               "count": "_s = _s + 1;"}[n]
        if mask is not None:
            upd = f"if ({self.cexpr(mask, iv)}) {upd}"
        return f"([&]() {{ {ct} _s = {init}; {loops}{{ {upd} }} return _s; }})()"

    def new_tmp(self) -> int:
        self.tmp += 1
        return self.tmp

    # ------------------------------------------------------------------
    # arguments
    def dummy_kinds(self, u: Unit) -> list:
        sc = self.scope_of_cached(u)
        out = []
        for a in u.args:
            s = sc[a]
            if s.rank == 0:
                out.append(("ref", s.base))
            elif any(d == ":" for d in s.decl.dims):
                out.append(("assumed", s.base))
            else:
                out.append(("ptr", s.base))
        return out

    def contiguous_first(self, e: Ref):
        """&first element if the section is contiguous in memory, else None."""
        s = self.sc[e.name]
        slices = [i for i, a in enumerate(e.args) if isinstance(a, Slice)]
        if not slices:
            return None
        last = slices[-1]
        for i in range(last):
            a = e.args[i]
            if not (isinstance(a, Slice) and a.lo is None and a.hi is None and a.step is None):
                return None
        if e.args[last].step is not None:
            return None
        subs = []
        for d, a in enumerate(e.args):
            if isinstance(a, Slice):
                subs.append(self.cexpr(a.lo) if a.lo is not None else f"{s.cname}.lb[{d}]")
            else:
                subs.append(self.cexpr(a))
        return f"&{s.cname}({', '.join(subs)})"

    def actual(self, a, kind, base, pre, post, allow_temp=True):
        """C++ for one actual argument."""
        if isinstance(a, Kw):
            raise FortranError(f"{self.where}: keyword arguments to procedures are not supported")
        if kind == "val":
            return self.cexpr(a)
        if kind == "ref":
            if isinstance(a, Name) and a.name not in MPI_CONST:
                s = self.lookup(a.name)
                if s is not None and s.rank == 0 and s.kind not in ("param", "mparam"):
                    return s.cname
                if s is not None and s.rank > 0:
                    return f"{s.cname}({', '.join(f'{s.cname}.lb[{d}]' for d in range(s.rank))})"
            if isinstance(a, Ref) and self.is_array(a.name) and not any(
                    isinstance(x, Slice) for x in a.args):
                return self.caref(a, None)
            if not allow_temp:
                return None
            t = f"_t{self.new_tmp()}"
            ct = CTYPE[base] if base else "auto"
            pre.append(f"{ct} {t} = {self.cexpr(a)};")
            return t
        # buf / ptr: an address
        if isinstance(a, Name) and a.name not in MPI_CONST:
            s = self.lookup(a.name)
            if s is not None and s.rank > 0:
                return f"{s.cname}.data()" if kind == "ptr" else f"(void*){s.cname}.data()"
            if s is not None and s.kind not in ("param", "mparam"):
                return f"&{s.cname}" if kind == "ptr" else f"(void*)&{s.cname}"
        if isinstance(a, Ref) and self.is_array(a.name):
            if not any(isinstance(x, Slice) for x in a.args):
                r = f"&{self.caref(a, None)}"
                return r if kind == "ptr" else f"(void*){r}"
            first = self.contiguous_first(a)
            if first is not None:
                return first if kind == "ptr" else f"(void*){first}"
            # copy-in / copy-out through a temporary
            b, rank = self.etype(a)
            ext = self.extents(a)
            t = f"_t{self.new_tmp()}"
            ct = CTYPE[b]
            pre.append(f"frt::Arr<{ct}> {t}({{{', '.join(f'{{1, {x}}}' for x in ext)}}});")
            iv = [f"_c{self.new_tmp()}" for _ in range(rank)]
            loops = "".join(f"for (int64_t {iv[d]} = 0; {iv[d]} < {ext[d]}; ++{iv[d]}) "
                            for d in reversed(range(rank)))
            tel = f"{t}({', '.join(f'1 + {v}' for v in iv)})"
            pre.append(f"{loops}{tel} = {self.cexpr(a, iv)};")
            post.append(f"{loops}{self.cexpr(a, iv)} = {tel};")
            return f"{t}.data()" if kind == "ptr" else f"(void*){t}.data()"
        # an expression or a constant: a temporary holds it
        b, rank = self.etype(a)
        if rank:
            raise FortranError(f"{self.where}: array expression as an actual argument")
        t = f"_t{self.new_tmp()}"
        pre.append(f"{CTYPE[b if kind == 'buf' else (base or b)]} {t} = {self.cexpr(a)};")
        return f"&{t}" if kind == "ptr" else f"(void*)&{t}"

    def cuser_call(self, e, expr=False):
        u = self.units[e.name]
        kinds = self.dummy_kinds(u)
        if len(e.args) != len(kinds):
            raise FortranError(f"{self.where}: {e.name} takes {len(kinds)} arguments, "
                               f"{len(e.args)} given")
        pre, post, parts = [], [], []
        for a, (k, base) in zip(e.args, kinds):
            if k == "assumed":
                if isinstance(a, Name) and self.is_array(a.name):
                    parts.append(self.sc[a.name].cname)
                    continue
                raise FortranError(f"{self.where}: section passed to an assumed-shape dummy")
            parts.append(self.actual(a, k, base, pre, post))
        call = f"F_{e.name}({', '.join(parts)})"
        if expr:
            if post:
                raise FortranError(f"{self.where}: copy-out in a function call")
            if pre:
                return f"([&]() {{ {' '.join(pre)} return {call}; }})()"
            return call
        return pre, call, post

    # ------------------------------------------------------------------
    # statements
    def emit(self, line: str, ind: int):
        self.out.append("  " * ind + line)

    def stmts(self, body, ind):
        for st in body:
            self.stmt(st, ind)

    def stmt(self, st, ind):
        self.where = st.where
        if isinstance(st, Assign):
            self.assign(st, ind)
        elif isinstance(st, Call):
            self.call(st, ind)
        elif isinstance(st, If):
            first = True
            for cond, body in st.branches:
                if cond is None:
                    self.emit("} else {", ind)
                elif first:
                    self.emit(f"if ({self.cexpr(cond)}) {{", ind)
                else:
                    self.emit(f"}} else if ({self.cexpr(cond)}) {{", ind)
                first = False
                self.stmts(body, ind + 1)
            self.emit("}", ind)
        elif isinstance(st, Do):
            v = self.lookup(st.var)
            t = self.new_tmp()
            lo, hi = self.cexpr(st.lo), self.cexpr(st.hi)
            step = self.cexpr(st.step) if st.step is not None else "1"
            self.emit(f"{{ const int32_t _lo{t} = {lo}, _hi{t} = {hi}, _st{t} = {step};", ind)
            self.emit(f"for ({v.cname} = _lo{t}; _st{t} > 0 ? {v.cname} <= _hi{t} : "
                      f"{v.cname} >= _hi{t}; {v.cname} += _st{t}) {{", ind + 1)
            self.stmts(st.body, ind + 2)
            self.emit("} }", ind + 1)
        elif isinstance(st, DoWhile):
            if st.cond is None:
                self.emit("for (;;) {", ind)
            else:
                self.emit(f"while ({self.cexpr(st.cond)}) {{", ind)
            self.stmts(st.body, ind + 1)
            self.emit("}", ind)
        elif isinstance(st, Select):
            t = self.new_tmp()
            self.emit(f"{{ const auto _sel{t} = {self.cexpr(st.expr)};", ind)
            first = True
            for vals, body in st.cases:
                if vals is None:
                    cond = "true"
                else:
                    cs = []
                    for v in vals:
                        if isinstance(v, Slice):
                            c = []
                            if v.lo is not None:
                                c.append(f"_sel{t} >= {self.cexpr(v.lo)}")
                            if v.hi is not None:
                                c.append(f"_sel{t} <= {self.cexpr(v.hi)}")
                            cs.append("(" + " && ".join(c) + ")")
                        else:
                            cs.append(f"_sel{t} == {self.cexpr(v)}")
                    cond = " || ".join(cs)
                self.emit(f"{'if' if first else '} else if'} ({cond}) {{", ind + 1)
                first = False
                self.stmts(body, ind + 2)
            if not first:
                self.emit("}", ind + 1)
            self.emit("}", ind)
        elif isinstance(st, Where):
            self.where_stmt(st, ind)
        elif isinstance(st, Simple):
            if st.what == "exit":
                self.emit("break;", ind)
            elif st.what == "cycle":
                self.emit("continue;", ind)
            elif st.what == "return":
                self.emit(f"return {self.result_c};" if self.result_c else "return;", ind)
            elif st.what == "stop":
                self.emit(f'frt::stop("{st.where}");', ind)
            elif st.what == "continue":
                self.emit(";", ind)
            else:
                self.emit(f"/* {st.arg[:60].replace('*/', '* /')} */", ind)
        elif isinstance(st, Alloc):
            for it in st.items:
                if st.dealloc:
                    self.emit(f"{self.sc[it.name].cname}.deallocate();", ind)
                else:
                    s = self.sc[it.name]
                    bs = []
                    for a in it.args:
                        if isinstance(a, Slice):
                            bs.append(f"{{{self.cexpr(a.lo)}, {self.cexpr(a.hi)}}}")
                        else:
                            bs.append(f"{{1, {self.cexpr(a)}}}")
                    self.emit(f"{s.cname}.allocate({{{', '.join(bs)}}});", ind)
        elif isinstance(st, Goto):
            self.emit(f"goto L{st.label};", ind)
        elif isinstance(st, Label):
            self.emit(f"L{st.label}:;", ind)
        else:
            raise FortranError(f"{st.where}: cannot emit {type(st).__name__}")

    def call(self, st: Call, ind):
        n = st.name
        if n in RUNTIME_CALLS:
            spec = RUNTIME_CALLS[n]
            if len(spec) != len(st.args):
                raise FortranError(f"{st.where}: {n} with {len(st.args)} arguments")
            pre, post, parts = [], [], []
            for a, k in zip(st.args, spec):
                if k == "ref" and n.endswith("_plan_") or (k == "ref" and n.startswith("fftw")) \
                        or (k == "ref" and n.startswith("rfftw")):
                    parts.append(self.actual(a, "ref", "int8", pre, post))
                elif k == "ref":
                    parts.append(self.actual(a, "ref", "int", pre, post))
                elif k == "ptr":
                    parts.append(self.actual(a, "ptr", None, pre, post))
                else:
                    parts.append(self.actual(a, k, None, pre, post))
            if n in ("mpi_irecv",) and post:
                raise FortranError(f"{st.where}: non-contiguous receive buffer")
            self.emit("{", ind)
            for p in pre:
                self.emit(p, ind + 1)
            self.emit(f"frt::{n}({', '.join(parts)});", ind + 1)
            for p in post:
                self.emit(p, ind + 1)
            self.emit("}", ind)
            return
        if n not in self.units:
            raise FortranError(f"{st.where}: call of unknown procedure {n}")
        self.called.add(n)
        pre, call, post = self.cuser_call(Ref(n, st.args))
        if pre or post:
            self.emit("{", ind)
            for p in pre:
                self.emit(p, ind + 1)
            self.emit(call + ";", ind + 1)
            for p in post:
                self.emit(p, ind + 1)
            self.emit("}", ind)
        else:
            self.emit(call + ";", ind)

    def lhs_is_array(self, lhs) -> bool:
        if isinstance(lhs, Name):
            return self.is_array(lhs.name)
        if isinstance(lhs, Ref) and self.is_array(lhs.name):
            return any(isinstance(a, Slice) for a in lhs.args)
        return False

    def convert(self, rhs_c, rb, lb):
        if lb in ("int", "int8") and rb in ("real",):
            return f"frt::fint({rhs_c})" if lb == "int" else f"(int64_t)({rhs_c})"
        if lb == "real" and rb == "complex":
            return f"({rhs_c}).real()"
        if lb == "complex" and rb != "complex":
            return f"frt::cplx((double)({rhs_c}), 0.0)"
        return rhs_c

    @staticmethod
    def names_in(e) -> set:
        out = set()
        stack = [e]
        while stack:
            x = stack.pop()
            if isinstance(x, Name):
                out.add(x.name)
            elif isinstance(x, Ref):
                out.add(x.name)
                stack.extend(x.args)
            elif isinstance(x, (Bin,)):
                stack.extend([x.a, x.b])
            elif isinstance(x, Un):
                stack.append(x.a)
            elif isinstance(x, Kw):
                stack.append(x.value)
            elif isinstance(x, Slice):
                stack.extend([v for v in (x.lo, x.hi, x.step) if v is not None])
            elif isinstance(x, Ctor):
                stack.extend(x.items)
        return out

    def assign(self, st: Assign, ind, mask=None):
        lhs, rhs = st.lhs, st.rhs
        lb = self.etype(lhs)[0]
        if not self.lhs_is_array(lhs):
            if mask is not None:
                raise FortranError(f"{st.where}: scalar assignment inside WHERE")
            if isinstance(lhs, Name) and lhs.name in self.sc and self.sc[lhs.name].kind in (
                    "param", "mparam"):
                raise FortranError(f"{st.where}: assignment to parameter {lhs.name}")
            rb = self.etype(rhs)[0]
            self.emit(f"{self.cexpr(lhs)} = {self.convert(self.cexpr(rhs), rb, lb)};", ind)
            return
        ext = self.extents(lhs)
        rank = len(ext)
        if isinstance(rhs, Ctor):
            if rank != 1:
                raise FortranError(f"{st.where}: array constructor for rank {rank}")
            self.emit("{", ind)
            for k, it in enumerate(rhs.items):
                rb = self.etype(it)[0]
                self.emit(f"{self.cexpr(lhs, [str(k)])} = {self.convert(self.cexpr(it), rb, lb)};",
                          ind + 1)
            self.emit("}", ind)
            return
        rb, rr = self.etype(rhs)
        if rr not in (0, rank):
            raise FortranError(f"{st.where}: rank mismatch {rank} = {rr}")
        lname = lhs.name
        overlap = lname in self.names_in(rhs)
        t = self.new_tmp()
        iv = [f"_i{t}_{d}" for d in range(rank)]
        ev = [f"_e{t}_{d}" for d in range(rank)]
        self.emit("{", ind)
        for d in range(rank):
            self.emit(f"const int64_t {ev[d]} = {ext[d]};", ind + 1)
        loops = "".join(f"for (int64_t {iv[d]} = 0; {iv[d]} < {ev[d]}; ++{iv[d]}) "
                        for d in reversed(range(rank)))
        relem = self.convert(self.cexpr(rhs, iv if rr else None), rb, lb)
        lelem = self.cexpr(lhs, iv)
        cond = f"if ({self.cexpr(mask, iv)}) " if mask is not None else ""
        if overlap:
            ct = CTYPE[lb]
            tmp = f"_a{t}"
            self.emit(f"frt::Arr<{ct}> {tmp}({{{', '.join(f'{{0, {e} - 1}}' for e in ev)}}});",
                      ind + 1)
            tel = f"{tmp}({', '.join(iv)})"
            self.emit(f"{loops}{{ {cond}{tel} = {relem}; }}", ind + 1)
            self.emit(f"{loops}{{ {cond}{lelem} = {tel}; }}", ind + 1)
        else:
            self.emit(f"{loops}{{ {cond}{lelem} = {relem}; }}", ind + 1)
        self.emit("}", ind)

    def where_stmt(self, st: Where, ind):
        prev = []
        for mask, body in st.branches:
            if mask is None:
                m = None
                for p in prev:
                    m = Un(".not.", p) if m is None else Bin(".and.", m, Un(".not.", p))
            else:
                m = mask
                for p in prev:
                    m = Bin(".and.", m, Un(".not.", p))
                prev.append(mask)
            for a in body:
                if not isinstance(a, Assign):
                    raise FortranError(f"{st.where}: only assignments inside WHERE")
                self.where = a.where
                self.assign(a, ind, mask=m)

    # ------------------------------------------------------------------
    # program units
    def bounds_c(self, dims) -> str:
        bs = []
        for d in dims:
            if d in (":", "*"):
                raise FortranError(f"{self.where}: deferred bounds here")
            lo, hi = d
            bs.append(f"{{{self.cexpr(lo) if lo is not None else '1'}, {self.cexpr(hi)}}}")
        return "{" + ", ".join(bs) + "}"

    def signature(self, u: Unit) -> str:
        sc = self.scope_of_cached(u)
        parts = []
        for a, (k, base) in zip(u.args, self.dummy_kinds(u)):
            ct = CTYPE[base]
            if k == "ref":
                parts.append(f"{ct}& F_{a}")
            elif k == "ptr":
                parts.append(f"{ct}* F_{a}_p")
            else:
                parts.append(f"frt::Arr<{ct}> F_{a}")
        if u.kind == "function":
            ret = CTYPE[sc[u.result].base]
        else:
            ret = "void"
        return f"{ret} F_{u.name}({', '.join(parts)})"

    def emit_unit(self, u: Unit):
        self.sc = dict(self.scope_of_cached(u))
        self._implicit_none = u.implicit_none
        self.implicit_locals = []
        self.where = f"{u.file}:{u.name}"
        self.result_c = self.sc[u.result].cname if u.kind == "function" else ""
        head = len(self.out)
        self.emit(self.signature(u) + " {", 0)
        # dummy array views, parameters, locals (in declaration order)
        body_start = len(self.out)
        for a, (k, base) in zip(u.args, self.dummy_kinds(u)):
            if k == "ptr":
                s = self.sc[a]
                dims = [d if d != "*" else (None, Num("2147483647", "int")) for d in s.decl.dims]
                if any(d == ":" for d in dims):
                    raise FortranError(f"{u.file}: {u.name}: mixed dummy shape")
                self.emit(f"frt::Arr<{CTYPE[base]}> F_{a} = frt::Arr<{CTYPE[base]}>::view("
                          f"F_{a}_p, {self.bounds_c(dims)});", 1)
        for name, d in u.decls.items():
            s = self.sc.get(name)
            if s is None or s.kind in ("dummy",):
                continue
            ct = CTYPE[d.base]
            if s.kind == "param":
                self.emit(f"const {ct} {s.cname} = {self.convert(self.cexpr(d.init), self.etype(d.init)[0], d.base)};", 1)
            elif s.kind == "result":
                self.emit(f"{ct} {s.cname} = {ct}();", 1)
            elif d.dims is None:
                static = "static " if ("save" in d.attrs or d.init is not None) else ""
                init = self.cexpr(d.init) if d.init is not None else f"{ct}()"
                self.emit(f"{static}{ct} {s.cname} = {init};", 1)
            elif "allocatable" in d.attrs:
                self.emit(f"frt::Arr<{ct}> {s.cname};", 1)
            else:
                static = "static " if "save" in d.attrs else ""
                self.emit(f"{static}frt::Arr<{ct}> {s.cname}({self.bounds_c(d.dims)});", 1)
        if u.kind == "function" and self.sc[u.result].kind == "result" and u.result not in u.decls:
            s = self.sc[u.result]
            self.emit(f"{CTYPE[s.base]} {s.cname} = {CTYPE[s.base]}();", 1)
        decl_end = len(self.out)
        self.stmts(u.body, 1)
        if u.kind == "function":
            self.emit(f"return {self.result_c};", 1)
        self.emit("}", 0)
        # implicitly typed locals discovered while emitting the body
        for s in self.implicit_locals:
            self.out.insert(decl_end, f"  {CTYPE[s.base]} {s.cname} = {CTYPE[s.base]}();")

    def module_code(self, m: Unit, ns_init: str) -> tuple:
        """(globals, init function body) of a module."""
        self.sc = {}
        for name, d in m.decls.items():
            kind = "mparam" if "parameter" in d.attrs else "module"
            self.sc[name] = Sym(d, kind, f"F_{name}")
        self._implicit_none = True
        self.implicit_locals = []
        glob, init = [], []
        for name, d in m.decls.items():
            ct = CTYPE[d.base]
            self.where = d.where
            if d.dims is None:
                glob.append(f"{ct} F_{name} = {ct}();")
                if "parameter" in d.attrs:
                    v = self.convert(self.cexpr(d.init), self.etype(d.init)[0], d.base)
                    if d.base in ("int", "int8", "real"):
                        init.append(f'F_{name} = frt::param<{ct}>("{name}", {v});')
                    else:
                        init.append(f"F_{name} = {v};")
                elif d.init is not None:
                    init.append(f"F_{name} = {self.cexpr(d.init)};")
            else:
                glob.append(f"frt::Arr<{ct}> F_{name};")
                if "allocatable" not in d.attrs:
                    init.append(f"F_{name}.allocate({self.bounds_c(d.dims)});")
                else:
                    init.append(f"F_{name}.deallocate();")
        return glob, init

    def reachable(self, roots) -> list:
        seen, order, stack = set(), [], list(roots)

        def calls_in(body, acc):
            for st in body:
                if isinstance(st, Call):
                    acc.add(st.name)
                for attr in ("body",):
                    if hasattr(st, attr) and isinstance(getattr(st, attr), list):
                        calls_in(getattr(st, attr), acc)
                if isinstance(st, If):
                    for _, b in st.branches:
                        calls_in(b, acc)
                if isinstance(st, Select):
                    for _, b in st.cases:
                        calls_in(b, acc)
                if isinstance(st, Where):
                    for _, b in st.branches:
                        calls_in(b, acc)
                for e in self._exprs_of(st):
                    for n in self.names_in(e):
                        if n in self.units and self.units[n].kind == "function":
                            acc.add(n)
        while stack:
            n = stack.pop()
            if n in seen or n not in self.units:
                continue
            seen.add(n)
            order.append(n)
            acc = set()
            calls_in(self.units[n].body, acc)
            stack.extend(sorted(acc))
        return order

    @staticmethod
    def _exprs_of(st):
        if isinstance(st, Assign):
            return [st.lhs, st.rhs]
        if isinstance(st, Call):
            return [a.value if isinstance(a, Kw) else a for a in st.args]
        if isinstance(st, If):
            return [c for c, _ in st.branches if c is not None]
        if isinstance(st, Do):
            return [x for x in (st.lo, st.hi, st.step) if x is not None]
        if isinstance(st, DoWhile):
            return [st.cond] if st.cond is not None else []
        if isinstance(st, Where):
            return [c for c, _ in st.branches if c is not None]
        return []

    def generate(self, roots, header="frt.h") -> str:
        names = self.reachable(roots)
        missing = [r for r in roots if r not in self.units]
        if missing:
            raise FortranError(f"roots not found: {missing}")
        ns = self.program
        self.out = []
        self.called = set()
        glob_all, init_all = [], []
        for mname, m in self.modules.items():
            g, i = self.module_code(m, mname)
            glob_all += g
            init_all += i
        # procedures
        protos = [self.signature(self.units[n]) + ";" for n in names]
        bodies_start = len(self.out)
        for n in names:
            self.emit_unit(self.units[n])
            self.emit("", 0)
        bodies = self.out[bodies_start:]
        src = [f"// Generated from the reference's Fortran by oracle/fortran (test infrastructure).",
               f'#include "{header}"', "#include <limits>", "#include <algorithm>", "",
               f"namespace {ns} {{", ""]
        src += glob_all + [""]
        src += ["void init_modules() {"] + ["  " + x for x in init_all] + ["}", ""]
        src += protos + [""] + bodies
        # variable table and entry points
        src += ["struct VarEntry { const char* name; int type; void* addr; int is_array; };",
                "static VarEntry vars[] = {"]
        tcode = {"int": 0, "int8": 1, "real": 2, "complex": 3, "logical": 4, "char": 5}
        for m in self.modules.values():
            for name, d in m.decls.items():
                src.append(f'  {{"{name}", {tcode[d.base]}, (void*)&F_{name}, {1 if d.dims else 0}}},')
        src += ["  {nullptr, 0, nullptr, 0}};", ""]
        noarg = [n for n in names if self.units[n].kind == "subroutine" and not self.units[n].args]
        src += ["static std::string last_error;",
                "}  // namespace " + ns, "",
                'extern "C" {',
                f"const char* {ns}_error() {{ return {ns}::last_error.c_str(); }}",
                f"void {ns}_override(const char* name, double v) {{ frt::overrides()[name] = v; }}",
                f"void {ns}_clear_overrides() {{ frt::overrides().clear(); }}",
                f"int {ns}_init() {{ try {{ {ns}::init_modules(); }} catch (std::exception& e) "
                f"{{ {ns}::last_error = e.what(); return -1; }} return 0; }}",
                f"int {ns}_call(const char* name) {{",
                "  try {"]
        for n in noarg:
            src.append(f'    if (std::string(name) == "{n}") {{ {ns}::F_{n}(); return 0; }}')
        src += [f'    {ns}::last_error = std::string("no such subroutine: ") + name; return -2;',
                f"  }} catch (std::exception& e) {{ {ns}::last_error = e.what(); return -1; }}",
                "}",
                f"int {ns}_var(const char* name, int* type, int* rank, int64_t* lb, int64_t* ub, void** data) {{",
                f"  for ({ns}::VarEntry* v = {ns}::vars; v->name; ++v) {{",
                "    if (std::string(name) != v->name) continue;",
                "    *type = v->type;",
                "    if (!v->is_array) { *rank = 0; *data = v->addr; return 0; }",
                "    void* d = nullptr; int r = 0;",
                "    switch (v->type) {",
                "      case 0: { auto* a = (frt::Arr<int32_t>*)v->addr; r = a->rank; d = a->p; for (int k = 0; k < r; ++k) { lb[k] = a->lb[k]; ub[k] = a->ub[k]; } break; }",
                "      case 1: { auto* a = (frt::Arr<int64_t>*)v->addr; r = a->rank; d = a->p; for (int k = 0; k < r; ++k) { lb[k] = a->lb[k]; ub[k] = a->ub[k]; } break; }",
                "      case 2: { auto* a = (frt::Arr<double>*)v->addr; r = a->rank; d = a->p; for (int k = 0; k < r; ++k) { lb[k] = a->lb[k]; ub[k] = a->ub[k]; } break; }",
                "      case 3: { auto* a = (frt::Arr<frt::cplx>*)v->addr; r = a->rank; d = a->p; for (int k = 0; k < r; ++k) { lb[k] = a->lb[k]; ub[k] = a->ub[k]; } break; }",
                "      case 4: { auto* a = (frt::Arr<bool>*)v->addr; r = a->rank; d = a->p; for (int k = 0; k < r; ++k) { lb[k] = a->lb[k]; ub[k] = a->ub[k]; } break; }",
                "      default: return -1;",
                "    }",
                "    *rank = r; *data = d; return d ? 0 : -3;",
                "  }",
                "  return -2;",
                "}",
                '}  // extern "C"', ""]
        return "\n".join(src)
