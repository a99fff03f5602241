"""Build recipe for a CPU build of the reference's own hot-path Fortran.

TEST INFRASTRUCTURE ONLY.  There is no Fortran compiler in this environment,
so this recipe translates the reference's Fortran 90 source files, as they
lie in the reference's Sources/ and libMaster/ directories (the reference's
root is F3D_REFERENCE_ROOT, or --reference DIR, and defaults to a directory
named "reference" beside this repository), mechanically into C and compiles that C
with gcc (-O2 -ffp-contract=off).  Only the generated C and the library go
to oracle/_ref/ (git-ignored); nothing of the reference is copied into the
repository.  The result is used to generate the golden vectors of
tests/golden/ that pin the CPU oracle (oracle/f3d_oracle.cpp), and bench.py
times it as the reference's CPU path.  On a host without the sources (the
oracle/_ref/ folder copied there, its library left behind) ``build``
compiles the translation already in oracle/_ref/.

    python oracle/ref_translate.py [--reference DIR] [--force]   -> oracle/_ref/libf3dref.so

One routine is rewritten at the source level before its translation:
libMaster/get_dbs_value_plane.f90 keeps its own statements for the time
interval and the vertical interpolation, while its netCDF calls (nf90_open,
nf90_inq_varid, nf90_get_var, nf90_close, get_dbs_property_int) become calls
of small C accessors (dbs_nt, dbs_nz, dbs_time, dbs_alt, dbs_plane) that
serve a database registered from memory (ref_dbs_set), and its word
dictionary and message strings are dropped (the caller passes the case the
dictionary would select).

The translator covers the Fortran subset of the transport path: modules
with declarations (scalars, explicit-shape and allocatable arrays, SAVE and
PARAMETER entities), subroutines with explicit-shape / assumed-size dummy
arrays, DO / DO WHILE / IF / SELECT CASE / GOTO, whole-array and section
assignments, SUM, and the intrinsics the files use.  Fortran semantics that
C does not share are made explicit:

* evaluation order and kinds: default-real literals are binary32 (so
  ``2.0/3.0`` is a binary32 quotient), mixed-kind operands are widened, a
  real raised to a small integer constant is expanded into multiplications
  as gfortran does, a real exponent calls pow();
* MAX/MIN follow gfortran 4.8: mvar = a; if (b .op. mvar .or. isnan(mvar))
  mvar = b;
* SIGN(a,b) is |a| with the sign of b; a NaN b counts as positive, which is
  the aarch64 behaviour (its default NaN is positive; x86 produces a
  negative one);
* a DO variable keeps its Fortran value after the loop;
* MPI (bcast, parallel_sum, exchange_*, collect_*), I/O (write, format,
  open, ...) and log-only calls (addtime, wriwar) are serial no-ops, as in
  the reference's serial build (Sources/Parallel.F90 without WITH_MPI);
  runend aborts.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("F3D_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
REF = os.path.join(REF_ROOT, "Sources")
DBS_PLANE_FILE = os.path.join("..", "libMaster", "get_dbs_value_plane.f90")  # relative to Sources/

MODULE_FILES = ["KindType.f90", "Numeric.f90", "Master.f90", "InpOut.f90"]
UNIT_FILES = ["setbcc.f90", "advctzc.f90", "advctx.f90", "advcty.f90", "diffz.f90", "diffx.f90",
              "diffy.f90", "wetdep.f90", "accum.f90", "cmass2d.f90", "cmass3d.f90", "finddt.f90",
              "kappa3.f90", "setvset.f90", "setpsi.f90", "setvdrydep.f90", "corvver.f90",
              "setdivu.f90", "setsrc.f90", "sizloop.f90", "meteo.f90", "source.f90", "endstep.f90",
              "setcut.f90", "ter2asl.f90", "addradialwind.f90", "divcorr.f90",
              "agrsrc.f90"]
# units from those files that are translated (others in the files are skipped)
WANTED = {"setbcc", "advctzc", "advctx", "advcty", "diffz", "diffx", "diffy", "wetdep", "accum",
          "cmass2d", "cmass3d", "finddt", "kappa3", "setvset", "vsettl", "setpsi", "get_gama",
          "setvdrydep", "corvver", "setdivu", "setsrc", "sizloop", "meteo", "source", "getc0",
          "getmem1", "getmem2", "outmem2", "setcut_fl", "standard_atm", "ter2asl",
          "addradialwind", "divcorr", "agrsrc", "agrpar", "water_phase", "get_gamas"}
NOOP_CALLS = {"bcast", "parallel_sum", "exchange_1layer", "exchange_2layer", "collect_cz",
              "collect_c", "collect_cload", "addtime", "wriwar", "flush", "reamet", "reasrc",
              "settemplume", "cpu_time"}
SKIP_STMTS = ("write", "format", "print", "open", "close", "read", "rewind", "inquire")

# module scalars supplied by the serial runtime (Sources/Parallel.F90 and
# Sources/Domain.f90 with one process)
RUNTIME_DECLS = {
    "mpime": ("int", 0), "nproc": ("int", 1), "root": ("int", 0), "group": ("int", 0),
    "grp_intra": ("int", 0), "ic_loc": ("int", 1), "nc_loc": ("int", 0), "iz_loc": ("int", 1),
    "nz_loc": ("int", 0),
}


class TranslateError(Exception):
    pass


# C accessors standing in for the netCDF calls of get_dbs_value_plane
# (name -> arguments as (name, ctype, is_array))
EXTERN_PROTOS = {
    "dbs_nt": [("nt", "int", False)],
    "dbs_nz": [("nz", "int", False)],
    "dbs_time": [("time", "int", True)],
    "dbs_alt": [("alt", "double", True)],
    "dbs_plane": [("var", "double", True), ("ialt", "int", False), ("itime", "int", False)],
}
EXTERN_C = r"""
/* an in-memory DBS for the rewritten get_dbs_value_plane: data is
   (nt, nz, ny, nx) binary32 for a 3-D word, (nt, ny, nx) or (ny, nx) for 2-D */
static struct { int nt, nz, nx, ny, rank; const int* time; const float* alt; const float* data; } dbs_mem;
void ref_dbs_set(int nt, int nz, int nx, int ny, int rank, const int* time, const float* alt,
                 const float* data) {
  dbs_mem.nt = nt; dbs_mem.nz = nz; dbs_mem.nx = nx; dbs_mem.ny = ny; dbs_mem.rank = rank;
  dbs_mem.time = time; dbs_mem.alt = alt; dbs_mem.data = data;
}
void f90_dbs_nt(int* v) { *v = dbs_mem.nt; }
void f90_dbs_nz(int* v) { *v = dbs_mem.nz; }
void f90_dbs_time(int* t) { for (int i = 0; i < dbs_mem.nt; ++i) t[i] = dbs_mem.time[i]; }
void f90_dbs_alt(double* a) { for (int i = 0; i < dbs_mem.nz; ++i) a[i] = (double)dbs_mem.alt[i]; }
void f90_dbs_plane(double* v, int* ialt, int* itime) {
  const size_t pl = (size_t)dbs_mem.nx * dbs_mem.ny;
  const float* p = dbs_mem.data;
  if (dbs_mem.rank == 1) p += (size_t)(*itime - 1) * pl;
  if (dbs_mem.rank == 2) p += ((size_t)(*itime - 1) * dbs_mem.nz + (size_t)(*ialt - 1)) * pl;
  for (size_t i = 0; i < pl; ++i) v[i] = (double)p[i];
}
"""


def rewrite_dbs_plane(lines):
    """libMaster/get_dbs_value_plane.f90 with its netCDF calls replaced by
    the C accessors of EXTERN_PROTOS, its word dictionary and message strings
    dropped, and the dictionary's case (varcase) taken as the first argument."""
    out, skip_dict = [], False
    for label, st in lines:
        low = st.strip()
        if low.startswith("subroutine get_dbs_value_plane"):
            out.append((label, "subroutine get_dbs_value_plane(varcase,timesec,z,nx,ny,var,endsec,istat)"))
            continue
        if low.startswith("use netcdf") or re.match(r"^character\b", low):
            continue
        if low.startswith("if(word(") or low.startswith("if (word("):
            skip_dict = True
        if skip_dict:
            if re.match(r"^end\s*if$", low):
                skip_dict = False
            continue
        if low.startswith("ilen =") or low.startswith("message(") or low.startswith("mymessage"):
            continue
        m = re.match(r"^call get_dbs_property_int\(fname,'(nt|nz)',(\w+),istat,message\)$", low, re.I)
        if m:
            out.append((label, f"call dbs_{m.group(1).lower()}({m.group(2)})"))
            continue
        if "nf90_open" in low or "nf90_inq_varid" in low or "nf90_close" in low:
            if label:  # keep a goto target
                out.append((label, "continue"))
            continue
        m = re.match(r"^if\s*\(\s*nf90_get_var\(ncid,(\w+),(\w+)(?:,start=\(/(.*)/\))?\)\s*/=\s*0\s*\)\s*goto\s+\d+$", low)
        if m:
            src, dst, start = m.group(1), m.group(2), m.group(3)
            if src == "timeid":
                out.append((label, f"call dbs_time({dst})"))
            elif src == "altid":
                out.append((label, f"call dbs_alt({dst})"))
            else:
                idx = [x.strip() for x in start.split(",")]
                ialt = idx[2] if len(idx) == 4 else "0"
                itime = idx[-1] if len(idx) >= 3 else "0"
                out.append((label, f"call dbs_plane({dst},{ialt},{itime})"))
            continue
        if "nf90_" in low:
            raise TranslateError(f"unhandled netCDF statement in get_dbs_value_plane: {st}")
        out.append((label, st))
    return out


# ------------------------------------------------------------------ lexing
def logical_lines(text):
    """Fortran free form -> (label, statement) with continuations joined,
    comments removed, case folded outside strings."""
    out = []
    buf = ""
    for raw in text.splitlines():
        line = raw.rstrip("\n")
        # strip comments outside strings
        s, q = [], None
        for ch in line:
            if q:
                s.append(ch)
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                s.append(ch)
            elif ch == "!":
                break
            else:
                s.append(ch)
        line = "".join(s).rstrip()
        if not line.strip():
            continue
        if line.lstrip().startswith("#"):  # preprocessor line
            continue
        cont = line.endswith("&")
        if cont:
            line = line[:-1]
        ls = line.lstrip()
        if buf and ls.startswith("&"):
            ls = ls[1:]
        buf += (" " if buf else "") + ls
        if cont:
            continue
        out.append(buf)
        buf = ""
    res = []
    for st in out:
        for part in split_semicolons(st):
            m = re.match(r"^\s*(\d+)\s+(.*)$", part)
            label, body = (m.group(1), m.group(2)) if m else (None, part.strip())
            res.append((label, fold_case(body)))
    return res


def split_semicolons(st):
    parts, cur, q = [], [], None
    for ch in st:
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
    return [p for p in parts if p.strip()]


def fold_case(s):
    out, q = [], None
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


TOKEN_RE = re.compile(r"""
    (?P<ws>\s+)
  | (?P<num>(\d+\.(?!(?:and|or|not|eq|ne|lt|le|gt|ge|true|false|eqv|neqv)\.)\d*|\.\d+|\d+)([ed][+-]?\d+)?(_\w+)?)
  | (?P<dotop>\.(and|or|not|eq|ne|lt|le|gt|ge|true|false|eqv|neqv)\.)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|==|/=|<=|>=|//|\(/|/\)|::|[-+*/(),:=<>%])
""", re.X)


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = TOKEN_RE.match(s, pos)
        if not m:
            raise TranslateError(f"cannot tokenize at {s[pos:pos + 20]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        toks.append((kind, m.group(kind)))
    toks.append(("eof", ""))
    return toks


# ------------------------------------------------------------------ parsing
class P:
    """Pratt parser over one statement's tokens."""

    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, val):
        if self.peek()[1] == val:
            self.i += 1
            return True
        return False

    def expect(self, val):
        tok = self.next()
        if tok[1] != val:
            raise TranslateError(f"expected {val!r}, got {tok[1]!r}")
        return tok

    # precedence: .eqv. < .or. < .and. < .not. < rel < // < +- < */ < unary < **
    def expr(self):
        return self.eqv()

    def eqv(self):
        a = self.lor()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.next()[1]
            a = ("bin", op, a, self.lor())
        return a

    def lor(self):
        a = self.land()
        while self.peek()[1] == ".or.":
            self.next()
            a = ("bin", ".or.", a, self.land())
        return a

    def land(self):
        a = self.lnot()
        while self.peek()[1] == ".and.":
            self.next()
            a = ("bin", ".and.", a, self.lnot())
        return a

    def lnot(self):
        if self.peek()[1] == ".not.":
            self.next()
            return ("not", self.lnot())
        return self.rel()

    REL = {"==": "==", ".eq.": "==", "/=": "!=", ".ne.": "!=", "<": "<", ".lt.": "<", "<=": "<=",
           ".le.": "<=", ">": ">", ".gt.": ">", ">=": ">=", ".ge.": ">="}

    def rel(self):
        a = self.add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.next()[1]]
            a = ("rel", op, a, self.add())
        return a

    def add(self):
        # a leading sign applies to the first term: -a*b = -(a*b)
        if self.peek()[1] in ("+", "-"):
            op = self.next()[1]
            a = self.mul()
            a = ("neg", a) if op == "-" else a
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.next()[1]
            a = ("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.power()
        while self.peek()[1] in ("*", "/"):
            op = self.next()[1]
            a = ("bin", op, a, self.power())
        return a

    def power(self):
        a = self.primary()
        if self.peek()[1] == "**":
            self.next()
            # right associative; a signed exponent is allowed (gfortran extension)
            if self.peek()[1] in ("+", "-"):
                sg = self.next()[1]
                b = self.power()
                b = ("neg", b) if sg == "-" else b
            else:
                b = self.power()
            return ("pow", a, b)
        return a

    def primary(self):
        kind, val = self.next()
        if kind == "num":
            return ("num", val)
        if kind == "str":
            return ("str", val[1:-1])
        if kind == "dotop" and val in (".true.", ".false."):
            return ("log", val == ".true.")
        if val == "(":
            e = self.expr()
            self.expect(")")
            return ("paren", e)
        if val == "(/":
            items = [self.expr()]
            while self.accept(","):
                items.append(self.expr())
            self.expect("/)")
            return ("ctor", items)
        if kind == "name":
            if self.peek()[1] == "(":
                self.next()
                args = []
                if self.peek()[1] != ")":
                    args.append(self.arg())
                    while self.accept(","):
                        args.append(self.arg())
                self.expect(")")
                return ("ref", val, args)
            return ("name", val)
        raise TranslateError(f"unexpected token {val!r}")

    def arg(self):
        # section lo:hi, :, or keyword=value (ignored keyword) or expression
        if self.peek()[1] == ":":
            self.next()
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return ("slice", None, hi)
        if self.peek()[0] == "name" and self.peek(1)[1] == "=" and self.peek(2)[1] != "=":
            self.next()
            self.next()
            return ("kw", self.expr())
        e = self.expr()
        if self.peek()[1] == ":":
            self.next()
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return ("slice", e, hi)
        return e


# ------------------------------------------------------------------ symbols
class Sym:
    def __init__(self, name, ctype, dims=None, is_arg=False, alloc=False, save=False, param=False,
                 init=None, strlen=None, module=None):
        self.name = name
        self.ctype = ctype  # int, long long, float, double, logical, char
        self.dims = dims    # list of (lo_expr, hi_expr) or None; hi '*' allowed
        self.is_arg = is_arg
        self.alloc = alloc
        self.save = save
        self.param = param
        self.init = init
        self.strlen = strlen
        self.module = module
        self.c = ("m_" if module is not None else "v_") + name


def parse_type(spec_toks, params):
    """('real', '(', 'rp', ')') -> ctype; character -> ('char', len)."""
    s = " ".join(spec_toks)
    base = spec_toks[0]
    if base == "double":
        return "double", None
    kind = None
    m = re.search(r"\(\s*(?:kind\s*=\s*)?(\w+)\s*\)", s)
    if m and base != "character":
        kv = m.group(1)
        kind = int(kv) if kv.isdigit() else params.get(kv)
    if base == "integer":
        return ("long long" if kind == 8 else "int"), None
    if base == "real":
        return ("double" if kind == 8 else "float"), None
    if base == "logical":
        return "int", None
    if base == "character":
        m = re.search(r"len\s*=\s*(\w+)", s) or re.search(r"\(\s*(\w+)\s*\)", s)
        ln = 1
        if m:
            v = m.group(1)
            ln = int(v) if v.isdigit() else params.get(v, 1)
        return "char", ln
    raise TranslateError(f"unknown type {s}")


# ------------------------------------------------------------------ codegen
def lit(val):
    """Fortran numeric literal -> (C text, ctype)."""
    m = re.match(r"^(?P<m>\d+\.\d*|\.\d+|\d+)(?P<e>[ed][+-]?\d+)?(?:_(?P<k>\w+))?$", val)
    if m is None:
        raise TranslateError(f"bad literal {val}")
    mant, exp, kind = m.group("m"), m.group("e"), m.group("k")
    is_real = "." in mant or exp is not None
    if not is_real:
        if kind in ("rp", "8"):
            return f"{mant}LL", "long long"
        return mant, "int"
    dbl = (exp is not None and exp[0] == "d") or kind in ("rp", "8")
    e = ("e" + exp[1:]) if exp else ""
    if dbl:
        return f"{mant}{e}", "double"
    return f"{mant}{e}f", "float"


RANK = {"int": 0, "long long": 1, "float": 2, "double": 3}


def promote(a, b):
    return a if RANK.get(a, 0) >= RANK.get(b, 0) else b


class Unit:
    def __init__(self, kind, name, args):
        self.kind = kind
        self.name = name
        self.args = args
        self.decls = []   # raw declaration statements
        self.body = []    # (label, stmt)
        self.uses = []


def split_units(lines, fname):
    """Top-level split into modules (declarations + contained units) and
    subroutines."""
    units, modules = [], []
    i = 0
    stack = []
    cur_mod = None
    in_contains = False
    while i < len(lines):
        label, st = lines[i]
        low = st.strip()
        m_mod = re.match(r"^module\s+(\w+)$", low)
        m_sub = re.match(r"^(?:recursive\s+)?subroutine\s+(\w+)\s*(?:\((.*)\))?$", low)
        m_fun = re.match(r"^(?:real.*|integer.*|logical.*)?\s*function\s+(\w+)", low)
        if m_mod and not low.startswith("module procedure"):
            cur_mod = Unit("module", m_mod.group(1), [])
            modules.append(cur_mod)
            in_contains = False
        elif low == "contains":
            in_contains = True
        elif re.match(r"^end\s*module", low):
            cur_mod = None
            in_contains = False
        elif m_sub:
            u = Unit("sub", m_sub.group(1), [a.strip() for a in (m_sub.group(2) or "").split(",") if a.strip()])
            u.module = cur_mod.name if cur_mod else None
            i += 1
            depth_decl = True
            while i < len(lines):
                lb, s2 = lines[i]
                l2 = s2.strip()
                if re.match(r"^end\s*subroutine", l2) or (l2 == "end"):
                    break
                if depth_decl and is_decl(l2):
                    if l2.startswith("use "):
                        u.uses.append(l2[4:].split(",")[0].strip())
                    else:
                        u.decls.append(l2)
                else:
                    if l2 not in ("implicit none",):
                        depth_decl = False
                        u.body.append((lb, l2))
                i += 1
            units.append(u)
        elif m_fun:
            # a function: a unit whose result variable is declared from its header
            hdr = re.match(r"^(real\s*(?:\([^)]*\))?|integer\s*(?:\([^)]*\))?|logical)?\s*function\s+(\w+)\s*\((.*)\)$", low)
            if not hdr or not hdr.group(1):
                raise TranslateError(f"unsupported function header: {low}")
            u = Unit("fun", hdr.group(2), [a.strip() for a in hdr.group(3).split(",") if a.strip()])
            u.module = cur_mod.name if cur_mod else None
            u.decls.append(f"{hdr.group(1)} :: {hdr.group(2)}")
            i += 1
            depth_decl = True
            while i < len(lines):
                lb, s2 = lines[i]
                l2 = s2.strip()
                if re.match(r"^end\s*function", l2) or (l2 == "end"):
                    break
                if depth_decl and is_decl(l2):
                    if l2.startswith("use "):
                        u.uses.append(l2[4:].split(",")[0].strip())
                    else:
                        u.decls.append(l2)
                else:
                    if l2 not in ("implicit none",):
                        depth_decl = False
                        u.body.append((lb, l2))
                i += 1
            units.append(u)
        elif cur_mod and not in_contains:
            if low.startswith("use "):
                cur_mod.uses.append(low[4:].split(",")[0].strip())
            elif is_decl(low):
                cur_mod.decls.append(low)
        i += 1
    return modules, units


def is_decl(s):
    return bool(re.match(r"^(integer|real|logical|character|double precision|type|use |implicit|"
                         r"save$|dimension|parameter)", s)) and not re.match(r"^real\s*\(\s*\w+\s*\)\s*=", s)


class Gen:
    def __init__(self):
        self.params = {"ip": 4, "rp": 8}
        self.globals = {}   # name -> Sym
        self.unit_syms = {}
        self.protos = {}
        self.funcs = {}  # user function -> result ctype
        self.out = []
        self.tmp = 0

    # ---------------- declarations
    def parse_decl(self, st, is_module, unit_args=(), module=None):
        st = st.strip()
        if st.startswith("implicit") or st == "save" or st.startswith("use "):
            return []
        if "::" in st:
            spec, ents = st.split("::", 1)
        else:
            m = re.match(r"^(integer\s*(\([^)]*\))?|real\s*(\([^)]*\))?|logical|double precision|"
                         r"character\s*(\([^)]*\))?)\s+(.*)$", st)
            if not m:
                raise TranslateError(f"cannot parse declaration {st}")
            spec, ents = m.group(1), m.group(5)
        attrs = [a.strip() for a in split_top(spec, ",")]
        tspec = attrs[0]
        ctype, slen = parse_type(tokens_text(tspec), self.params)
        is_param = any(a == "parameter" for a in attrs[1:])
        is_alloc = any(a == "allocatable" for a in attrs[1:])
        is_save = any(a == "save" for a in attrs[1:]) or is_module
        dim_attr = None
        for a in attrs[1:]:
            if a.startswith("dimension"):
                dim_attr = a[a.index("(") + 1:a.rindex(")")]
        syms = []
        for ent in split_top(ents, ","):
            ent = ent.strip()
            init = None
            if "=" in ent and not ent.startswith("("):
                eq = find_top(ent, "=")
                if eq >= 0:
                    init = ent[eq + 1:].strip()
                    ent = ent[:eq].strip()
            m = re.match(r"^(\w+)\s*(\((.*)\))?\s*(\*\s*\w+)?$", ent)
            if not m:
                raise TranslateError(f"cannot parse entity {ent}")
            name = m.group(1)
            dtext = m.group(3) if m.group(2) else dim_attr
            dims = None
            if dtext is not None:
                dims = []
                for dd in split_top(dtext, ","):
                    dd = dd.strip()
                    if ":" in dd:
                        lo, hi = dd.split(":", 1)
                        dims.append((lo.strip() or None, hi.strip() or None))
                    else:
                        dims.append(("1", dd))
            sym = Sym(name, ctype, dims, is_arg=name in unit_args, alloc=is_alloc, save=is_save,
                      param=is_param, init=init, strlen=slen, module=module)
            if is_param and init is not None and dims is None and ctype in ("int", "long long"):
                try:
                    self.params[name] = int(eval_int(init, self.params))
                except Exception:
                    pass
            syms.append(sym)
        return syms

    # ---------------- expressions
    def sym(self, name):
        s = self.unit_syms.get(name)
        if s is None:
            s = self.globals.get(name)
        return s

    def scal(self, s):
        return f"(*{s.c})" if (s.is_arg and s.dims is None and s.ctype != "char") else s.c

    def bounds(self, s, d):
        """(lb_text, extent_text) of dimension d."""
        if s.alloc or s.module is not None:
            return f"{s.c}_lb[{d}]", f"{s.c}_ex[{d}]"
        return f"{s.c}_lb{d}", f"{s.c}_ex{d}"

    def index(self, s, subs):
        parts = []
        for d in reversed(range(len(subs))):
            lb, ex = self.bounds(s, d)
            term = f"((long long)({subs[d]})-{lb})"
            parts.append((term, ex))
        # column major: off = i0 + ex0*(i1 + ex1*(i2 ...))
        expr = None
        for d in range(len(subs) - 1, -1, -1):
            lb, ex = self.bounds(s, d)
            term = f"((long long)({subs[d]})-{lb})"
            expr = term if expr is None else f"{term}+{ex}*({expr})"
        return expr

    def e(self, n, elem=None):
        """Returns (C text, ctype).  elem maps section dims to loop vars."""
        k = n[0]
        if k == "num":
            return lit(n[1])
        if k == "log":
            return ("1" if n[1] else "0"), "int"
        if k == "str":
            return '"' + n[1].replace('"', '\\"') + '"', "str"
        if k == "paren":
            t, ty = self.e(n[1], elem)
            return f"({t})", ty
        if k == "neg":
            t, ty = self.e(n[1], elem)
            return f"(-({t}))", ty
        if k == "not":
            t, _ = self.e(n[1], elem)
            return f"(!({t}))", "int"
        if k == "rel":
            a, ta = self.e(n[2], elem)
            b, tb = self.e(n[3], elem)
            if ta == "str" or tb == "str" or ta == "char" or tb == "char":
                eq = f"f90_streq({a},{b})"
                return (eq if n[1] == "==" else f"(!{eq})"), "int"
            return f"(({a}) {n[1]} ({b}))", "int"
        if k == "bin":
            op = n[1]
            a, ta = self.e(n[2], elem)
            b, tb = self.e(n[3], elem)
            if op == ".and.":
                return f"(({a}) && ({b}))", "int"
            if op == ".or.":
                return f"(({a}) || ({b}))", "int"
            if op in (".eqv.", ".neqv."):
                return f"((!!({a})) {'==' if op == '.eqv.' else '!='} (!!({b})))", "int"
            ty = promote(ta, tb)
            a = self.cast(a, ta, ty)
            b = self.cast(b, tb, ty)
            return f"({a} {op} {b})", ty
        if k == "pow":
            a, ta = self.e(n[1], elem)
            ex = n[2]
            if ex[0] == "num" and lit(ex[1])[1] in ("int", "long long"):
                p = int(lit(ex[1])[0].rstrip("L"))
                return self.powi(a, ta, p), ta
            b, tb = self.e(ex, elem)
            if tb in ("int", "long long") and ta in ("int", "long long"):
                return f"f90_ipow({a},{b})", "int"
            ty = promote(ta, tb)
            if ty in ("int", "long long"):
                ty = "double"
            if ty == "float":
                return f"powf({a},{b})", "float"
            return f"pow((double)({a}),(double)({b}))", "double"
        if k == "name":
            s = self.sym(n[1])
            if s is None:
                raise TranslateError(f"unknown name {n[1]} in {self.cur}")
            if s.dims is not None:
                if elem is None:
                    raise TranslateError(f"whole array {n[1]} in scalar context ({self.cur})")
                subs = [elem["vars"][d] + f"+{self.bounds(s, d)[0]}" for d in range(len(s.dims))]
                elem["used"] = True
                return f"{s.c}[{self.index(s, subs)}]", s.ctype
            if s.ctype == "char":
                return s.c, "char"
            return self.scal(s), s.ctype
        if k == "ref":
            name, args = n[1], n[2]
            s = self.sym(name)
            if s is not None and s.dims is not None:
                subs = []
                sec = 0
                for d, a in enumerate(args):
                    if a[0] == "slice":
                        if elem is None:
                            raise TranslateError(f"section of {name} in scalar context")
                        lo = self.e(a[1])[0] if a[1] is not None else self.bounds(s, d)[0]
                        subs.append(f"({lo})+{elem['vars'][sec]}")
                        sec += 1
                        elem["used"] = True
                    else:
                        subs.append(self.e(a, elem)[0])
                if s.ctype == "char":  # 1-D character array, lower bound 1
                    return f"{s.c}[(long long)({subs[0]})-1]", "char"
                return f"{s.c}[{self.index(s, subs)}]", s.ctype
            return self.intrinsic(name, args, elem)
        if k == "ctor":
            raise TranslateError("array constructor in expression")
        raise TranslateError(f"cannot translate {n}")

    def cast(self, t, fr, to):
        if fr == to or fr == "str":
            return t
        return f"(({to})({t}))"

    def powi(self, a, ta, p):
        if p == 0:
            return "1" if ta in ("int", "long long") else ("1.0f" if ta == "float" else "1.0")
        if p < 0:
            return f"(1.0/({self.powi(a, ta, -p)}))"
        # binary powering as __builtin_powi: x^2 = x*x, x^3 = (x*x)*x, x^4 = (x*x)*(x*x)
        v = self.newtmp()
        self.pre.append(f"{ta} {v} = {a};")
        res, base, q, first = None, v, p, True
        terms = []
        while q:
            if q & 1:
                terms.append(base)
            q >>= 1
            if q:
                nb = self.newtmp()
                self.pre.append(f"{ta} {nb} = {base}*{base};")
                base = nb
        res = terms[0]
        for t in terms[1:]:
            res = f"({res}*{t})"
        return res

    def newtmp(self):
        self.tmp += 1
        return f"_t{self.tmp}"

    def intrinsic(self, name, args, elem):
        if name in self.funcs:  # a user function: arguments by reference
            out = []
            for a, (pname, ptype, parr) in zip(args, self.protos[name]):
                t, ty = self.e(a, elem)
                tmp = self.newtmp()
                self.pre.append(f"{ptype} {tmp} = {self.cast(t, ty, ptype)};")
                out.append(f"&{tmp}")
            return f"f90_{name}({', '.join(out)})", self.funcs[name]
        if name == "sum":
            return self.reduce_sum(args[0])
        if name in ("maxval", "minval"):
            return self.reduce_ext(args[0], name == "maxval")
        if name == "size":
            return "0", "int"
        vals = [self.e(a, elem) for a in args if a[0] != "kw"]
        texts = [v[0] for v in vals]
        types = [v[1] for v in vals]
        if name in ("max", "min", "amax1", "amin1", "dmax1", "dmin1"):
            ty = types[0]
            for t in types[1:]:
                ty = promote(ty, t)
            fn = "max" if name.endswith("max") or name.endswith("max1") else "min"
            if name.startswith("max") or name in ("amax1", "dmax1"):
                fn = "max"
            if ty in ("int", "long long"):
                out = texts[0]
                for t in texts[1:]:
                    out = f"f90_i{fn}({out},{t})"
                return out, ty
            out = self.cast(texts[0], types[0], ty)
            for t, tt in zip(texts[1:], types[1:]):
                out = f"f90_{fn}{'f' if ty == 'float' else 'd'}({out},{self.cast(t, tt, ty)})"
            return out, ty
        if name in ("abs", "dabs"):
            if types[0] in ("int", "long long"):
                return f"abs({texts[0]})", types[0]
            return (f"fabsf({texts[0]})" if types[0] == "float" else f"fabs({texts[0]})"), types[0]
        if name == "sign":
            ty = promote(types[0], types[1])
            if ty in ("int", "long long"):
                return f"f90_isign({texts[0]},{texts[1]})", ty
            return f"f90_sign({self.cast(texts[0], types[0], 'double')},{self.cast(texts[1], types[1], 'double')})", "double"
        if name in ("sqrt", "exp", "log", "log10", "acos", "tan", "atan", "sin", "cos", "asin",
                    "dsqrt", "dexp", "dlog"):
            fn = name.lstrip("d") if name.startswith("d") and name not in ("dabs",) else name
            if types[0] == "float":
                return f"{fn}f({texts[0]})", "float"
            return f"{fn}((double)({texts[0]}))", "double"
        if name in ("int", "ifix", "idint"):
            return f"((int)({texts[0]}))", "int"
        if name in ("real", "float", "sngl"):
            return f"((float)({texts[0]}))", "float"
        if name in ("dble", "dfloat"):
            return f"((double)({texts[0]}))", "double"
        if name == "mod":
            ty = promote(types[0], types[1])
            if ty in ("int", "long long"):
                return f"(({texts[0]}) % ({texts[1]}))", ty
            return f"fmod((double)({texts[0]}),(double)({texts[1]}))", "double"
        if name == "sum":
            return self.reduce_sum(args[0])
        if name in ("trim", "adjustl"):
            return texts[0], "char"
        if name == "len_trim":
            return f"f90_len_trim({texts[0]})", "int"
        if name in ("maxval", "minval", "size"):
            return "0", "int"
        raise TranslateError(f"unknown function {name} in {self.cur}")

    def reduce_sum(self, arr):
        """SUM(array or section): sequential in array element order."""
        lo_hi = self.section_extents(arr)
        acc = self.newtmp()
        ty = self.elem_type(arr)
        lines = [f"{ty} {acc} = 0;"]
        vars_ = [self.newtmp() for _ in lo_hi]
        elem = {"vars": vars_, "used": False}
        save_pre = self.pre
        self.pre = []
        body, _ = self.e(arr, elem)
        inner = self.pre
        self.pre = save_pre
        loops = ""
        for d in reversed(range(len(lo_hi))):
            loops += f"for (long long {vars_[d]} = 0; {vars_[d]} < ({lo_hi[d][1]}); {vars_[d]}++) "
        lines.append(loops + "{ " + " ".join(inner) + f" {acc} = {acc} + {body}; }}")
        self.pre.extend(lines)
        return acc, ty

    def reduce_ext(self, arr, is_max):
        """MAXVAL / MINVAL (whole array or section) of a real array: the
        largest (smallest) element, NaN elements skipped; -HUGE (+HUGE) for
        an empty one, as gfortran returns.  MAXVAL(-a) is -MINVAL(a)."""
        if arr[0] == "neg":
            inner, ty = self.reduce_ext(arr[1], not is_max)
            return f"(-{inner})", ty
        lo_hi = self.section_extents(arr)
        acc = self.newtmp()
        ty = self.elem_type(arr)
        huge = "DBL_MAX" if ty == "double" else "FLT_MAX"
        lines = [f"{ty} {acc} = {'-' if is_max else ''}{huge};"]
        vars_ = [self.newtmp() for _ in lo_hi]
        elem = {"vars": vars_, "used": False}
        save_pre = self.pre
        self.pre = []
        body, _ = self.e(arr, elem)
        inner = self.pre
        self.pre = save_pre
        loops = ""
        for d in reversed(range(len(lo_hi))):
            loops += f"for (long long {vars_[d]} = 0; {vars_[d]} < ({lo_hi[d][1]}); {vars_[d]}++) "
        op = ">" if is_max else "<"
        lines.append(loops + "{ " + " ".join(inner) + f" if (({body}) {op} {acc}) {acc} = {body}; }}")
        self.pre.extend(lines)
        return acc, ty

    def elem_type(self, n):
        if n[0] in ("name", "ref"):
            s = self.sym(n[1])
            if s is not None:
                return s.ctype
        return "double"

    def section_extents(self, n):
        """Extents (lo, count) of the section dims of an array reference."""
        if n[0] == "name":
            s = self.sym(n[1])
            return [(self.bounds(s, d)[0], self.bounds(s, d)[1]) for d in range(len(s.dims))]
        if n[0] == "ref":
            s = self.sym(n[1])
            res = []
            for d, a in enumerate(n[2]):
                if a[0] == "slice":
                    lb, ex = self.bounds(s, d)
                    lo = self.e(a[1])[0] if a[1] is not None else lb
                    hi = self.e(a[2])[0] if a[2] is not None else f"({lb}+{ex}-1)"
                    res.append((lo, f"(({hi})-({lo})+1)"))
            return res
        raise TranslateError("section expected")

    # ---------------- statements
    def stmt(self, label, st):
        out = []
        if label:
            out.append(f"L{label}:;")
        low = st.strip()
        if not low:
            return out
        if any(re.match(rf"^{k}\b", low) for k in SKIP_STMTS):
            return out
        self.pre = []
        m = re.match(r"^if\s*\((.*)\)\s*then$", low)
        if m and balanced(m.group(1)):
            c = self.cond(m.group(1))
            self.blocks.append(1)
            return out + self.pre + [f"if ({c}) {{"]
        m = re.match(r"^else\s*if\s*\((.*)\)\s*then$", low)
        if m:
            c = self.cond(m.group(1))
            if self.pre:
                raise TranslateError("else if condition needs temporaries")
            return out + [f"}} else if ({c}) {{"]
        if low == "else":
            return out + ["} else {"]
        if re.match(r"^end\s*(if|do)$", low):
            return out + ["}" * self.blocks.pop()]
        m = re.match(r"^if\s*\(", low)
        if m:
            close = match_paren(low, low.index("("))
            cond = low[low.index("(") + 1:close]
            rest = low[close + 1:].strip()
            c = self.cond(cond)
            pre = self.pre
            inner = self.stmt(None, rest)
            return out + pre + [f"if ({c}) {{"] + inner + ["}"]
        m = re.match(r"^do\s+while\s*\((.*)\)$", low)
        if m:
            c = self.cond(m.group(1))
            if self.pre:
                raise TranslateError("do while condition needs temporaries")
            self.blocks.append(1)
            return out + [f"while ({c}) {{"]
        m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", low)
        if m:
            var = m.group(1)
            parts = split_top(m.group(2), ",")
            a = self.expr_text(parts[0])
            b = self.expr_text(parts[1])
            v = self.scalar_lhs(var)
            hi = self.newtmp()
            self.blocks.append(2)
            if len(parts) > 2:
                sstep = self.expr_text(parts[2])
                stp = self.newtmp()
                return out + self.pre + [f"{{ long long {hi} = {b}; long long {stp} = {sstep};",
                                         f"for ({v} = {a}; ({stp} > 0) ? ({v} <= {hi}) : ({v} >= {hi}); {v} += {stp}) {{"]
            return out + self.pre + [f"{{ long long {hi} = {b};", f"for ({v} = {a}; {v} <= {hi}; {v}++) {{"]
        if low == "enddo" or low == "end do":
            return out + ["}" * self.blocks.pop()]
        m = re.match(r"^goto\s+(\d+)$", low) or re.match(r"^go\s+to\s+(\d+)$", low)
        if m:
            return out + [f"goto L{m.group(1)};"]
        if low == "continue":
            return out
        if low == "return":
            return out + ["goto L_end;"]
        if low in ("exit",):
            return out + ["break;"]
        if low in ("cycle",):
            return out + ["continue;"]
        if low.startswith("stop"):
            return out + ['f90_runend("stop");']
        m = re.match(r"^select\s+case\s*\((.*)\)$", low)
        if m:
            self.select_stack.append(m.group(1))
            self.select_first.append(True)
            return out + ["{"]
        m = re.match(r"^case\s*\((.*)\)$", low)
        if m:
            subj = self.expr_text(self.select_stack[-1])
            val = self.expr_text(m.group(1))
            cond = f"f90_streq({subj},{val})" if val.startswith('"') else f"(({subj}) == ({val}))"
            first = self.select_first[-1]
            self.select_first[-1] = False
            return out + ([f"if ({cond}) {{"] if first else [f"}} else if ({cond}) {{"])
        if low == "case default":
            return out + ["} else {"]
        if re.match(r"^end\s*select$", low):
            self.select_stack.pop()
            first = self.select_first.pop()
            return out + (["}"] if first else ["}", "}"])
        m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?$", low)
        if m:
            return out + self.call(m.group(1), m.group(3) or "")
        m = re.match(r"^allocate\s*\((.*)\)$", low)
        if m:
            return out + self.allocate(m.group(1))
        m = re.match(r"^deallocate\s*\((.*)\)$", low)
        if m:
            res = []
            for ent in split_top(m.group(1), ","):
                ent = ent.strip()
                if ent.startswith("stat"):
                    continue
                cn = self.sym(ent).c
                res.append(f"free({cn}); {cn} = 0;")
            return out + res
        eq = find_top(low, "=")
        if eq > 0:
            return out + self.assign(low[:eq].strip(), low[eq + 1:].strip())
        raise TranslateError(f"cannot translate statement {low!r} in {self.cur}")

    def cond(self, text):
        return self.expr_text(text)

    def expr_text(self, text):
        p = P(tokenize(text))
        n = p.expr()
        if p.peek()[0] != "eof":
            raise TranslateError(f"trailing tokens in {text!r}")
        return self.e(n)[0]

    def scalar_lhs(self, name):
        s = self.sym(name)
        if s is None:
            raise TranslateError(f"unknown variable {name} in {self.cur}")
        return self.scal(s)

    def assign(self, lhs, rhs):
        p = P(tokenize(lhs))
        ln = p.primary()
        rp_ = P(tokenize(rhs))
        rn = rp_.expr()
        s = self.sym(ln[1])
        if s is None:
            raise TranslateError(f"assignment to unknown {ln[1]} in {self.cur}")
        if s.ctype == "char":
            src, _ = self.e(rn)
            tgt = s.c if ln[0] == "name" else self.e(ln)[0]
            return self.pre + [f"f90_strset({tgt}, {s.strlen}, {src});"]
        whole = ln[0] == "name" and s.dims is not None
        has_sec = ln[0] == "ref" and any(a[0] == "slice" for a in ln[2])
        if not whole and not has_sec:
            t, tt = self.e(ln)
            r, tr = self.e(rn)
            return self.pre + [f"{t} = {self.cast(r, tr, s.ctype)};"]
        ext = self.section_extents(ln)
        vars_ = [self.newtmp() for _ in ext]
        elem = {"vars": vars_, "used": False}
        t, _ = self.e(ln, elem)
        pre_l = self.pre
        self.pre = []
        r, tr = self.e(rn, elem)
        pre_r = self.pre
        loops = ""
        for d in reversed(range(len(ext))):
            loops += f"for (long long {vars_[d]} = 0; {vars_[d]} < ({ext[d][1]}); {vars_[d]}++) "
        return pre_l + [loops + "{ " + " ".join(pre_r) + f" {t} = {self.cast(r, tr, s.ctype)}; }}"]

    def allocate(self, text):
        res = []
        for ent in split_top(text, ","):
            ent = ent.strip()
            if ent.startswith("stat"):
                continue
            m = re.match(r"^(\w+)\s*\((.*)\)$", ent)
            name, dims = m.group(1), split_top(m.group(2), ",")
            s = self.sym(name)
            name = s.c
            tot = []
            for d, dd in enumerate(dims):
                if ":" in dd:
                    lo, hi = dd.split(":", 1)
                else:
                    lo, hi = "1", dd
                lo_t = self.expr_text(lo)
                hi_t = self.expr_text(hi)
                res.append(f"{name}_lb[{d}] = {lo_t}; {name}_ex[{d}] = ({hi_t}) - ({lo_t}) + 1; "
                           f"if ({name}_ex[{d}] < 0) {name}_ex[{d}] = 0;")
                tot.append(f"{name}_ex[{d}]")
            res.append(f"{name} = ({s.ctype}*)calloc((size_t)({'*'.join(tot)}) + 1, sizeof({s.ctype}));")
        return self.pre + res

    def call(self, name, argtext):
        if name in NOOP_CALLS or name.startswith("mpi_"):
            return []
        if name == "runend":
            return ['f90_runend("runend");']
        if name not in self.protos:
            raise TranslateError(f"call to untranslated routine {name} in {self.cur}")
        pargs = self.protos[name]
        args = split_top(argtext, ",") if argtext.strip() else []
        out_args = []
        for a, (pname, ptype, parr) in zip(args, pargs):
            p = P(tokenize(a))
            n = p.expr()
            if n[0] == "name":
                s = self.sym(n[1])
                if s.dims is not None or s.ctype == "char":
                    out_args.append(s.c)
                elif s.is_arg:
                    out_args.append(s.c)
                else:
                    out_args.append(f"&{s.c}")
                continue
            if n[0] == "ref" and self.sym(n[1]) is not None and self.sym(n[1]).dims is not None:
                if any(x[0] == "slice" for x in n[2]):
                    raise TranslateError(f"section argument in call {name}")
                t, _ = self.e(n)
                out_args.append(f"&{t}")
                continue
            t, ty = self.e(n)
            tmp = self.newtmp()
            self.pre.append(f"{ptype} {tmp} = {self.cast(t, ty, ptype)};")
            out_args.append(f"&{tmp}")
        return self.pre + [f"f90_{name}({', '.join(out_args)});"]

    # ---------------- units
    def emit_module_vars(self, mod):
        for st in mod.decls:
            for s in self.parse_decl(st, True, module=mod.name):
                if s.name in self.globals:
                    continue
                self.globals[s.name] = s
                self.out.append(self.global_decl(s))

    def global_decl(self, s):
        ty = s.ctype
        if ty == "char":
            if s.dims:
                if s.dims[0][1] is None:  # deferred shape: not used on this path
                    return f"/* {s.c}: deferred-shape character array (unused) */"
                n = eval_int(s.dims[0][1], self.params)
                return f"char {s.c}[{n}][{s.strlen + 1}];"
            return f"char {s.c}[{s.strlen + 1}];"
        if s.dims is not None:
            if s.alloc or s.dims[0][0] is None:
                r = len(s.dims)
                return f"{ty}* {s.c} = 0; long long {s.c}_lb[{r}], {s.c}_ex[{r}];"
            # explicit-shape module array
            lbs, exs, tot = [], [], []
            for d, (lo, hi) in enumerate(s.dims):
                lo_v = eval_int(lo, self.params)
                hi_v = eval_int(hi, self.params)
                lbs.append(str(lo_v))
                exs.append(str(hi_v - lo_v + 1))
                tot.append(hi_v - lo_v + 1)
            n = 1
            for t in tot:
                n *= t
            r = len(s.dims)
            return (f"{ty} {s.c}[{n}]; long long {s.c}_lb[{r}] = {{{','.join(lbs)}}}, "
                    f"{s.c}_ex[{r}] = {{{','.join(exs)}}};")
        init = ""
        if s.init is not None and not s.init.startswith("(/"):
            self.cur = f"module {s.module}"
            self.unit_syms = {}
            self.pre = []
            init = f" = {self.expr_text(s.init)}"
        if s.param:
            return f"static const {ty} {s.c}{init};"
        return f"{ty} {s.c}{init};"

    def proto(self, u):
        syms = {}
        for st in u.decls:
            for s in self.parse_decl(st, False, u.args):
                syms[s.name] = s
        args = []
        for a in u.args:
            s = syms.get(a)
            if s is None:
                raise TranslateError(f"undeclared argument {a} of {u.name}")
            args.append((a, s.ctype if s.ctype != "char" else "char", s.dims is not None))
        self.protos[u.name] = args
        return syms

    def emit_unit(self, u):
        self.cur = u.name
        syms = self.proto(u)
        self.unit_syms = dict(syms)
        self.select_stack, self.select_first = [], []
        self.blocks = []
        params = []
        for a in u.args:
            s = syms[a]
            params.append(f"{'char' if s.ctype == 'char' else s.ctype}* {s.c}")
        rtype = syms[u.name].ctype if u.kind == "fun" else "void"
        body = [f"{rtype} f90_{u.name}({', '.join(params) if params else 'void'}) {{"]
        # locals
        for name, s in syms.items():
            if s.is_arg:
                continue
            st = "static " if (s.save or s.init is not None and not s.param) else ""
            if s.param:
                st = "const "
            if s.dims is not None:
                if s.alloc:
                    r = len(s.dims)
                    body.append(f"  {st}{s.ctype}* {s.c} = 0; {st}long long {s.c}_lb[{r}], {s.c}_ex[{r}];")
                else:
                    dims = [(eval_int(lo, self.params), eval_int(hi, self.params)) for lo, hi in s.dims]
                    n = 1
                    for lo, hi in dims:
                        n *= hi - lo + 1
                    body.append(f"  {st}{s.ctype} {s.c}[{n}];")
                    for d, (lo, hi) in enumerate(dims):
                        body.append(f"  const long long {s.c}_lb{d} = {lo}, {s.c}_ex{d} = {hi - lo + 1};")
                continue
            if s.ctype == "char":
                body.append(f"  char {s.c}[{s.strlen + 1}];")
                continue
            init = ""
            if s.init is not None:
                self.pre = []
                init = f" = {self.expr_text(s.init)}"
            elif not s.param:
                init = " = 0"
            body.append(f"  {st}{s.ctype} {s.c}{init};")
        # dummy array bounds (evaluated at entry, Fortran explicit shape)
        for a in u.args:
            s = syms[a]
            if s.dims is None:
                continue
            for d, (lo, hi) in enumerate(s.dims):
                self.pre = []
                lo_t = self.expr_text(lo) if lo else "1"
                if hi in (None, "*"):
                    ex_t = "0"
                else:
                    ex_t = f"(({self.expr_text(hi)}) - ({lo_t}) + 1)"
                body.append(f"  const long long {s.c}_lb{d} = {lo_t}, {s.c}_ex{d} = {ex_t};")
                body.append(f"  (void){s.c}_ex{d};")
        for label, st in u.body:
            try:
                lines = self.stmt(label, st)
            except TranslateError as e:
                raise TranslateError(f"{u.name}: {e}")
            body.extend("  " + ln for ln in lines)
        body.append("  L_end:;")
        if u.kind == "fun":
            body.append(f"  return {syms[u.name].c};")
        body.append("}")
        self.out.extend(body)


# ------------------------------------------------------------------ helpers
def tokens_text(s):
    return [t[1] for t in tokenize(s) if t[0] != "eof"]


def split_top(s, sep):
    parts, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


def find_top(s, ch):
    depth, q = 0, None
    for i, c in enumerate(s):
        if q:
            if c == q:
                q = None
            continue
        if c in "'\"":
            q = c
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        elif c == ch and depth == 0:
            if ch == "=" and (s[i + 1:i + 2] == "=" or s[i - 1:i] in "<>/="):
                continue
            return i
    return -1


def match_paren(s, i):
    depth = 0
    for j in range(i, len(s)):
        if s[j] == "(":
            depth += 1
        elif s[j] == ")":
            depth -= 1
            if depth == 0:
                return j
    raise TranslateError("unbalanced parentheses")


def balanced(s):
    d = 0
    for c in s:
        d += c == "("
        d -= c == ")"
        if d < 0:
            return False
    return d == 0


def eval_int(text, params):
    text = text.strip()
    if text.isdigit():
        return int(text)
    expr = re.sub(r"[a-z_]\w*", lambda m: str(params[m.group(0)]), text)
    return int(eval(expr, {}, {}))


RUNTIME_C = r"""
#include <math.h>
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
/* gfortran 4.8 MAX/MIN on reals; SIGN with a NaN b counted as positive. */
static inline double f90_maxd(double a, double b) { return (b > a || isnan(a)) ? b : a; }
static inline double f90_mind(double a, double b) { return (b < a || isnan(a)) ? b : a; }
static inline float f90_maxf(float a, float b) { return (b > a || isnan(a)) ? b : a; }
static inline float f90_minf(float a, float b) { return (b < a || isnan(a)) ? b : a; }
static inline long long f90_imax(long long a, long long b) { return b > a ? b : a; }
static inline long long f90_imin(long long a, long long b) { return b < a ? b : a; }
static inline double f90_sign(double a, double b) {
  double m = fabs(a); if (isnan(b)) return m; return signbit(b) ? -m : m; }
static inline long long f90_isign(long long a, long long b) { long long m = a < 0 ? -a : a; return b < 0 ? -m : m; }
static inline long long f90_ipow(long long a, long long b) { long long r = 1; while (b-- > 0) r *= a; return r; }
static int f90_len_trim(const char* s) { int n = (int)strlen(s); while (n > 0 && s[n-1] == ' ') --n; return n; }
static int f90_streq(const char* a, const char* b) {
  int la = f90_len_trim(a), lb = f90_len_trim(b);
  return la == lb && strncmp(a, b, (size_t)la) == 0; }
static void f90_strset(char* dst, int len, const char* src) {
  int n = (int)strlen(src); if (n > len) n = len; memcpy(dst, src, (size_t)n);
  for (int i = n; i < len; ++i) dst[i] = ' '; dst[len] = 0; }
int f90_error = 0;
static void f90_runend(const char* m) { fprintf(stderr, "translated reference: %s\n", m); abort(); }
"""


def translate(ref_dir=REF) -> str:
    g = Gen()
    g.out.append(RUNTIME_C)
    g.out.append(EXTERN_C)
    for name, args in EXTERN_PROTOS.items():
        g.protos[name] = list(args)
    # serial runtime of Parallel/Domain
    for name, (ty, val) in RUNTIME_DECLS.items():
        g.globals[name] = Sym(name, ty, module="runtime")
        g.out.append(f"{ty} m_{name} = {val};")
    all_units = []
    for f in MODULE_FILES:
        text = open(os.path.join(ref_dir, f), encoding="latin-1").read()
        mods, units = split_units(logical_lines(text), f)
        for m in mods:
            g.emit_module_vars(m)
        all_units += [u for u in units if u.name in WANTED]
    for f in UNIT_FILES:
        text = open(os.path.join(ref_dir, f), encoding="latin-1").read()
        mods, units = split_units(logical_lines(text), f)
        all_units += [u for u in units if u.name in WANTED]
    text = open(os.path.join(ref_dir, DBS_PLANE_FILE), encoding="latin-1").read()
    mods, units = split_units(rewrite_dbs_plane(logical_lines(text)), "get_dbs_value_plane.f90")
    all_units += [u for u in units if u.name == "get_dbs_value_plane"]
    emit_units(g, all_units)
    return "\n".join(g.out) + "\n"


def emit_units(g, all_units):
    for u in all_units:
        g.unit_syms = {}
        syms = g.proto(u)
        if u.kind == "fun":
            g.funcs[u.name] = syms[u.name].ctype
    # prototypes
    for u in all_units:
        params = []
        for a, ty, arr in g.protos[u.name]:
            params.append(f"{ty}* v_{a}")
        rtype = g.funcs.get(u.name, "void") if u.kind == "fun" else "void"
        g.out.append(f"{rtype} f90_{u.name}({', '.join(params) if params else 'void'});")
    for u in all_units:
        g.emit_unit(u)


# The pre-processing utilities whose generators the input layer restates:
# each is a program of its own with its own Master module, so each becomes a
# library of its own.  name -> (directory under Utilities/, module files,
# unit files, wanted units)
UTILITIES = {
    "settgsd": ("SetTgsd", ["KindType.f90", "Master.f90"], ["setfrac.f90"],
                {"setfrac", "m0_fi_gaussian", "fer", "getmem"}),
    "setsrc": ("SetSrc", ["KindType.f90", "Master.f90"], ["solvesuzuki.f90", "getsrc.f90"],
               {"solvesuzuki", "getsrc", "getshape"}),
    "setdbs": ("SetDbs", ["KindType.f90"], ["get_par_ABL.f90"], {"get_par_abl"}),
}


def translate_utility(name, ref_root=REF_ROOT) -> str:
    sub, module_files, unit_files, wanted = UTILITIES[name]
    d = os.path.join(ref_root, "Utilities", sub)
    g = Gen()
    g.out.append(RUNTIME_C)
    for rname, (ty, val) in RUNTIME_DECLS.items():
        g.globals[rname] = Sym(rname, ty, module="runtime")
        g.out.append(f"{ty} m_{rname} = {val};")
    all_units = []
    for f in module_files:
        text = open(os.path.join(d, f), encoding="latin-1").read()
        mods, units = split_units(logical_lines(text), f)
        for m in mods:
            g.emit_module_vars(m)
        all_units += [u for u in units if u.name in wanted]
    for f in unit_files:
        text = open(os.path.join(d, f), encoding="latin-1").read()
        mods, units = split_units(logical_lines(text), f)
        all_units += [u for u in units if u.name in wanted]
    emit_units(g, all_units)
    return "\n".join(g.out) + "\n"


def build_utility(name, force=False, ref_root=REF_ROOT) -> str:
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, f"lib{name}.so")
    if os.path.exists(lib) and not force:
        return lib
    csrc = os.path.join(OUT, f"{name}.c")
    with open(csrc, "w") as f:
        f.write(translate_utility(name, ref_root))
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=gnu11",
           "-w", "-o", lib, csrc, "-lm"]
    subprocess.run(cmd, check=True)
    return lib


def build(force=False, ref_dir=REF) -> str:
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libf3dref.so")
    if os.path.exists(lib) and not force:
        return lib
    csrc = os.path.join(OUT, "f3dref.c")
    if os.path.isdir(ref_dir):
        with open(csrc, "w") as f:
            f.write(translate(ref_dir))
    elif not os.path.exists(csrc):
        raise FileNotFoundError(f"reference sources not found at {ref_dir} and no translation in {OUT}")
    # else: compile the translation made where the sources were mounted
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=gnu11",
           "-w", "-o", lib, csrc, "-lm"]
    subprocess.run(cmd, check=True)
    return lib


if __name__ == "__main__":
    args = sys.argv[1:]
    ref = REF
    if "--reference" in args:
        ref = os.path.join(args[args.index("--reference") + 1], "Sources")
    print(build(force="--force" in args, ref_dir=ref))
    root = os.path.dirname(ref)
    for name in UTILITIES:
        print(build_utility(name, force="--force" in args, ref_root=root))
