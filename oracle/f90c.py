"""Fortran-90 subset to C translator for the reference's RTM modules.

Test infrastructure (part of the oracle), never part of the product.

The reference's RTM and Born path lives in Fortran-90 modules
(2d_rtm_restart/Src_working/{model-mod,source-mod,abc-mod,rtmlib-modF,
rtmlib-mod,image-mod-rtm,rtm-mod-adj}.f90) and no Fortran compiler exists in
this image.  This script reads those files as they are and emits one C
translation unit that executes them statement by statement, so that the
oracle can be checked against an execution of the reference's own code rather
than only against a restatement of it.  The C adjoint recursion those modules
call (rtm_op3_c_, rtmlib-modC.c) is the reference's C, compiled unchanged.

Semantics kept:
- default REAL is IEEE binary32 and every operation is evaluated in binary32
  in the source's grouping (the generated C is fully parenthesised from the
  parse tree and compiled with -ffp-contract=off, no fast-math), as a Fortran
  build without fused multiply-adds evaluates it; EXP of a REAL calls expf;
- arrays are column-major with lower bound 1; explicit-shape dummies are
  sequence-associated with the actual's first element (so a section such as
  V(:,:,it) passes the plane), assumed-shape dummies and POINTER variables
  carry the actual's extents;
- scalar dummies are passed by reference, expressions as temporaries;
- array assignments evaluate the whole right-hand side before storing when
  the left-hand array appears on the right with other subscripts.

Deliberate departures, none of which changes a computed value:
- SEPlib output (to_history, sep_write), WRITE/CLOSE and the timers are
  dropped; an IF whose body is only such output is dropped with its
  condition (the progress bar's MOD(it, nt/59) divides by zero for nt < 59);
- the executable WRITE statements inside rtmlib-modF.f90's INTERFACE body
  are ignored;
- ALLOCATE of an already allocated array frees it first (the reference
  allocates once per process; the tests call it repeatedly), and allocations
  are zero-filled;
- a hook call can be requested before chosen CALL statements so that the
  driver can copy intermediate module state (the forward wavefield) out.

Only the procedures reachable from the requested entry points are emitted;
anything outside the supported subset inside them is an error.

--set pml translates the split-field PML Born modelling program of
2d_rtm_restart/working_Src (born-mod.f90 with bornlib-mod.f90, pml-mod.f90,
source-mod.f90, seis-mod-born.f90, snap-mod-born.f90; entries elastic_init
and elastic_op) into refpml.c, with the two six-argument source routines
that born-mod.f90 calls taken from pml_source_shim.f90 (source-mod.f90
defines them with four arguments).  LOG and NINT are supported for it.
"""
import argparse
import os
import re
import sys

MODULE_FILES = ["model-mod.f90", "source-mod.f90", "abc-mod.f90", "rtmlib-modF.f90",
                "rtmlib-mod.f90", "image-mod-rtm.f90", "rtm-mod-adj.f90"]
ENTRIES = [("rtm_mod_adj", "rtm_init"), ("rtm_mod_adj", "rtm_op"), ("rtm_mod_adj", "rtm_op2")]
# calls into libraries that are not part of the computation (SEPlib I/O, OpenMP timers)
STUB_CALLS = {"to_history", "sep_write", "sep_read", "from_param", "from_history", "sep_init", "sep_close"}
STUB_FUNCS = {"omp_get_wtime": ("double", "0.0")}
HOOKS = {("rtm_op2", "image_init"): "ref90_hook_forward"}

CTYPE = {"real": "float", "double": "double", "int": "int", "logical": "int"}
ATYPE = {"real": "rarr", "double": "darr", "int": "iarr", "logical": "iarr"}


class F90Error(Exception):
    pass


# --------------------------------------------------------------------------- reading
def strip_comment(line):
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:i]
    return line


def read_statements(path):
    """Free-form source -> list of (line number, lower-cased statement)."""
    out, buf, start = [], "", 0
    with open(path, encoding="latin-1") as f:
        for no, raw in enumerate(f, 1):
            t = strip_comment(raw.rstrip("\n")).strip()
            if not t:
                continue
            if buf:
                if t.startswith("&"):
                    t = t[1:]
                buf += " " + t
            else:
                buf, start = t, no
            if buf.endswith("&"):
                buf = buf[:-1]
                continue
            for part in split_top(buf, ";"):
                if part.strip():
                    out.append((start, part.strip().lower()))
            buf = ""
    return out


def split_top(s, sep=","):
    """Split on sep outside parentheses and quotes."""
    parts, depth, q, cur = [], 0, None, ""
    for ch in s:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == sep and depth == 0:
            parts.append(cur)
            cur = ""
            continue
        cur += ch
    parts.append(cur)
    return parts


def match_paren(s, i):
    """Index of the parenthesis closing the one at s[i]."""
    depth, q = 0, None
    for j in range(i, len(s)):
        ch = s[j]
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return j
    raise F90Error("unbalanced parentheses: " + s)


# --------------------------------------------------------------------------- expressions
TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<num>(\d+\.(?!(and|or|not|eq|ne|lt|le|gt|ge|true|false|eqv|neqv)\.)\d*|\.\d+|\d+)([ed][+-]?\d+)?(_\w+)?)
  | (?P<dotop>\.(and|or|not|eq|ne|lt|le|gt|ge|true|false|eqv|neqv)\.)
  | (?P<name>[a-z_]\w*)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<op>\*\*|==|/=|<=|>=|=>|[-+*/(),:<>=%])
""", re.X)


def tokenize(s):
    toks, i = [], 0
    while i < len(s):
        m = TOKEN.match(s, i)
        if not m:
            raise F90Error("cannot tokenize %r at %d" % (s, i))
        i = m.end()
        k = m.lastgroup
        if k == "ws":
            continue
        toks.append((k, m.group(k)))
    toks.append(("end", None))
    return toks


class P:
    """Recursive-descent parser for Fortran expressions."""
    REL = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=",
           ".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}

    def __init__(self, s):
        self.t = tokenize(s)
        self.i = 0
        self.s = s

    def peek(self):
        return self.t[self.i]

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1] != val:
            raise F90Error("expected %r in %r" % (val, self.s))
        self.i += 1
        return tok

    def parse(self):
        e = self.expr()
        if self.peek()[0] != "end":
            raise F90Error("trailing tokens in %r" % self.s)
        return e

    def expr(self):
        e = self.and_()
        while self.peek()[1] == ".or.":
            self.take()
            e = ("bin", "||", e, self.and_())
        return e

    def and_(self):
        e = self.not_()
        while self.peek()[1] == ".and.":
            self.take()
            e = ("bin", "&&", e, self.not_())
        return e

    def not_(self):
        if self.peek()[1] == ".not.":
            self.take()
            return ("un", "!", self.not_())
        return self.rel()

    def rel(self):
        e = self.add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.take()[1]]
            e = ("bin", op, e, self.add())
        return e

    def add(self):
        if self.peek()[1] in ("-", "+"):
            op = self.take()[1]
            e = self.mul()
            e = ("un", "-", e) if op == "-" else e
        else:
            e = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            e = ("bin", op, e, self.mul())
        return e

    def mul(self):
        e = self.pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            e = ("bin", op, e, self.pow())
        return e

    def pow(self):
        e = self.prim()
        if self.peek()[1] == "**":
            self.take()
            e = ("pow", e, self.pow() if self.peek()[1] not in ("-", "+") else self.add())
        return e

    def prim(self):
        k, v = self.take()
        if k == "num":
            return num_node(v)
        if k == "dotop" and v in (".true.", ".false."):
            return ("lit", "logical", "1" if v == ".true." else "0")
        if k == "str":
            return ("str", v)
        if v == "(":
            e = self.expr()
            self.take(")")
            return ("par", e)
        if k == "name":
            if self.peek()[1] == "(":
                self.take("(")
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.arg())
                        if self.peek()[1] == ",":
                            self.take()
                            continue
                        break
                self.take(")")
                return ("ref", v, args)
            return ("name", v)
        raise F90Error("unexpected %r in %r" % (v, self.s))

    def arg(self):
        """An actual argument or subscript: expression, ':' range, or keyword=expr."""
        if self.peek()[0] == "name" and self.t[self.i + 1][1] == "=":
            name = self.take()[1]
            self.take("=")
            return ("kw", name, self.expr())
        lo = hi = None
        if self.peek()[1] != ":":
            lo = self.expr()
            if self.peek()[1] != ":":
                return lo
        self.take(":")
        if self.peek()[1] not in (",", ")"):
            hi = self.expr()
        if self.peek()[1] == ":":
            raise F90Error("strided sections are not supported: " + self.s)
        return ("range", lo, hi)


def num_node(v):
    kind = None
    if "_" in v:
        v, kind = v.split("_", 1)
    if re.fullmatch(r"\d+", v):
        return ("lit", "int", v)
    typ = "double" if ("d" in v or kind in ("8", "dp", "c_double")) else "real"
    v = v.replace("d", "e")
    if v.startswith("."):
        v = "0" + v
    mant = re.split(r"e", v)[0]
    if "." not in mant:
        v = mant + ".0" + v[len(mant):]
    elif v.endswith(".") or mant.endswith("."):
        v = mant + "0" + v[len(mant):]
    return ("lit", typ, v + ("f" if typ == "real" else ""))


def parse_expr(s):
    return P(s).parse()


# --------------------------------------------------------------------------- program structure
class Sym:
    def __init__(self, name, typ, dims, attrs, init, storage):
        self.name, self.typ, self.dims, self.attrs, self.init, self.storage = name, typ, dims, attrs, init, storage
        self.cname = None

    @property
    def rank(self):
        return len(self.dims) if self.dims else 0

    @property
    def kind(self):
        """How an array is held: explicit (dummy, pointer to first element), desc (descriptor), assumed_size."""
        if not self.dims:
            return None
        if self.storage == "dummy" and all(d not in (":", "*") for d in self.dims):
            return "explicit"
        if self.dims == ["*"]:
            return "assumed_size"
        return "desc"


class Proc:
    def __init__(self, module, name, kind, args, result, bind=None):
        self.module, self.name, self.kind, self.args, self.result, self.bind = module, name, kind, args, result, bind
        self.syms = {}
        self.body = []
        self.line = 0

    @property
    def cname(self):
        return self.bind if self.bind else "F_%s_%s" % (self.module.name, self.name)


class Module:
    def __init__(self, name, path):
        self.name, self.path = name, path
        self.uses, self.syms, self.procs, self.ifaces = [], {}, {}, {}
        self.default_private = False


TYPE_RE = re.compile(r"^(integer|real|logical|double\s+precision)\b\s*(\*\s*\d+|\([^)]*\))?\s*(.*)$")


def parse_type(base, kind):
    if base.startswith("double"):
        return "double"
    if base == "real":
        if kind:
            k = kind.strip("*() ").replace("kind=", "")
            if k in ("8", "c_double", "dp"):
                return "double"
        return "real"
    return "int" if base == "integer" else "logical"


def parse_decl(text, storage):
    """Type declaration statement -> list of Sym."""
    m = TYPE_RE.match(text)
    base, kind, rest = m.group(1), m.group(2), m.group(3)
    typ = parse_type(base, kind)
    if "::" in rest:
        attr_s, ents = rest.split("::", 1)
        attrs_l = [a.strip() for a in split_top(attr_s) if a.strip()]
    else:
        attrs_l, ents = [], rest
    attrs, dims = set(), None
    for a in attrs_l:
        if a.startswith("dimension"):
            dims = [d.strip() for d in split_top(a[a.index("(") + 1:match_paren(a, a.index("("))])]
        elif a.startswith("intent"):
            attrs.add("intent")
        else:
            attrs.add(a)
    out = []
    for ent in split_top(ents):
        ent = ent.strip()
        if not ent:
            continue
        init = None
        if "=>" in ent:
            ent = ent.split("=>")[0].strip()
        elif "=" in ent:
            ent, ini = ent.split("=", 1)
            ent, init = ent.strip(), parse_expr(ini.strip())
        edims = dims
        if "(" in ent:
            nm = ent[:ent.index("(")].strip()
            edims = [d.strip() for d in split_top(ent[ent.index("(") + 1:match_paren(ent, ent.index("("))])]
            ent = nm
        out.append(Sym(ent, typ, list(edims) if edims else None, set(attrs), init, storage))
    return out


def parse_files(src_dir, files=MODULE_FILES):
    modules = {}
    for fname in files:
        path = os.path.join(src_dir, fname)
        stmts = read_statements(path)
        parse_module_file(stmts, path, modules)
    return modules


def parse_module_file(stmts, path, modules):
    i = 0
    mod = None
    in_contains = False
    in_iface = False
    while i < len(stmts):
        no, s = stmts[i]
        m = re.match(r"^module\s+(\w+)$", s)
        if m:
            mod = Module(m.group(1), path)
            modules[mod.name] = mod
            in_contains = False
            i += 1
            continue
        if mod is None:
            raise F90Error("%s:%d: statement outside a module: %s" % (path, no, s))
        if re.match(r"^end\s*module", s):
            mod = None
            i += 1
            continue
        if s.startswith("use "):
            mod.uses.append(s.split()[1].strip(","))
        elif s == "implicit none" or s == "import":
            pass
        elif s == "contains":
            in_contains = True
        elif s == "interface":
            in_iface = True
        elif re.match(r"^end\s*interface", s):
            in_iface = False
        elif s in ("private",):
            mod.default_private = True
        elif re.match(r"^(recursive\s+)?subroutine\b", s) or re.match(r"^(\w+\s+)?function\b", s):
            proc, i = parse_proc(stmts, i, mod, iface=in_iface)
            if in_iface:
                mod.ifaces[proc.name] = proc
            else:
                mod.procs[proc.name] = proc
            continue
        elif TYPE_RE.match(s) and not in_contains:
            for sym in parse_decl(s, "module"):
                mod.syms[sym.name] = sym
        else:
            raise F90Error("%s:%d: unsupported module-level statement: %s" % (path, no, s))
        i += 1


def parse_proc(stmts, i, mod, iface=False):
    no, s = stmts[i]
    bind = None
    mb = re.search(r"bind\s*\(\s*c\s*,\s*name\s*=\s*['\"](\w+)['\"]\s*\)", s)
    if mb:
        bind = mb.group(1)
        s = s[:mb.start()].strip()
    m = re.match(r"^(?:recursive\s+)?subroutine\s+(\w+)\s*(?:\((.*)\))?$", s)
    if m:
        kind, name, args, result = "subroutine", m.group(1), m.group(2), None
    else:
        m = re.match(r"^(?:\w+\s+)?function\s+(\w+)\s*\((.*?)\)\s*(?:result\s*\(\s*(\w+)\s*\))?$", s)
        if not m:
            raise F90Error("%s:%d: cannot parse procedure header: %s" % (mod.path, no, s))
        kind, name, args, result = "function", m.group(1), m.group(2), m.group(3) or m.group(1)
    args = [a.strip() for a in (args or "").split(",") if a.strip()]
    proc = Proc(mod, name, kind, args, result, bind)
    proc.line = no
    i += 1
    decl_phase = True
    stack = [proc.body]
    blocks = []
    while i < len(stmts):
        no, s = stmts[i]
        if re.match(r"^end\s*(subroutine|function)\b", s) or s == "end":
            i += 1
            break
        if iface:
            if TYPE_RE.match(s):
                for sym in parse_decl(s, "dummy"):
                    proc.syms[sym.name] = sym
            i += 1
            continue
        if TYPE_RE.match(s) and decl_phase:
            for sym in parse_decl(s, "local"):
                proc.syms[sym.name] = sym
            i += 1
            continue
        if s in ("implicit none", "import"):
            i += 1
            continue
        decl_phase = False
        st = parse_stmt(s, mod, no)
        if st[0] == "do":
            node = ["do", st[1], st[2], st[3], st[4], []]
            stack[-1].append(node)
            stack.append(node[5])
            blocks.append(("do", no))
        elif st[0] == "enddo":
            if not blocks or blocks[-1][0] != "do":
                raise F90Error("%s:%d: unmatched end do" % (mod.path, no))
            blocks.pop()
            stack.pop()
        elif st[0] == "ifthen":
            node = ["if", [[st[1], []]], None]
            stack[-1].append(node)
            stack.append(node[1][0][1])
            blocks.append(("if", node))
        elif st[0] == "elseif":
            node = blocks[-1][1]
            stack.pop()
            node[1].append([st[1], []])
            stack.append(node[1][-1][1])
        elif st[0] == "else":
            node = blocks[-1][1]
            stack.pop()
            node[2] = []
            stack.append(node[2])
        elif st[0] == "endif":
            if not blocks or blocks[-1][0] != "if":
                raise F90Error("%s:%d: unmatched end if" % (mod.path, no))
            blocks.pop()
            stack.pop()
        else:
            stack[-1].append(list(st) + [no])
        i += 1
    if blocks:
        raise F90Error("%s: unterminated block in %s" % (mod.path, name))
    for a in args:
        if a in proc.syms:
            proc.syms[a].storage = "dummy"
        else:
            proc.syms[a] = Sym(a, implicit_type(a), None, set(), None, "dummy")
    if kind == "function" and result not in proc.syms:
        proc.syms[result] = Sym(result, implicit_type(result), None, set(), None, "local")
    return proc, i


def implicit_type(name):
    return "int" if name[0] in "ijklmn" else "real"


IO_RE = re.compile(r"^(write|print|close|open|flush)\b")


def parse_stmt(s, mod, no):
    if IO_RE.match(s):
        return ("nop",)
    m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", s)
    if m:
        parts = split_top(m.group(2))
        step = parse_expr(parts[2]) if len(parts) > 2 else ("lit", "int", "1")
        return ("do", m.group(1), parse_expr(parts[0]), parse_expr(parts[1]), step)
    if re.match(r"^end\s*do$", s):
        return ("enddo",)
    if re.match(r"^end\s*if$", s):
        return ("endif",)
    if s == "else":
        return ("else",)
    m = re.match(r"^else\s*if\s*\(", s)
    if m:
        j = match_paren(s, s.index("("))
        if s[j + 1:].strip() != "then":
            raise F90Error("bad else if: " + s)
        return ("elseif", parse_expr(s[s.index("(") + 1:j]))
    if re.match(r"^if\s*\(", s):
        j = match_paren(s, s.index("("))
        cond = parse_expr(s[s.index("(") + 1:j])
        rest = s[j + 1:].strip()
        if rest == "then":
            return ("ifthen", cond)
        return ("if1", cond, parse_stmt(rest, mod, no))
    m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?$", s)
    if m:
        args = P("x(" + m.group(3) + ")").parse()[2] if m.group(3) and m.group(3).strip() else []
        return ("call", m.group(1), args)
    m = re.match(r"^(de)?allocate\s*\((.*)\)$", s)
    if m:
        items = [parse_expr(x) for x in split_top(m.group(2))]
        return ("dealloc" if m.group(1) else "alloc", items)
    if s in ("return",):
        return ("return",)
    if s.startswith("stop"):
        return ("stop",)
    # pointer assignment
    m = re.match(r"^(\w+)\s*=>\s*(.*)$", s)
    if m:
        return ("ptr", m.group(1), parse_expr(m.group(2)))
    # assignment: the first top-level '=' that is not part of a relational operator
    depth = 0
    for k, ch in enumerate(s):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0:
            prev = s[k - 1] if k else ""
            nxt = s[k + 1] if k + 1 < len(s) else ""
            if prev in "=/<>" or nxt in "=>":
                continue
            return ("assign", parse_expr(s[:k].strip()), parse_expr(s[k + 1:].strip()))
    raise F90Error("%s:%d: unsupported statement: %s" % (mod.path, no, s))


# --------------------------------------------------------------------------- code generation
class Gen:
    def __init__(self, modules, hooks=None, header="ref90.h"):
        self.mods = modules
        self.hooks = HOOKS if hooks is None else hooks
        self.header = header
        self.needed = []
        self.seen = set()
        self.tmp = 0
        self.warn = []

    # name lookup --------------------------------------------------------
    def visible_modules(self, mod, seen=None):
        """mod, then the modules it uses (transitively), in use order."""
        seen = seen if seen is not None else set()
        if mod.name in seen:
            return []
        seen.add(mod.name)
        out = [mod]
        for u in mod.uses:
            if u in self.mods:
                out += self.visible_modules(self.mods[u], seen)
        return out

    def lookup_var(self, proc, name):
        if name in proc.syms:
            return proc.syms[name]
        for i, m in enumerate(self.visible_modules(proc.module)):
            if name in m.syms and (i == 0 or not self.is_private(m, m.syms[name])):
                return m.syms[name]
        return None

    def is_private(self, mod, sym):
        if "private" in sym.attrs:
            return True
        if "public" in sym.attrs:
            return False
        return mod.default_private

    def lookup_proc(self, proc, name):
        for m in self.visible_modules(proc.module):
            if name in m.procs:
                return m.procs[name]
            if name in m.ifaces:
                return m.ifaces[name]
        return None

    # naming -------------------------------------------------------------
    def name_syms(self):
        for mod in self.mods.values():
            for s in mod.syms.values():
                s.cname = "M_%s_%s" % (mod.name, s.name)
            for p in list(mod.procs.values()) + list(mod.ifaces.values()):
                for s in p.syms.values():
                    s.cname = ("a_" if s.storage == "dummy" else "l_") + s.name

    # expressions --------------------------------------------------------
    def scalar_ref(self, sym):
        """C lvalue of a scalar variable."""
        if sym.storage == "dummy" and "value" not in sym.attrs:
            return "(*%s)" % sym.cname
        return sym.cname

    def extent(self, sym, k):
        return "%s.n[%d]" % (sym.cname, k)

    def elem(self, sym, subs):
        """C lvalue of an array element; subs are C expressions (1-based)."""
        if len(subs) != sym.rank and sym.kind != "assumed_size":
            raise F90Error("rank mismatch for %s" % sym.name)
        if sym.kind == "assumed_size":
            return "%s[(long)(%s)-1]" % (sym.cname, subs[0])
        off = "(long)(%s)-1" % subs[-1]
        for k in range(len(subs) - 2, -1, -1):
            off = "(long)(%s)-1 + %s*(%s)" % (subs[k], self.extent(sym, k), off)
        return "%s.p[%s]" % (sym.cname, off)

    def etype(self, e, proc):
        """Result type of a scalar expression: int, real, double, logical."""
        t = e[0]
        if t == "lit":
            return e[1]
        if t == "par":
            return self.etype(e[1], proc)
        if t == "name":
            s = self.lookup_var(proc, e[1])
            if s is None:
                raise F90Error("unknown name %s in %s" % (e[1], proc.name))
            return s.typ
        if t == "ref":
            s = self.lookup_var(proc, e[1])
            if s is not None:
                return s.typ
            if e[1] in ("exp", "log", "sqrt", "abs", "sin", "cos", "min", "max"):
                return self.etype(e[2][0], proc)
            if e[1] in ("mod", "int", "nint"):
                return "int"
            if e[1] in ("real", "float"):
                return "real"
            if e[1] in STUB_FUNCS:
                return STUB_FUNCS[e[1]][0]
            p = self.lookup_proc(proc, e[1])
            if p is not None and p.kind == "function":
                return p.syms[p.result].typ
            raise F90Error("unknown function %s" % e[1])
        if t == "un":
            return "logical" if e[1] == "!" else self.etype(e[2], proc)
        if t == "pow":
            return self.etype(e[1], proc)
        if t == "bin":
            if e[1] in ("&&", "||", "==", "!=", "<", "<=", ">", ">="):
                return "logical"
            a, b = self.etype(e[2], proc), self.etype(e[3], proc)
            for k in ("double", "real", "int"):
                if k in (a, b):
                    return k
        raise F90Error("cannot type %r" % (e,))

    def section_dims(self, e, proc):
        """For an array-valued primary: list of (sym, k) section dimensions, else []."""
        if e[0] == "name":
            s = self.lookup_var(proc, e[1])
            if s is not None and s.rank:
                return [(s, k) for k in range(s.rank)]
            return []
        if e[0] == "ref":
            s = self.lookup_var(proc, e[1])
            if s is not None and s.rank:
                return [(s, k) for k, a in enumerate(e[2]) if a[0] == "range"]
        return []

    def is_array_expr(self, e, proc):
        t = e[0]
        if t in ("name", "ref"):
            if self.section_dims(e, proc):
                return True
            if t == "ref" and self.lookup_var(proc, e[1]) is None:
                return any(self.is_array_expr(a, proc) for a in e[2] if a[0] not in ("kw", "range"))
            return False
        if t in ("par", "un"):
            return self.is_array_expr(e[-1], proc)
        if t in ("bin", "pow"):
            return any(self.is_array_expr(x, proc) for x in e[-2:])
        return False

    def cexpr(self, e, proc, loop=None):
        """C text of an expression.  loop: list of C index expressions (0-based
        offsets) for the section dimensions, when evaluating elementwise."""
        t = e[0]
        if t == "lit":
            return e[2]
        if t == "str":
            raise F90Error("string in computation")
        if t == "par":
            return "(%s)" % self.cexpr(e[1], proc, loop)
        if t == "un":
            return "(%s%s)" % (e[1], self.cexpr(e[2], proc, loop))
        if t == "bin":
            return "(%s %s %s)" % (self.cexpr(e[2], proc, loop), e[1], self.cexpr(e[3], proc, loop))
        if t == "pow":
            ex = e[2]
            if ex[0] == "lit" and ex[1] == "int" and ex[2] == "2":
                b = self.cexpr(e[1], proc, loop)
                return "(%s*%s)" % (b, b)
            raise F90Error("unsupported power %r" % (e,))
        if t == "name":
            s = self.lookup_var(proc, e[1])
            if s is None:
                raise F90Error("unknown name %s in %s" % (e[1], proc.name))
            if s.rank:
                if loop is None:
                    raise F90Error("array %s used as a scalar" % e[1])
                if len(loop) != s.rank:
                    raise F90Error("shape mismatch for %s" % e[1])
                return self.elem(s, ["%s+1" % l for l in loop])
            return self.scalar_ref(s)
        if t == "ref":
            s = self.lookup_var(proc, e[1])
            if s is not None and s.rank:
                subs, li = [], 0
                for a in e[2]:
                    if a[0] == "range":
                        if loop is None:
                            raise F90Error("section of %s used as a scalar" % e[1])
                        lo = self.cexpr(a[1], proc) if a[1] is not None else "1"
                        subs.append("(%s)+%s" % (lo, loop[li]))
                        li += 1
                    else:
                        subs.append(self.cexpr(a, proc))
                if loop is not None and li not in (0, len(loop)):
                    raise F90Error("shape mismatch for %s" % e[1])
                return self.elem(s, subs)
            name, args = e[1], e[2]
            ca = [self.cexpr(a, proc, loop) for a in args]
            if name == "nint":
                ty = self.etype(args[0], proc)
                return "((int)lround%s(%s))" % ("f" if ty == "real" else "", ca[0])
            if name in ("exp", "log", "sqrt", "abs", "sin", "cos"):
                ty = self.etype(args[0], proc)
                fn = {"abs": "fabs"}.get(name, name)
                if ty == "int" and name == "abs":
                    return "abs(%s)" % ca[0]
                return "%s%s(%s)" % (fn, "f" if ty == "real" else "", ca[0])
            if name == "mod":
                return "((%s) %% (%s))" % (ca[0], ca[1])
            if name in ("real", "float"):
                return "((float)(%s))" % ca[0]
            if name == "int":
                return "((int)(%s))" % ca[0]
            if name in ("min", "max"):
                op = "<" if name == "min" else ">"
                return "((%s) %s (%s) ? (%s) : (%s))" % (ca[0], op, ca[1], ca[0], ca[1])
            if name in STUB_FUNCS:
                return STUB_FUNCS[name][1]
            p = self.lookup_proc(proc, name)
            if p is not None and p.kind == "function":
                self.require(p)
                return "%s(%s)" % (p.cname, ", ".join(self.actuals(proc, p, args)))
            raise F90Error("unknown function %s in %s" % (name, proc.name))
        raise F90Error("cannot generate %r" % (e,))

    # calls --------------------------------------------------------------
    def actuals(self, proc, callee, args):
        if len(args) != len(callee.args):
            raise F90Error("call of %s with %d arguments, %d expected" % (callee.name, len(args), len(callee.args)))
        out = []
        for a, dn in zip(args, callee.args):
            d = callee.syms[dn]
            if a[0] == "kw":
                raise F90Error("keyword arguments are not supported")
            if d.rank == 0:
                if "value" in d.attrs:
                    out.append(self.cexpr(a, proc))
                    continue
                if a[0] == "name":
                    s = self.lookup_var(proc, a[1])
                    if s is not None and not s.rank:
                        out.append("&" + self.scalar_ref(s) if not (s.storage == "dummy" and "value" not in s.attrs)
                                   else s.cname)
                        continue
                if a[0] == "ref":
                    s = self.lookup_var(proc, a[1])
                    if s is not None and s.rank and not self.section_dims(a, proc):
                        out.append("&" + self.cexpr(a, proc))
                        continue
                out.append("&(%s){%s}" % (CTYPE[d.typ], self.cexpr(a, proc)))
                continue
            # array dummy
            s = self.lookup_var(proc, a[1]) if a[0] in ("name", "ref") else None
            if s is None or not s.rank:
                raise F90Error("array argument %s of %s is not an array" % (dn, callee.name))
            first = self.first_elem(a, s, proc)
            if d.kind in ("explicit", "assumed_size"):
                out.append("&" + first)
            else:
                out.append(self.section_desc(a, s, proc, first))
        return out

    def first_elem(self, a, s, proc):
        """C lvalue of the first element of a whole array, contiguous section or element."""
        if a[0] == "name":
            return self.elem(s, ["1"] * s.rank) if s.kind != "assumed_size" else "%s[0]" % s.cname
        subs, seen_scalar = [], False
        for k, x in enumerate(a[2]):
            if x[0] == "range":
                if seen_scalar or x[1] is not None or x[2] is not None:
                    raise F90Error("non-contiguous section passed to a procedure")
                subs.append("1")
            else:
                seen_scalar = True
                subs.append(self.cexpr(x, proc))
        return self.elem(s, subs)

    def section_desc(self, a, s, proc, first):
        """Descriptor for an assumed-shape dummy."""
        if a[0] == "name" or all(x[0] == "range" for x in a[2]):
            return s.cname
        ext = [self.extent(s, k) for k, x in enumerate(a[2]) if x[0] == "range"]
        ext += ["1"] * (3 - len(ext))
        return "(%s){&%s, {%s}}" % (ATYPE[s.typ], first, ", ".join(ext))

    def require(self, p):
        if p.bind:
            if ("iface", p.name) not in self.seen:
                self.seen.add(("iface", p.name))
                self.needed.append(p)
            return
        key = (p.module.name, p.name)
        if key not in self.seen:
            self.seen.add(key)
            self.needed.append(p)

    # statements ---------------------------------------------------------
    def stmts(self, body, proc, ind):
        out = []
        for st in body:
            out += self.stmt(st, proc, ind)
        return out

    def stmt(self, st, proc, ind):
        pad = "    " * ind
        k = st[0]
        if k in ("nop",):
            return []
        if k == "assign":
            return [pad + x for x in self.assign(st[1], st[2], proc)]
        if k == "ptr":
            s = self.lookup_var(proc, st[1])
            t = st[2]
            if t[0] != "name":
                raise F90Error("pointer target must be a whole array")
            ts = self.lookup_var(proc, t[1])
            if ts.kind == "explicit":
                ext = [self.extent(ts, k2) for k2 in range(ts.rank)] + ["1"] * (3 - ts.rank)
                return [pad + "%s = (%s){%s.p, {%s}};" % (s.cname, ATYPE[s.typ], ts.cname, ", ".join(ext))]
            return [pad + "%s = %s;" % (s.cname, ts.cname)]
        if k == "call":
            name, args = st[1], st[2]
            if name in STUB_CALLS:
                return [pad + "/* %s: SEPlib I/O, dropped */" % name]
            callee = self.lookup_proc(proc, name)
            if callee is None:
                raise F90Error("unknown subroutine %s called from %s" % (name, proc.name))
            self.require(callee)
            pre = []
            hook = self.hooks.get((proc.name, name))
            if hook:
                pre = [pad + "%s();" % hook]
            return pre + [pad + "%s(%s);" % (callee.cname, ", ".join(self.actuals(proc, callee, args)))]
        if k == "do":
            var = self.lookup_var(proc, st[1])
            v = self.scalar_ref(var)
            step = st[4]
            if step[0] == "un" and step[2][0] == "lit":
                sv = -int(step[2][2])
            elif step[0] == "lit" and step[1] == "int":
                sv = int(step[2])
            else:
                raise F90Error("DO step must be an integer literal")
            self.tmp += 1
            e = "e%d" % self.tmp
            cmp = "<=" if sv > 0 else ">="
            out = [pad + "{ int %s = %s;" % (e, self.cexpr(st[3], proc)),
                   pad + "for (%s = %s; %s %s %s; %s += %d) {" % (v, self.cexpr(st[2], proc), v, cmp, e, v, sv)]
            out += self.stmts(st[5], proc, ind + 1)
            out += [pad + "} }"]
            return out
        if k == "if":
            branches, els = st[1], st[2]
            bodies = [self.stmts(b, proc, ind + 1) for _, b in branches]
            ebody = self.stmts(els, proc, ind + 1) if els is not None else []
            if not any(_live(b) for b in bodies) and not _live(ebody):
                return []
            out = []
            for j, ((cond, _), b) in enumerate(zip(branches, bodies)):
                out.append(pad + ("if (%s) {" if j == 0 else "} else if (%s) {") % self.cexpr(cond, proc))
                out += b
            if els is not None:
                out.append(pad + "} else {")
                out += ebody
            out.append(pad + "}")
            return out
        if k == "if1":
            inner = self.stmt(list(st[2]), proc, ind + 1)
            if not _live(inner):
                return []
            return [pad + "if (%s) {" % self.cexpr(st[1], proc)] + inner + [pad + "}"]
        if k == "alloc":
            out = []
            for item in st[1]:
                if item[0] != "ref":
                    raise F90Error("bad allocate item")
                s = self.lookup_var(proc, item[1])
                ext = [self.cexpr(x, proc) for x in item[2]] + ["1"] * (3 - len(item[2]))
                out.append(pad + "f90_alloc_%s(&%s, %s);" % (CTYPE[s.typ][0], s.cname, ", ".join(ext)))
            return out
        if k == "dealloc":
            return [pad + "f90_free_%s(&%s);" % (CTYPE[self.lookup_var(proc, it[1]).typ][0],
                                                 self.lookup_var(proc, it[1]).cname) for it in st[1]]
        if k == "return":
            if proc.kind == "function":
                return [pad + "return %s;" % proc.syms[proc.result].cname]
            return [pad + "return;"]
        if k == "stop":
            return [pad + "f90_stop();"]
        raise F90Error("cannot generate statement %r" % (st,))

    def assign(self, lhs, rhs, proc):
        if lhs[0] == "name":
            s = self.lookup_var(proc, lhs[1])
            if s is None:
                raise F90Error("assignment to unknown %s in %s" % (lhs[1], proc.name))
            if not s.rank:
                if self.is_array_expr(rhs, proc):
                    raise F90Error("array value assigned to scalar %s" % lhs[1])
                return ["%s = %s;" % (self.scalar_ref(s), self.cexpr(rhs, proc))]
        s = self.lookup_var(proc, lhs[1])
        dims = self.section_dims(lhs, proc)
        if not dims:
            return ["%s = %s;" % (self.cexpr(lhs, proc), self.cexpr(rhs, proc))]
        # extents of the section dimensions of the left-hand side
        ext = []
        for (sym, k) in dims:
            rng = lhs[2][k] if lhs[0] == "ref" else ("range", None, None)
            lo = self.cexpr(rng[1], proc) if rng[1] is not None else "1"
            hi = self.cexpr(rng[2], proc) if rng[2] is not None else self.extent(sym, k)
            ext.append("(long)(%s)-(long)(%s)+1" % (hi, lo))
        self.tmp += 1
        n = self.tmp
        loopv = ["j%d_%d" % (n, k) for k in range(len(dims))]
        need_tmp = self.rhs_aliases(lhs, rhs, proc)
        lines = ["{"]
        lines += ["    long n%d_%d = %s;" % (n, k, ext[k]) for k in range(len(dims))]
        cty = CTYPE[s.typ]
        if need_tmp:
            tot = "*".join("n%d_%d" % (n, k) for k in range(len(dims)))
            lines.append("    %s *t%d = (%s *)malloc(sizeof(%s) * (size_t)(%s));" % (cty, n, cty, cty, tot))
        flat = " + ".join(["%s" % loopv[0]] + ["%s*%s" % (loopv[k], "*".join("n%d_%d" % (n, q) for q in range(k)))
                                                 for k in range(1, len(dims))])

        def nest(body):
            out, ind = [], "    "
            for k in range(len(dims) - 1, -1, -1):
                out.append(ind + "for (long %s = 0; %s < n%d_%d; %s++)" % (loopv[k], loopv[k], n, k, loopv[k]))
                ind += "    "
            out.append(ind + body)
            return out

        rv = self.cexpr(rhs, proc, loopv) if self.is_array_expr(rhs, proc) else self.cexpr(rhs, proc)
        lv = self.cexpr(lhs, proc, loopv)
        if need_tmp:
            lines += nest("t%d[%s] = %s;" % (n, flat, rv))
            lines += nest("%s = t%d[%s];" % (lv, n, flat))
            lines.append("    free(t%d);" % n)
        else:
            lines += nest("%s = %s;" % (lv, rv))
        lines.append("}")
        return lines

    def rhs_aliases(self, lhs, rhs, proc):
        """True when the left-hand array appears on the right with other subscripts."""
        name = lhs[1]
        found = []

        def walk(e):
            if not isinstance(e, tuple):
                return
            if e[0] in ("name", "ref") and e[1] == name:
                found.append(e)
            for x in e[1:]:
                if isinstance(x, tuple):
                    walk(x)
                elif isinstance(x, list):
                    for y in x:
                        walk(y)
        walk(rhs)
        norm = lambda e: ("name", e[1]) if e[0] == "name" else e
        lhs_n = lhs if lhs[0] == "ref" else ("ref", name, [("range", None, None)] * len(self.section_dims(lhs, proc)))
        for e in found:
            en = e if e[0] == "ref" else ("ref", name, [("range", None, None)] * len(self.section_dims(e, proc)))
            if en != lhs_n:
                return True
        return False

    # procedures ----------------------------------------------------------
    def proto(self, p):
        if p.kind == "function":
            ret = CTYPE[p.syms[p.result].typ]
        else:
            ret = "void"
        params = []
        for a in p.args:
            s = p.syms[a]
            if s.rank:
                if s.kind in ("explicit", "assumed_size"):
                    params.append("%s *%s%s" % (CTYPE[s.typ], s.cname, "_p" if s.kind == "explicit" else ""))
                else:
                    params.append("%s %s" % (ATYPE[s.typ], s.cname))
            elif "value" in s.attrs:
                params.append("%s %s" % (CTYPE[s.typ], s.cname))
            else:
                params.append("%s *%s" % (CTYPE[s.typ], s.cname))
        return "%s %s(%s)" % (ret, p.cname, ", ".join(params) or "void")

    def proc_body(self, p):
        lines = [self.proto(p) + "\n{"]
        # locals (scalars and descriptors); explicit-shape dummies get a descriptor
        for s in p.syms.values():
            if s.storage == "dummy":
                continue
            if s.rank:
                lines.append("    %s %s = {0};" % (ATYPE[s.typ], s.cname))
            else:
                init = " = %s" % self.cexpr(s.init, p) if s.init is not None else " = 0"
                lines.append("    %s %s%s;" % (CTYPE[s.typ], s.cname, init))
        for a in p.args:
            s = p.syms[a]
            if s.kind == "explicit":
                ext = [self.cexpr(parse_expr(d), p) for d in s.dims] + ["1"] * (3 - s.rank)
                lines.append("    %s %s = {%s_p, {%s}};" % (ATYPE[s.typ], s.cname, s.cname, ", ".join(ext)))
        body = self.stmts(p.body, p, 1)
        lines += body
        if p.kind == "function":
            lines.append("    return %s;" % p.syms[p.result].cname)
        lines.append("}")
        return "\n".join(lines)

    def generate(self, entries):
        self.name_syms()
        for mname, pname in entries:
            self.require(self.mods[mname].procs[pname])
        bodies = {}
        i = 0
        while i < len(self.needed):
            p = self.needed[i]
            if not p.bind:
                bodies[(p.module.name, p.name)] = self.proc_body(p)
            i += 1
        out = [C_PRELUDE.replace('"ref90.h"', '"%s"' % self.header)]
        # module variables
        for mod in self.mods.values():
            for s in mod.syms.values():
                if s.rank:
                    out.append("static %s %s = {0};" % (ATYPE[s.typ], s.cname))
                else:
                    init = self.const_init(s, mod)
                    out.append("static %s %s = %s;" % (CTYPE[s.typ], s.cname, init))
        for h in sorted(set(self.hooks.values())):
            out.append("void %s(void);" % h)
        for p in self.needed:
            if p.bind:
                out.append("extern " + self.proto(p) + ";")
            else:
                out.append(self.proto(p) + ";")
        for p in self.needed:
            if not p.bind:
                out.append("")
                out.append("/* %s:%d %s %s */" % (os.path.basename(p.module.path), p.line, p.kind, p.name))
                out.append(bodies[(p.module.name, p.name)])
        out.append(self.table())
        return "\n".join(out) + "\n"

    def const_init(self, s, mod):
        if s.init is None:
            return "0"
        fake = Proc(mod, "_init", "subroutine", [], None)
        return self.cexpr(s.init, fake)

    def table(self):
        rows = []
        for mod in self.mods.values():
            for s in mod.syms.values():
                if s.rank and s.typ == "real":
                    rows.append('    {"%s.%s", &%s},' % (mod.name, s.name, s.cname))
        return ("\nconst struct ref90_var ref90_vars[] = {\n" + "\n".join(rows) +
                '\n    {0, 0}\n};\n')


def _live(lines):
    return any(not l.strip().startswith("/*") for l in lines)


C_PRELUDE = r"""/* Generated from the reference's Fortran modules by oracle/f90c.py.
 * Test infrastructure only: an execution of the reference's own code. */
#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include "ref90.h"

static void f90_alloc_f(rarr *a, long n1, long n2, long n3)
{
    free(a->p);
    a->p = (float *)calloc((size_t)(n1 * n2 * n3), sizeof(float));
    if (!a->p) { fprintf(stderr, "ref90: out of memory\n"); abort(); }
    a->n[0] = n1; a->n[1] = n2; a->n[2] = n3;
}
static void f90_free_f(rarr *a) { free(a->p); a->p = 0; }
static void f90_stop(void) { fprintf(stderr, "ref90: STOP\n"); abort(); }
"""

H_TEXT = r"""/* Descriptors of the translated reference modules (test infrastructure). */
#ifndef REF90_H
#define REF90_H
typedef struct { float *p; long n[3]; } rarr;
typedef struct { double *p; long n[3]; } darr;
typedef struct { int *p; long n[3]; } iarr;
struct ref90_var { const char *name; rarr *arr; };
extern const struct ref90_var ref90_vars[];
void F_rtm_mod_adj_rtm_init(int *a_nz_in, float *a_dz_in, int *a_nx_in, float *a_dx_in, float *a_dt_in,
                            int *a_xsource_in, int *a_zsource_in, int *a_zrec_in, float *a_fp_in, int *a_nt_in,
                            int *a_abc_in, int *a_free_surface_in, rarr a_m1_in, rarr a_m2_in, rarr a_m3_in,
                            int *a_lame_in);
void F_rtm_mod_adj_rtm_op2(int *a_adj, rarr a_dm1_in, rarr a_dm2_in, rarr a_dm3_in, rarr a_vx_in, rarr a_vz_in,
                           rarr a_sigmaxx_in, rarr a_sigmazz_in, rarr a_sigmaxz_in);
#endif
"""


# The split-field PML Born modelling program of 2d_rtm_restart/working_Src
# (born.f90 -> born-mod.f90 with bornlib-mod.f90, pml-mod.f90, source-mod.f90,
# seis-mod-born.f90, snap-mod-born.f90).  born-mod.f90:521-545 calls
# explosive_sourcex/explosive_sourcez with six arguments, while
# source-mod.f90:77-100 defines them with four; pml_source_shim.f90 (beside
# this script) supplies the six-argument forms with the four-argument bodies.
PML_FILES = ["source-mod.f90", "seis-mod-born.f90", "bornlib-mod.f90", "snap-mod-born.f90", "pml-mod.f90",
             "born-mod.f90"]
PML_ENTRIES = [("born_mod", "elastic_init"), ("born_mod", "elastic_op")]
PML_SHIM = "pml_source_shim.f90"

H_PML = r"""/* Descriptors of the translated reference PML Born modules (test infrastructure). */
#ifndef REFPML_H
#define REFPML_H
typedef struct { float *p; long n[3]; } rarr;
typedef struct { double *p; long n[3]; } darr;
typedef struct { int *p; long n[3]; } iarr;
struct ref90_var { const char *name; rarr *arr; };
extern const struct ref90_var ref90_vars[];
#endif
"""


def load_pml(src_dir):
    mods = parse_files(src_dir, PML_FILES)
    shim = {}
    here = os.path.dirname(os.path.abspath(__file__))
    parse_module_file(read_statements(os.path.join(here, PML_SHIM)), os.path.join(here, PML_SHIM), shim)
    src = mods["source_mod"]
    for name, proc in shim["source_shim"].procs.items():
        proc.module = src
        src.procs[name] = proc
    return mods


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--src", required=True, help="directory of the reference's Fortran modules")
    ap.add_argument("--out", required=True, help="output directory")
    ap.add_argument("--set", default="rtm", choices=["rtm", "pml"],
                    help="rtm: Src_working's RTM modules; pml: working_Src's PML Born modelling modules")
    a = ap.parse_args()
    if a.set == "rtm":
        mods, entries, hooks, base, header = parse_files(a.src), ENTRIES, HOOKS, "ref90", H_TEXT
    else:
        mods, entries, hooks, base, header = load_pml(a.src), PML_ENTRIES, {}, "refpml", H_PML
    g = Gen(mods, hooks, base + ".h")
    text = g.generate(entries)
    os.makedirs(a.out, exist_ok=True)
    with open(os.path.join(a.out, base + ".c"), "w") as f:
        f.write(text)
    with open(os.path.join(a.out, base + ".h"), "w") as f:
        f.write(header)
    print("%s: %d procedures translated" % (base, sum(1 for p in g.needed if not p.bind)), file=sys.stderr)


if __name__ == "__main__":
    main()
