"""Build recipe for oracle/_ref: the reference's own sweep subroutine
(`cliffs.f`, subroutine cliffs, lines 17-346), compiled here from its source
for checking the oracle against it (test infrastructure only).

Neither machine has a Fortran compiler, so this script translates the
Fortran of that one file into C, mechanically, and compiles the C with gcc.
It handles exactly the subset the file uses: fixed-form lines with tabs and
`&` continuations, `!` comments, numeric labels; INTEGER, REAL*8 and LOGICAL
declarations of scalars and arrays (1- and 2-D, 1-based); a REAL*8 PARAMETER;
IF/THEN/ELSE/END IF and one-line IF; DO with and without a terminal label,
GOTO, CONTINUE; FORALL and WHERE blocks; whole-array and section assignments
and the array constructor (/ ... /); the operators .eq. .ne. .lt. .le. .gt.
.ge. .and. .or. .not. == and **2; sqrt and max.  Anything else stops the
translation with an error naming the line.

Semantics kept from the Fortran:
- a real literal without an exponent or kind (0.125, 1.41421356) is default
  REAL, i.e. single precision, and enters REAL*8 arithmetic converted from
  float: it is emitted as (double)<literal>f;
- expressions are evaluated left to right within a precedence level, as
  gfortran does without -ffast-math; the C is compiled with
  -ffp-contract=off, so no multiply-add is fused (the reference's Makefile
  builds with gfortran's defaults, which on x86-64 fuse nothing either);
- x**2 is x*x.
- Local arrays are zeroed on entry (the Fortran leaves them undefined; the
  subroutine writes every element it reads on the paths a line can take).

The module arrays and scalars the subroutine uses (MASTER: dep, cel, xvel,
yvel, s1, s2, zeta, grav, edge1, edge2; PARAMETERS: ground, crough, dt,
celmin) become arguments of

    void ref_cliffs(int iu, int irw, int n, int nx, int ny, int mx,
                    double *dep, double *cel, double *xvel, double *yvel,
                    const double *s1, const double *s2, const double *zeta,
                    const double *edge1, const double *edge2, double grav,
                    double ground, double crough, double dt, double celmin);

with the reference's shapes, column-major: dep, cel, xvel, yvel (nx, ny),
s1 (nx-1, ny), s2 (ny-1), zeta (ny), edge1 and edge2 (mx, 3).

Output: oracle/_ref/cliffs_ref.c (generated) and oracle/_ref/libcliffs_ref.so.
Both stay out of version control: they are built from the reference checkout
wherever it is present.

    python oracle/ref_f2c.py [path/to/reference]
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFDIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REFDIR, "libcliffs_ref.so")
CSRC = os.path.join(REFDIR, "cliffs_ref.c")

MODULE_ARRAYS = {  # name -> C index expression of 1-based Fortran subscripts
    "dep": "dep[((size_t)({1})-1)*nx+({0})-1]",
    "cel": "cel[((size_t)({1})-1)*nx+({0})-1]",
    "xvel": "xvel[((size_t)({1})-1)*nx+({0})-1]",
    "yvel": "yvel[((size_t)({1})-1)*nx+({0})-1]",
    "s1": "s1[((size_t)({1})-1)*(nx-1)+({0})-1]",
    "s2": "s2[({0})-1]",
    "zeta": "zeta[({0})-1]",
    "edge1": "edge1[((size_t)({1})-1)*mx+({0})-1]",
    "edge2": "edge2[((size_t)({1})-1)*mx+({0})-1]",
}


class F2CError(Exception):
    pass


# ---- source lines ----------------------------------------------------------

def statements(text):
    """(label, statement, line number) of the fixed-form source, comments
    removed, continuations joined, `;` split, lower case."""
    out = []
    for no, raw in enumerate(text.splitlines(), 1):
        line = raw.rstrip("\n")
        if not line.strip() or line[:1] in ("c", "C", "*", "!"):
            continue
        # label field and continuation column (a tab ends the label field)
        head = line.split("\t", 1)[0] if "\t" in line[:6] else line[:6]
        body = line[len(head):] if "\t" in line[:6] else line[6:]
        cont = "\t" not in line[:6] and len(line) > 5 and line[5] not in " 0"
        if cont:
            head, body = line[:5], line[6:]
        body = body.split("!", 1)[0]  # no character constants in this file
        label = head.strip()
        if cont:
            if not out:
                raise F2CError(f"line {no}: continuation of nothing")
            lab, st, n0 = out[-1]
            out[-1] = (lab, st + " " + body.strip(), n0)
            continue
        if not body.strip():
            continue
        parts = [p.strip() for p in body.split(";") if p.strip()]
        for k, p in enumerate(parts):
            out.append((label if k == 0 else "", p.lower(), no))
    return out


# ---- expressions -----------------------------------------------------------

TOKEN = re.compile(r"\s*(?:(\(/|/\))|(\.(?:eq|ne|lt|le|gt|ge|and|or|not|true|false)\.)|"
                   r"(\d+\.\d+(?:[ed][+-]?\d+)?|\d+\.(?![a-z])|\.\d+(?:[ed][+-]?\d+)?|\d+[ed][+-]?\d+|\d+)|"
                   r"([a-z_][a-z0-9_]*)|(\*\*|==|/=|<=|>=|[-+*/(),:<>=]))")


def tokens(s):
    pos, out = 0, []
    s = s.strip()
    while pos < len(s):
        m = TOKEN.match(s, pos)
        if not m or m.end() == pos:
            raise F2CError(f"cannot read '{s[pos:]}'")
        pos = m.end()
        kind = [i for i in range(1, 6) if m.group(i) is not None][0]
        out.append(({1: "ctor", 2: "dot", 3: "num", 4: "id", 5: "op"}[kind], m.group(kind)))
    return out


class Expr:
    """Recursive-descent translation of one Fortran expression into C.
    arrays: local arrays (name -> rank); idx: element substitution for bare
    array names in whole-array statements (None outside them)."""

    def __init__(self, toks, arrays, idx=None):
        self.t, self.p, self.arrays, self.idx = toks, 0, arrays, idx

    def peek(self, k=0):
        return self.t[self.p + k] if self.p + k < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise F2CError(f"expected '{val}', found '{tok[1]}'")
        self.p += 1
        return tok

    def parse(self):
        e = self.or_()
        if self.p != len(self.t):
            raise F2CError(f"unread tokens from '{self.peek()[1]}'")
        return e

    def or_(self):
        e = self.and_()
        while self.peek()[1] == ".or.":
            self.take()
            e = f"({e} || {self.and_()})"
        return e

    def and_(self):
        e = self.not_()
        while self.peek()[1] == ".and.":
            self.take()
            e = f"({e} && {self.not_()})"
        return e

    def not_(self):
        if self.peek()[1] == ".not.":
            self.take()
            return f"(!{self.not_()})"
        return self.rel()

    REL = {".eq.": "==", "==": "==", ".ne.": "!=", "/=": "!=", ".lt.": "<", "<": "<", ".le.": "<=",
           "<=": "<=", ".gt.": ">", ">": ">", ".ge.": ">=", ">=": ">="}

    def rel(self):
        e = self.add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.take()[1]]
            e = f"({e} {op} {self.add()})"
        return e

    def add(self):
        if self.peek()[1] in ("-", "+"):  # leading sign applies to the first term
            op = self.take()[1]
            e = f"({op}{self.mul()})"
        else:
            e = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            e = f"({e} {op} {self.mul()})"
        return e

    def mul(self):
        e = self.pow_()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            e = f"({e} {op} {self.pow_()})"
        return e

    def pow_(self):
        e = self.primary()
        if self.peek()[1] == "**":
            self.take()
            k = self.take()
            if k != ("num", "2"):
                raise F2CError("only **2 is translated")
            e = f"SQ({e})"
        return e

    def args(self):
        self.take("(")
        out = [self.or_()]
        while self.peek()[1] == ",":
            self.take()
            out.append(self.or_())
        self.take(")")
        return out

    def primary(self):
        kind, val = self.peek()
        if kind == "num":
            self.take()
            if re.fullmatch(r"\d+", val):
                return val
            if "d" in val:
                return "(" + val.replace("d", "e") + ")"
            return f"((double){val if ('.' in val or 'e' in val) else val + '.'}f)"
        if kind == "dot" and val in (".true.", ".false."):
            self.take()
            return "1" if val == ".true." else "0"
        if val == "(":
            self.take()
            e = self.or_()
            self.take(")")
            return f"({e})"
        if kind == "id":
            self.take()
            if val in ("sqrt", "max"):
                a = self.args()
                return f"sqrt({a[0]})" if val == "sqrt" else f"IMAX({a[0]}, {a[1]})"
            if val in MODULE_ARRAYS:
                a = self.args() if self.peek()[1] == "(" else None
                if a is None:
                    if self.idx is None:
                        raise F2CError(f"whole module array {val} outside an array statement")
                    a = [self.idx]
                return "(" + MODULE_ARRAYS[val].format(*a) + ")"
            if val in self.arrays:
                if self.peek()[1] == "(":
                    a = self.args()
                    return f"{val}[{a[0]}]" if len(a) == 1 else f"{val}[{a[1]}][{a[0]}]"
                if self.idx is None:
                    raise F2CError(f"whole array {val} outside an array statement")
                return f"{val}[{self.idx}]"
            return val
        raise F2CError(f"unexpected '{val}'")


# ---- statements ------------------------------------------------------------

DECL = re.compile(r"^(integer|real\*8|logical)\b\s*(.*)$")


def split_top(s, sep=","):
    """Split s at top-level separators (outside parentheses)."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return [x.strip() for x in out]


def find_assign(st):
    """Index of the assignment '=' at top level (not part of ==, <=, >=, /=)."""
    depth = 0
    for i, ch in enumerate(st):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0:
            prev = st[i - 1] if i else ""
            nxt = st[i + 1] if i + 1 < len(st) else ""
            if prev not in "=<>/" and nxt != "=":
                return i
    return -1


class Translator:
    def __init__(self):
        self.arrays = {}   # local array -> list of C extent expressions
        self.types = {}    # local name -> C type
        self.params = {}
        self.out = []
        self.ind = 1
        self.stack = []    # open blocks: ("if"|"do"|"dolabel"|"forall"|"where", extra)
        self.args = []

    def emit(self, s):
        self.out.append("  " * self.ind + s)

    def expr(self, s, idx=None):
        return Expr(tokens(s), self.arrays, idx).parse()

    def decl(self, typ, rest):
        ctype = {"integer": "int", "real*8": "double", "logical": "int"}[typ]
        if rest.startswith(","):  # real*8, parameter :: name=value
            m = re.fullmatch(r",\s*parameter\s*::\s*([a-z0-9_]+)\s*=\s*(.+)", rest)
            if not m:
                raise F2CError(f"declaration '{rest}'")
            self.params[m.group(1)] = self.expr(m.group(2))
            self.emit(f"const {ctype} {m.group(1)} = {self.params[m.group(1)]};")
            return
        for item in split_top(rest):
            m = re.fullmatch(r"([a-z0-9_]+)(?:\((.*)\))?", item)
            if not m:
                raise F2CError(f"declaration item '{item}'")
            name, dims = m.group(1), m.group(2)
            if name in self.args:
                continue
            self.types[name] = ctype
            if dims is None:
                self.emit(f"{ctype} {name} = 0;")
                continue
            ext = [self.expr(d) for d in split_top(dims)]
            self.arrays[name] = ext
            if len(ext) == 1:
                self.emit(f"{ctype} *{name} = ({ctype} *)calloc((size_t)({ext[0]}) + 2, sizeof({ctype}));")
                self.frees.append(name)
            else:
                self.emit(f"{ctype} {name}[({ext[1]}) + 1][({ext[0]}) + 1];")
                self.emit(f"memset({name}, 0, sizeof({name}));")

    def assign(self, st, mask=None):
        i = find_assign(st)
        lhs, rhs = st[:i].strip(), st[i + 1:].strip()
        m = re.fullmatch(r"([a-z0-9_]+)(?:\((.*)\))?", lhs)
        if not m:
            raise F2CError(f"assignment target '{lhs}'")
        name, subs = m.group(1), m.group(2)
        if rhs.startswith("(/"):  # array constructor into a section a(lo:hi, k)
            vals = split_top(rhs[2:-2])
            s = split_top(subs)
            lo, hi = s[0].split(":")
            for k, v in enumerate(vals):
                self.emit(f"{name}[{self.expr(s[1])}][({self.expr(lo)}) + {k}] = {self.expr(v)};")
            return
        whole = name in self.arrays and (subs is None or ":" in subs)
        if not whole:
            target = self.expr(lhs)
            line = f"{target} = {self.expr(rhs)};"
            self.emit(line if mask is None else f"if ({mask}) {line}")
            return
        # whole array or section lo:hi of a 1-D local array
        if subs is None:
            lo, hi = "1", self.arrays[name][0]
        else:
            lo, hi = subs.split(":")
            lo, hi = self.expr(lo), self.expr(hi)
        rhs_c = self.section_rhs(rhs)
        self.emit(f"for (int _i = {lo}; _i <= {hi}; ++_i) {name}[_i] = {rhs_c};")

    def section_rhs(self, rhs):
        m = re.fullmatch(r"([a-z0-9_]+)\((\d+):\((.*)\),([a-z0-9_]+)\)", rhs.replace(" ", ""))
        if m:  # a(1:(n-1), k): element (lo - 1 + _i, k)
            name, lo, _, k = m.groups()
            return "(" + MODULE_ARRAYS[name].format(f"({lo}) - 1 + _i", k) + ")"
        return self.expr(rhs, idx="_i")

    def run(self, stmts):
        for label, st, no in stmts:
            try:
                self.one(label, st)
            except F2CError as e:
                raise F2CError(f"cliffs.f line {no}: {e}: '{st}'") from None
        return self.out

    def close_label(self, label):
        while self.stack and self.stack[-1][0] == "dolabel" and self.stack[-1][1] == label:
            self.emit(f"L{label}:;")
            self.ind -= 1
            self.emit("}")
            self.stack.pop()

    def one(self, label, st):
        if st.startswith("subroutine"):
            m = re.fullmatch(r"subroutine\s+([a-z0-9_]+)\((.*)\)", st)
            self.args = split_top(m.group(2))
            self.frees = []
            return
        if st.startswith("use ") or st == "implicit none":
            return
        m = DECL.match(st)
        if m and ("parameter" in st or find_assign(st) < 0):
            self.decl(m.group(1), m.group(2).strip())
            return
        if st.startswith("end subroutine"):
            if label:
                self.emit(f"L{label}:;")
            for f in self.frees:
                self.emit(f"free({f});")
            return
        if label and st == "continue":
            if self.stack and self.stack[-1][0] == "dolabel" and self.stack[-1][1] == label:
                self.close_label(label)
            else:
                self.emit(f"L{label}:;")
            return
        if label:
            self.emit(f"L{label}:;")
        m = re.fullmatch(r"if\s*\((.*)\)\s*then", st)
        if m:
            self.emit(f"if ({self.expr(m.group(1))}) {{")
            self.ind += 1
            self.stack.append(("if", None))
            return
        if st == "else":
            self.ind -= 1
            self.emit("} else {")
            self.ind += 1
            return
        m = re.fullmatch(r"else\s*if\s*\((.*)\)\s*then", st)
        if m:
            self.ind -= 1
            self.emit(f"}} else if ({self.expr(m.group(1))}) {{")
            self.ind += 1
            return
        if st in ("endif", "end if", "enddo", "end do", "end forall", "end where"):
            kind = self.stack.pop()[0]
            self.ind -= 1
            self.emit("}")
            return
        m = re.fullmatch(r"do\s+(\d+)\s+([a-z0-9_]+)\s*=\s*(.*)", st)
        if m:
            lo, hi = split_top(m.group(3))
            self.emit(f"for ({m.group(2)} = {self.expr(lo)}; {m.group(2)} <= {self.expr(hi)}; ++{m.group(2)}) {{")
            self.ind += 1
            self.stack.append(("dolabel", m.group(1)))
            return
        m = re.fullmatch(r"do\s+([a-z0-9_]+)\s*=\s*(.*)", st)
        if m:
            lo, hi = split_top(m.group(2))
            self.emit(f"for ({m.group(1)} = {self.expr(lo)}; {m.group(1)} <= {self.expr(hi)}; ++{m.group(1)}) {{")
            self.ind += 1
            self.stack.append(("do", None))
            return
        m = re.fullmatch(r"forall\s*\(\s*([a-z0-9_]+)\s*=\s*(.*):(.*)\)", st)
        if m:
            self.emit(f"for ({m.group(1)} = {self.expr(m.group(2))}; {m.group(1)} <= {self.expr(m.group(3))}; "
                      f"++{m.group(1)}) {{")
            self.ind += 1
            self.stack.append(("forall", None))
            return
        m = re.fullmatch(r"where\s*\((.*)\)", st)
        if m:
            mask = m.group(1).strip()
            if mask not in self.arrays:
                raise F2CError("where over an expression")
            self.emit(f"for (int _w = 1; _w <= {self.arrays[mask][0]}; ++_w) {{")
            self.ind += 1
            self.stack.append(("where", mask))
            return
        m = re.fullmatch(r"goto\s+(\d+)", st) or re.fullmatch(r"go\s+to\s+(\d+)", st)
        if m:
            self.emit(f"goto L{m.group(1)};")
            return
        m = re.fullmatch(r"if\s*\((.*)\)\s*(goto\s+\d+|[a-z].*)", st)
        if m and find_assign(st[:st.index("(")]) < 0:
            # one-line IF: find the condition's closing parenthesis
            depth, k = 0, st.index("(")
            for k in range(st.index("("), len(st)):
                depth += st[k] == "("
                depth -= st[k] == ")"
                if depth == 0:
                    break
            cond, rest = st[st.index("(") + 1:k], st[k + 1:].strip()
            self.emit(f"if ({self.expr(cond)}) {{")
            self.ind += 1
            self.one("", rest)
            self.ind -= 1
            self.emit("}")
            return
        if find_assign(st) > 0:
            if self.stack and self.stack[-1][0] == "where":
                mask = self.stack[-1][1]
                name = st[:find_assign(st)].strip()
                self.emit(f"if ({mask}[_w]) {name}[_w] = {self.expr(st[find_assign(st) + 1:], idx='_w')};")
                return
            self.assign(st)
            return
        raise F2CError("statement not translated")


HEADER = """/* Generated by oracle/ref_f2c.py from the reference's cliffs.f (subroutine
 * cliffs); not for version control.  Fortran semantics: 1-based arrays,
 * column-major module arrays, default-REAL literals rounded to float. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#define SQ(x) ((x) * (x))
#define IMAX(a, b) ((a) > (b) ? (a) : (b))

void ref_cliffs(int iu, int irw, int n, int nx, int ny, int mx, double *dep, double *cel, double *xvel,
                double *yvel, const double *s1, const double *s2, const double *zeta, const double *edge1,
                const double *edge2, double grav, double ground, double crough, double dt, double celmin) {
  (void)ny;
"""


def translate(src_path):
    with open(src_path) as f:
        text = f.read()
    stmts = statements(text)
    # the subroutine cliffs only
    i0 = next(k for k, s in enumerate(stmts) if s[1].startswith("subroutine cliffs"))
    i1 = next(k for k, s in enumerate(stmts) if s[1].startswith("end subroutine cliffs"))
    tr = Translator()
    body = tr.run(stmts[i0:i1 + 1])
    if tr.stack:
        raise F2CError(f"unclosed blocks: {tr.stack}")
    return HEADER + "\n".join(body) + "\n}\n"


# Where this recipe looks for the reference checkout when CLIFFS_REFERENCE is
# not set: the checkout beside the build container's repository.
DEFAULT_REFERENCE = "/root/reference"


def reference_dir(need="cliffs.f"):
    """The reference checkout ($CLIFFS_REFERENCE, else DEFAULT_REFERENCE) when
    it holds `need`; None elsewhere (the GPU hosts have no checkout)."""
    path = os.environ.get("CLIFFS_REFERENCE") or DEFAULT_REFERENCE
    return path if os.path.exists(os.path.join(path, need)) else None


def build(reference, force=False):
    src = os.path.join(reference, "cliffs.f")
    os.makedirs(REFDIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src),
                                                                         os.path.getmtime(__file__)):
        return LIB
    code = translate(src)
    with open(CSRC, "w") as f:
        f.write(code)
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O1", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    "-Wall", "-Wno-unused-label", "-Wno-unused-variable", "-Wno-unused-but-set-variable",
                    CSRC, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else reference_dir(), force=True))
