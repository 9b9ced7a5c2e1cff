"""Programmatic writer of .oso text (the format oslc emits and the
executor reads, see src/liboslexec/osogram.y in the reference).

Op indices and jump targets are filled in automatically:

    b = OsoBuilder("myshader")
    Cout = b.param("color", "Cout", 0, output=True)
    t = b.tmp("float")
    b.op("noise", t, b.const("string", "perlin"), b.glob("point", "P"))
    with b.if_(cond) as br:
        b.op("assign", Cout, t)
        br.else_()
        b.op("assign", Cout, b.const("float", 0))
    text = b.text()

`if` carries (else start, end); `for`/`while`/`dowhile` carry
(cond start, body start, step start, end) like oslc's output.
"""


class Sym(str):
    """A symbol name that remembers its type."""

    def __new__(cls, name, type_):
        s = str.__new__(cls, name)
        s.type = type_
        return s


def _fmt(v):
    if isinstance(v, str):
        return '"' + v.replace("\\", "\\\\").replace('"', '\\"') + '"'
    if isinstance(v, bool):
        return "1" if v else "0"
    if isinstance(v, int):
        return str(v)
    r = repr(float(v))
    return r[:-2] if r.endswith(".0") else r


class _If:
    def __init__(self, b, idx):
        self.b, self.idx, self.has_else = b, idx, False

    def __enter__(self):
        return self

    def else_(self):
        self.b.ops[self.idx][2][0] = len(self.b.ops)
        self.has_else = True

    def __exit__(self, *exc):
        end = len(self.b.ops)
        if not self.has_else:
            self.b.ops[self.idx][2][0] = end
        self.b.ops[self.idx][2][1] = end
        return False


class _Loop:
    """Sections must be entered in order: init, cond, body, step."""

    def __init__(self, b, idx):
        self.b, self.idx = b, idx

    def __enter__(self):
        return self

    def _mark(self, k):
        self.b.ops[self.idx][2][k] = len(self.b.ops)

    def cond(self):
        self._mark(0)

    def body(self):
        self._mark(1)

    def step(self):
        self._mark(2)

    def __exit__(self, *exc):
        self._mark(3)
        return False


class _Function:
    """A user function's inlined body: oslc wraps each call in a
    functioncall op whose jump is the end of the body; a return inside
    leaves the body."""

    def __init__(self, b, idx):
        self.b, self.idx = b, idx

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.b.ops[self.idx][2][0] = len(self.b.ops)
        return False


class OsoBuilder:
    def __init__(self, name, shadertype="shader"):
        self.name, self.shadertype = name, shadertype
        self.syms = []   # (kind, type, name, defaults, hints)
        self.ops = []    # [name, args, jumps]
        self._consts = {}
        self._globals = {}
        self._ntmp = 0
        self.init_code = {}  # param name -> list of ops (default-value code)

    def _add(self, kind, type_, name, defaults=(), hints=""):
        self.syms.append((kind, type_, name, list(defaults), hints))
        return Sym(name, type_)

    def param(self, type_, name, default=0, output=False, lockgeom=True):
        d = default if isinstance(default, (list, tuple)) else [default]
        hints = "" if lockgeom else "%meta{int,lockgeom,0}"
        return self._add("oparam" if output else "param", type_, name, d, hints)

    def glob(self, type_, name):
        if name not in self._globals:
            self._globals[name] = self._add("global", type_, name)
        return self._globals[name]

    def local(self, type_, name):
        return self._add("local", type_, name)

    def tmp(self, type_):
        self._ntmp += 1
        return self._add("temp", type_, "$tmp%d" % self._ntmp)

    def const(self, type_, value):
        vals = tuple(value) if isinstance(value, (list, tuple)) else (value,)
        key = (type_, vals)
        if key not in self._consts:
            self._consts[key] = self._add("const", type_, "$const%d" % (len(self._consts) + 1), vals)
        return self._consts[key]

    def op(self, name, *args):
        self.ops.append([name, [str(a) for a in args], []])
        return len(self.ops) - 1

    def if_(self, cond):
        self.ops.append(["if", [str(cond)], [0, 0]])
        return _If(self, len(self.ops) - 1)

    def function(self, name):
        """with b.function("f"): body ops (return = b.op("return"))."""
        self.ops.append(["functioncall", [str(self.const("string", name))], [0]])
        return _Function(self, len(self.ops) - 1)

    def loop(self, kind, cond):
        """kind: for | while | dowhile. Ops emitted before .cond() form the init block."""
        self.ops.append([kind, [str(cond)], [0, 0, 0, 0]])
        return _Loop(self, len(self.ops) - 1)

    def text(self):
        lines = ["OpenShadingLanguage 1.00", "# written by openshadinglanguage_gb300.oso",
                 "%s %s" % (self.shadertype, self.name)]
        for kind, type_, name, defaults, hints in self.syms:
            parts = [kind, type_, name]
            if kind in ("param", "oparam", "const"):
                parts += [_fmt(v) for v in defaults]
            if hints:
                parts.append(hints)
            lines.append("\t".join(parts))
        lines.append("code ___main___")
        for name, args, jumps in self.ops:
            lines.append("\t" + "\t".join([name] + args + [str(j) for j in jumps]))
        lines.append("\tend")
        return "\n".join(lines) + "\n"
