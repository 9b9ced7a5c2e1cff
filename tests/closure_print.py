"""Test-side printer of closure records in OSL's closure print format.

The executor stores a closure output as records: [count] then per
component [id][w.rgb][12 parameter words], the weight already multiplied
down the MUL chain (as the reference's print_closure does,
src/liboslexec/closure.cpp:104-130). This module renders those records the
way the reference's `%s` of a closure does (closure.cpp:70-100):
`(w.r, w.g, w.b) * name (p0, p1, "key", value)`, components joined by
"\\n\\t+ ", floats as C++ ostream prints them (6 significant digits).

Parameters are stored positionally (the closure op's arguments in order);
the printer applies the closure's registered layout: fixed parameters
first, then keyword pairs, the last value of a repeated keyword winning
(llvm_gen_closure's keyword matching). Strings are FNV-1a hashes on the
device; the printer maps them back through the strings a test names.
"""
import numpy as np

# closure name -> (fixed parameter types, keyword parameters (key, type)),
# as testshade registers them (src/testshade/simplerend.cpp:135-230)
LAYOUTS = {
    "emission": ([], []),
    "diffuse": (["vector"], [("label", "string")]),
    "phong": (["vector", "float"], [("label", "string")]),
    "transparent": ([], []),
    "debug": (["string"], []),
    "holdout": ([], []),
}

WORDS = {"float": 1, "int": 1, "string": 1, "vector": 3, "color": 3}


def fnv1a(s):
    h = 2166136261
    for c in s.encode():
        h ^= c
        h = (h * 16777619) & 0xFFFFFFFF
    return h


def g6(x):
    """C++ `ostream << float` with the default precision: %g of the value."""
    return "%g" % float(np.float32(x))


class Printer:
    def __init__(self, names_by_id, strings=()):
        self.names = names_by_id
        self.strings = {fnv1a(s): s for s in strings}

    def value(self, t, w):
        if t == "float":
            return g6(w[:1].view(np.float32)[0])
        if t == "int":
            return str(int(w[:1].view(np.int32)[0]))
        if t == "string":
            return '"%s"' % self.strings[int(w[0])]
        f = w[:3].view(np.float32)
        return "(%s, %s, %s)" % (g6(f[0]), g6(f[1]), g6(f[2]))

    def component(self, rec):
        """rec: 16 uint32 words of one stored component."""
        cid = int(rec[0])
        name = self.names[cid]
        fixed, keys = LAYOUTS[name]
        w = rec[1:4].view(np.float32)
        p = rec[4:16]
        parts, k = [], 0
        for t in fixed:
            parts.append(self.value(t, p[k:]))
            k += WORDS[t]
        kw = {}
        ktypes = dict(keys)
        while k < len(p) and int(p[k]) in self.strings and self.strings[int(p[k])] in ktypes:
            key = self.strings[int(p[k])]
            kw[key] = self.value(ktypes[key], p[k + 1:])
            k += 1 + WORDS[ktypes[key]]
        for key, _ in keys:
            if key in kw:
                parts.append('"%s", %s' % (key, kw[key]))
        return "(%s, %s, %s) * %s (%s)" % (g6(w[0]), g6(w[1]), g6(w[2]), name, ", ".join(parts))

    def closure(self, words):
        """words: the uint32 record block of one closure output of one point."""
        n = int(words[0])
        return "\n\t+ ".join(self.component(words[1 + 16 * i: 17 + 16 * i]) for i in range(n))


def printed_states(text, marker):
    """The closures a reference run printed after `marker` ("Ci = "), in
    order: a state is the rest of the marker's line plus the "\\t+ " lines
    that follow it."""
    states = []
    for line in text.splitlines():
        if marker in line:
            states.append(line.split(marker, 1)[1])
        elif line.startswith("\t+ ") and states:
            states[-1] += "\n" + line
    return states
