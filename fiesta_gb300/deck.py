"""FIESTA input decks -> fst_config.

FIESTA reads its deck, a Lua script, with an embedded Lua VM
(src/luaReader.cpp): it pre-creates the table ``fiesta`` with the
sub-tables ``ceq noise restart bc time viscosity buoyancy grid mpi hdf5 eos
progress status`` (src/luaReader.cpp:39-71), runs the script, then pulls
keys out of ``fiesta`` with or without defaults (src/input.cpp:136-284) and
the species list (src/luaReader.cpp:163-209).  ``fiesta.initial_conditions
(x, y, z, v)`` is then called once per interior cell and conserved variable
(src/input.cpp:453-515).

This module evaluates the subset of Lua that decks are written in --
assignments (global, ``local``, several targets), table constructors, field
and index access, arithmetic, comparison, logic, string concatenation, the
``math`` library, and function definitions with ``local``/``if``/``for``/
``while``/``return`` bodies -- in Python, and maps the keys onto
``abi.FstConfig`` with the reference's defaults, required keys and error
texts.  It is host-side setup, not part of the right-hand-side path.

The library's own keys live in ``fiesta.gb300``::

    fiesta.gb300 = {mode = "mixed", audit_every = 20, classify_every = 4}

``mode`` is ``"plain"`` (FP64, bit-identical to the reference; default),
``"mixed"`` or ``"hybrid"``.  Older FIESTA builds ignore the table.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

from . import abi


class DeckError(Exception):
    """A deck the reference would reject, or a construct outside the subset."""


# ---------------------------------------------------------------------------
# values
# ---------------------------------------------------------------------------
class LuaTable:
    """A Lua table: hash part in a dict; integer keys are ordinary keys."""

    def __init__(self):
        self.h = {}

    def get(self, k):
        if isinstance(k, float) and k.is_integer():
            k = int(k)
        return self.h.get(k)

    def set(self, k, v):
        if k is None:
            raise DeckError("table index is nil")
        if isinstance(k, float) and k.is_integer():
            k = int(k)
        if v is None:
            self.h.pop(k, None)
        else:
            self.h[k] = v

    def length(self):  # the border of the sequence part, as lua_rawlen
        n = 0
        while (n + 1) in self.h:
            n += 1
        return n

    def __repr__(self):
        return f"LuaTable({self.h!r})"


class LuaFunction:
    def __init__(self, name, params, body, closure):
        self.name, self.params, self.body, self.closure = name, params, body, closure

    def __repr__(self):
        return f"<lua function {self.name}>"


class _Return(Exception):
    def __init__(self, values):
        self.values = values


class _Break(Exception):
    pass


# ---------------------------------------------------------------------------
# lexer
# ---------------------------------------------------------------------------
_KEYWORDS = {"and", "break", "do", "else", "elseif", "end", "false", "for", "function", "if",
             "in", "local", "nil", "not", "or", "repeat", "return", "then", "true", "until",
             "while"}
_TOKEN = re.compile(r"""
    (?P<ws>[ \t\r\n]+) |
    (?P<lcomment>--\[(?P<leq>=*)\[.*?\](?P=leq)\]) |
    (?P<comment>--[^\n]*) |
    (?P<num>0[xX][0-9a-fA-F]+|(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?) |
    (?P<lstr>\[(?P<seq>=*)\[.*?\](?P=seq)\]) |
    (?P<str>"(?:[^"\\\n]|\\.)*"|'(?:[^'\\\n]|\\.)*') |
    (?P<name>[A-Za-z_][A-Za-z0-9_]*) |
    (?P<op>\.\.\.|\.\.|==|~=|<=|>=|//|[-+*/%^\#<>=(){}\[\];:,.])
""", re.S | re.X)
_ESC = {"n": "\n", "t": "\t", "r": "\r", "\\": "\\", '"': '"', "'": "'", "a": "\a",
        "b": "\b", "f": "\f", "v": "\v", "0": "\0"}


def _unescape(s):
    out, i = [], 0
    while i < len(s):
        c = s[i]
        if c == "\\" and i + 1 < len(s):
            out.append(_ESC.get(s[i + 1], s[i + 1]))
            i += 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _lex(src):
    toks, pos, line = [], 0, 1
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise DeckError(f"line {line}: unexpected character {src[pos]!r}")
        kind = m.lastgroup
        text = m.group(0)
        if kind == "num":
            v = int(text, 16) if text[:2] in ("0x", "0X") else (
                float(text) if any(c in text for c in ".eE") else int(text))
            toks.append(("num", v, line))
        elif kind == "str":
            toks.append(("str", _unescape(text[1:-1]), line))
        elif kind == "lstr":
            n = len(m.group("seq")) + 2
            body = text[n:-n]
            toks.append(("str", body[1:] if body.startswith("\n") else body, line))
        elif kind == "name":
            toks.append(("kw" if text in _KEYWORDS else "name", text, line))
        elif kind == "op":
            toks.append(("op", text, line))
        line += text.count("\n")
        pos = m.end()
    toks.append(("eof", None, line))
    return toks


# ---------------------------------------------------------------------------
# parser: statements and expressions become nested tuples
# ---------------------------------------------------------------------------
_BINARY = {  # operator: (left priority, right priority), Lua 5.3's table
    "or": (1, 1), "and": (2, 2),
    "<": (3, 3), ">": (3, 3), "<=": (3, 3), ">=": (3, 3), "~=": (3, 3), "==": (3, 3),
    "..": (9, 8),  # right associative
    "+": (10, 10), "-": (10, 10),
    "*": (11, 11), "/": (11, 11), "//": (11, 11), "%": (11, 11),
    "^": (14, 13),  # right associative
}
_UNARY_PRIORITY = 12


class _Parser:
    def __init__(self, src):
        self.t = _lex(src)
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def check(self, kind, val=None):
        tok = self.peek()
        return tok[0] == kind and (val is None or tok[1] == val)

    def accept(self, kind, val=None):
        if self.check(kind, val):
            return self.next()
        return None

    def expect(self, kind, val=None):
        tok = self.next()
        if tok[0] != kind or (val is not None and tok[1] != val):
            raise DeckError(f"line {tok[2]}: expected {val or kind}, found {tok[1]!r}")
        return tok

    # -- blocks ------------------------------------------------------------
    def chunk(self):
        body = self.block()
        if not self.check("eof"):
            tok = self.peek()
            raise DeckError(f"line {tok[2]}: unexpected {tok[1]!r}")
        return body

    def block(self):
        stmts = []
        while True:
            if self.check("eof") or (self.check("kw") and self.peek()[1] in
                                     ("end", "else", "elseif", "until")):
                return stmts
            if self.check("kw", "return"):
                self.next()
                vals = []
                if not (self.check("eof") or self.check("op", ";") or (
                        self.check("kw") and self.peek()[1] in ("end", "else", "elseif",
                                                                "until"))):
                    vals = self.exprlist()
                self.accept("op", ";")
                stmts.append(("return", vals))
                return stmts
            s = self.statement()
            if s is not None:
                stmts.append(s)

    def statement(self):
        tok = self.peek()
        line = tok[2]
        if self.accept("op", ";"):
            return None
        if tok[0] == "kw":
            kw = tok[1]
            if kw == "local":
                self.next()
                if self.accept("kw", "function"):
                    name = self.expect("name")[1]
                    return ("localfunc", name, self.funcbody(name))
                names = [self.expect("name")[1]]
                while self.accept("op", ","):
                    names.append(self.expect("name")[1])
                vals = self.exprlist() if self.accept("op", "=") else []
                return ("local", names, vals)
            if kw == "function":
                self.next()
                path = [self.expect("name")[1]]
                while self.accept("op", "."):
                    path.append(self.expect("name")[1])
                if self.accept("op", ":"):
                    raise DeckError(f"line {line}: methods are outside the deck subset")
                return ("funcdef", path, self.funcbody(".".join(path)))
            if kw == "if":
                self.next()
                arms = []
                cond = self.expr()
                self.expect("kw", "then")
                arms.append((cond, self.block()))
                other = None
                while True:
                    if self.accept("kw", "elseif"):
                        c = self.expr()
                        self.expect("kw", "then")
                        arms.append((c, self.block()))
                    elif self.accept("kw", "else"):
                        other = self.block()
                        self.expect("kw", "end")
                        break
                    else:
                        self.expect("kw", "end")
                        break
                return ("if", arms, other)
            if kw == "while":
                self.next()
                c = self.expr()
                self.expect("kw", "do")
                b = self.block()
                self.expect("kw", "end")
                return ("while", c, b)
            if kw == "repeat":
                self.next()
                b = self.block()
                self.expect("kw", "until")
                return ("repeat", b, self.expr())
            if kw == "do":
                self.next()
                b = self.block()
                self.expect("kw", "end")
                return ("do", b)
            if kw == "for":
                self.next()
                n1 = self.expect("name")[1]
                if self.accept("op", "="):
                    a = self.expr()
                    self.expect("op", ",")
                    b = self.expr()
                    c = self.expr() if self.accept("op", ",") else ("const", 1)
                    self.expect("kw", "do")
                    body = self.block()
                    self.expect("kw", "end")
                    return ("fornum", n1, a, b, c, body)
                names = [n1]
                while self.accept("op", ","):
                    names.append(self.expect("name")[1])
                self.expect("kw", "in")
                it = self.exprlist()
                self.expect("kw", "do")
                body = self.block()
                self.expect("kw", "end")
                return ("forin", names, it, body)
            if kw == "break":
                self.next()
                return ("break",)
        # assignment or call
        e = self.suffixedexp()
        if self.check("op", "=") or self.check("op", ","):
            targets = [e]
            while self.accept("op", ","):
                targets.append(self.suffixedexp())
            self.expect("op", "=")
            for t in targets:
                if t[0] not in ("name", "index"):
                    raise DeckError(f"line {line}: cannot assign to this expression")
            return ("assign", targets, self.exprlist())
        if e[0] != "call":
            raise DeckError(f"line {line}: syntax error near {self.peek()[1]!r}")
        return ("callstat", e)

    def funcbody(self, name):
        self.expect("op", "(")
        params = []
        if not self.check("op", ")"):
            while True:
                if self.accept("op", "..."):
                    params.append("...")
                    break
                params.append(self.expect("name")[1])
                if not self.accept("op", ","):
                    break
        self.expect("op", ")")
        body = self.block()
        self.expect("kw", "end")
        return ("function", name, params, body)

    # -- expressions -------------------------------------------------------
    def exprlist(self):
        es = [self.expr()]
        while self.accept("op", ","):
            es.append(self.expr())
        return es

    def expr(self, limit=0):
        tok = self.peek()
        if (tok[0] == "kw" and tok[1] == "not") or (tok[0] == "op" and tok[1] in ("-", "#")):
            self.next()
            left = ("unop", tok[1], self.expr(_UNARY_PRIORITY))
        else:
            left = self.simpleexp()
        while True:
            tok = self.peek()
            op = tok[1] if tok[0] in ("op", "kw") else None
            if op not in _BINARY or _BINARY[op][0] <= limit:
                return left
            self.next()
            right = self.expr(_BINARY[op][1])
            left = ("binop", op, left, right)

    def simpleexp(self):
        tok = self.peek()
        if tok[0] == "num":
            self.next()
            return ("const", tok[1])
        if tok[0] == "str":
            self.next()
            return ("const", tok[1])
        if tok[0] == "kw":
            if tok[1] == "nil":
                self.next()
                return ("const", None)
            if tok[1] == "true":
                self.next()
                return ("const", True)
            if tok[1] == "false":
                self.next()
                return ("const", False)
            if tok[1] == "function":
                self.next()
                return self.funcbody("anonymous")
        if self.check("op", "{"):
            return self.table()
        if self.check("op", "..."):
            raise DeckError(f"line {tok[2]}: varargs are outside the deck subset")
        return self.suffixedexp()

    def primaryexp(self):
        tok = self.next()
        if tok[0] == "name":
            return ("name", tok[1])
        if tok[0] == "op" and tok[1] == "(":
            e = self.expr()
            self.expect("op", ")")
            return ("paren", e)
        raise DeckError(f"line {tok[2]}: unexpected {tok[1]!r}")

    def suffixedexp(self):
        e = self.primaryexp()
        while True:
            if self.accept("op", "."):
                e = ("index", e, ("const", self.expect("name")[1]))
            elif self.accept("op", "["):
                k = self.expr()
                self.expect("op", "]")
                e = ("index", e, k)
            elif self.check("op", "("):
                self.next()
                args = [] if self.check("op", ")") else self.exprlist()
                self.expect("op", ")")
                e = ("call", e, args)
            elif self.check("str"):
                e = ("call", e, [("const", self.next()[1])])
            elif self.check("op", "{"):
                e = ("call", e, [self.table()])
            elif self.check("op", ":"):
                raise DeckError(f"line {self.peek()[2]}: methods are outside the deck subset")
            else:
                return e

    def table(self):
        self.expect("op", "{")
        items = []
        while not self.check("op", "}"):
            if self.check("op", "["):
                self.next()
                k = self.expr()
                self.expect("op", "]")
                self.expect("op", "=")
                items.append(("kv", k, self.expr()))
            elif self.check("name") and self.peek(1)[0] == "op" and self.peek(1)[1] == "=":
                k = self.next()[1]
                self.next()
                items.append(("kv", ("const", k), self.expr()))
            else:
                items.append(("pos", self.expr()))
            if not (self.accept("op", ",") or self.accept("op", ";")):
                break
        self.expect("op", "}")
        return ("table", items)


# ---------------------------------------------------------------------------
# evaluator
# ---------------------------------------------------------------------------
def _num(v, what="arithmetic"):
    if isinstance(v, bool) or v is None:
        raise DeckError(f"attempt to perform {what} on a {_type(v)} value")
    if isinstance(v, (int, float)):
        return v
    if isinstance(v, str):  # Lua coerces numeric strings
        try:
            return float(v) if any(c in v for c in ".eEnN") else int(v)
        except ValueError:
            pass
    raise DeckError(f"attempt to perform {what} on a {_type(v)} value")


def _type(v):
    if v is None:
        return "nil"
    if isinstance(v, bool):
        return "boolean"
    if isinstance(v, (int, float)):
        return "number"
    if isinstance(v, str):
        return "string"
    if isinstance(v, LuaTable):
        return "table"
    return "function"


def _truthy(v):
    return v is not None and v is not False


def _tostr(v):
    if isinstance(v, float):
        if v.is_integer() and abs(v) < 1e16:
            return f"{v:.1f}"
        return f"{v:.14g}"
    if isinstance(v, (int, str)):
        return str(v)
    raise DeckError(f"attempt to concatenate a {_type(v)} value")


def _arith(op, a, b):
    a, b = _num(a), _num(b)
    both_int = isinstance(a, int) and isinstance(b, int)
    if op == "+":
        return a + b
    if op == "-":
        return a - b
    if op == "*":
        return a * b
    if op == "/":
        a, b = float(a), float(b)
        if b == 0.0:
            if a == 0.0 or a != a:
                return math.nan
            return math.copysign(math.inf, a) * math.copysign(1.0, b)
        return a / b
    if op == "^":
        return math.pow(float(a), float(b))
    if op == "//":
        if both_int:
            if b == 0:
                raise DeckError("attempt to perform 'n//0'")
            return a // b
        return math.floor(float(a) / float(b)) if b != 0 else _arith("/", a, b)
    if op == "%":
        if both_int:
            if b == 0:
                raise DeckError("attempt to perform 'n%%0'")
            return a % b
        a, b = float(a), float(b)
        return a - math.floor(a / b) * b if b != 0 else math.nan
    raise DeckError(f"unknown operator {op}")


class _Scope:
    def __init__(self, parent=None):
        self.vars, self.parent = {}, parent

    def find(self, name):
        s = self
        while s is not None:
            if name in s.vars:
                return s
            s = s.parent
        return None


def _math_table():
    m = LuaTable()
    def f1(fn):
        return lambda *a: fn(float(_num(a[0] if a else None)))
    for name, fn in (("sqrt", math.sqrt), ("sin", math.sin), ("cos", math.cos),
                     ("tan", math.tan), ("asin", math.asin), ("acos", math.acos),
                     ("exp", math.exp), ("abs", abs)):
        m.set(name, f1(fn))
    m.set("atan", lambda y, x=1.0: math.atan2(float(_num(y)), float(_num(x))))
    m.set("log", lambda x, b=None: math.log(float(_num(x))) if b is None
          else math.log(float(_num(x)), float(_num(b))))
    m.set("floor", lambda x: math.floor(_num(x)))
    m.set("ceil", lambda x: math.ceil(_num(x)))
    m.set("fmod", lambda a, b: math.fmod(float(_num(a)), float(_num(b))))
    m.set("min", lambda *a: min(_num(x) for x in a))
    m.set("max", lambda *a: max(_num(x) for x in a))
    m.set("tanh", lambda x: math.tanh(float(_num(x))))
    m.set("pi", math.pi)
    m.set("huge", math.inf)
    return m


class LuaState:
    """Globals plus an evaluator for the deck subset."""

    def __init__(self):
        self.g = _Scope()
        self.g.vars["math"] = _math_table()
        self.g.vars["print"] = lambda *a: None
        self.g.vars["tostring"] = lambda v: _tostr(v)
        self.g.vars["tonumber"] = lambda v: _num(v) if v is not None else None
        self.g.vars["type"] = lambda v: _type(v)
        self.steps = 0

    # -- statements ----------------------------------------------------------
    def run(self, stmts, scope):
        for s in stmts:
            self.exec(s, scope)

    def exec(self, s, scope):
        self.steps += 1
        if self.steps > 50_000_000:
            raise DeckError("deck evaluation did not finish (step limit)")
        kind = s[0]
        if kind == "assign":
            vals = self.evalmulti(s[2], scope, len(s[1]))
            for t, v in zip(s[1], vals):
                self.assign(t, v, scope)
        elif kind == "local":
            vals = self.evalmulti(s[2], scope, len(s[1]))
            for n, v in zip(s[1], vals):
                scope.vars[n] = v
        elif kind == "localfunc":
            scope.vars[s[1]] = None
            scope.vars[s[1]] = self.eval(s[2], scope)
        elif kind == "funcdef":
            fn = self.eval(s[2], scope)
            if len(s[1]) == 1:
                self.assign(("name", s[1][0]), fn, scope)
            else:
                t = self.eval(("name", s[1][0]), scope)
                for k in s[1][1:-1]:
                    t = self.index(t, k)
                self.setindex(t, s[1][-1], fn)
        elif kind == "callstat":
            self.eval(s[1], scope)
        elif kind == "if":
            for cond, body in s[1]:
                if _truthy(self.eval(cond, scope)):
                    self.run(body, _Scope(scope))
                    return
            if s[2] is not None:
                self.run(s[2], _Scope(scope))
        elif kind == "while":
            try:
                while _truthy(self.eval(s[1], scope)):
                    self.run(s[2], _Scope(scope))
            except _Break:
                pass
        elif kind == "repeat":
            try:
                while True:
                    inner = _Scope(scope)
                    self.run(s[1], inner)
                    if _truthy(self.eval(s[2], inner)):
                        break
            except _Break:
                pass
        elif kind == "do":
            self.run(s[1], _Scope(scope))
        elif kind == "fornum":
            a, b, c = (_num(self.eval(e, scope)) for e in s[2:5])
            if c == 0:
                raise DeckError("'for' step is zero")
            v = a
            try:
                while (c > 0 and v <= b) or (c < 0 and v >= b):
                    inner = _Scope(scope)
                    inner.vars[s[1]] = v
                    self.run(s[5], inner)
                    v = v + c
            except _Break:
                pass
        elif kind == "forin":
            it = self.evalmulti(s[2], scope, 3)
            f, st, ctl = it
            try:
                while True:
                    vals = self.call(f, [st, ctl])
                    if not vals or vals[0] is None:
                        break
                    ctl = vals[0]
                    inner = _Scope(scope)
                    for i, n in enumerate(s[1]):
                        inner.vars[n] = vals[i] if i < len(vals) else None
                    self.run(s[3], inner)
            except _Break:
                pass
        elif kind == "return":
            raise _Return(self.evalmulti(s[1], scope, None))
        elif kind == "break":
            raise _Break()
        else:
            raise DeckError(f"statement {kind} is outside the deck subset")

    def assign(self, target, v, scope):
        if target[0] == "name":
            sc = scope.find(target[1]) or self.g
            sc.vars[target[1]] = v
        else:
            self.setindex(self.eval(target[1], scope), self.eval(target[2], scope), v)

    def index(self, t, k):
        if isinstance(t, LuaTable):
            return t.get(k)
        if isinstance(t, str) and k == "len":
            return lambda s: len(s)
        raise DeckError(f"attempt to index a {_type(t)} value (key {k!r})")

    def setindex(self, t, k, v):
        if not isinstance(t, LuaTable):
            raise DeckError(f"attempt to index a {_type(t)} value (key {k!r})")
        t.set(k, v)

    # -- expressions -----------------------------------------------------------
    def evalmulti(self, exprs, scope, want):
        vals = []
        for n, e in enumerate(exprs):
            if n == len(exprs) - 1 and e[0] == "call":
                vals.extend(self.eval_call(e, scope))
            else:
                vals.append(self.eval(e, scope))
        if want is not None:
            vals = (vals + [None] * want)[:want]
        return vals

    def eval(self, e, scope):
        kind = e[0]
        if kind == "const":
            return e[1]
        if kind == "name":
            sc = scope.find(e[1])
            return sc.vars[e[1]] if sc else None
        if kind == "index":
            return self.index(self.eval(e[1], scope), self.eval(e[2], scope))
        if kind == "paren":
            return self.eval(e[1], scope)
        if kind == "call":
            r = self.eval_call(e, scope)
            return r[0] if r else None
        if kind == "function":
            return LuaFunction(e[1], e[2], e[3], scope)
        if kind == "table":
            t, n = LuaTable(), 0
            for idx, item in enumerate(e[1]):
                if item[0] == "kv":
                    t.set(self.eval(item[1], scope), self.eval(item[2], scope))
                else:
                    last = idx == len(e[1]) - 1
                    vals = self.evalmulti([item[1]], scope, None) if last else \
                        [self.eval(item[1], scope)]
                    for v in vals:
                        n += 1
                        t.set(n, v)
            return t
        if kind == "unop":
            v = self.eval(e[2], scope)
            if e[1] == "not":
                return not _truthy(v)
            if e[1] == "-":
                return -_num(v)
            if isinstance(v, str):
                return len(v)
            if isinstance(v, LuaTable):
                return v.length()
            raise DeckError(f"attempt to get length of a {_type(v)} value")
        if kind == "binop":
            op = e[1]
            if op == "and":
                a = self.eval(e[2], scope)
                return self.eval(e[3], scope) if _truthy(a) else a
            if op == "or":
                a = self.eval(e[2], scope)
                return a if _truthy(a) else self.eval(e[3], scope)
            a, b = self.eval(e[2], scope), self.eval(e[3], scope)
            if op == "==":
                return _eq(a, b)
            if op == "~=":
                return not _eq(a, b)
            if op in ("<", "<=", ">", ">="):
                if isinstance(a, str) and isinstance(b, str):
                    pass
                else:
                    a, b = _num(a, "comparison"), _num(b, "comparison")
                return {"<": a < b, "<=": a <= b, ">": a > b, ">=": a >= b}[op]
            if op == "..":
                return _tostr(a) + _tostr(b)
            return _arith(op, a, b)
        raise DeckError(f"expression {kind} is outside the deck subset")

    def eval_call(self, e, scope):
        f = self.eval(e[1], scope)
        args = self.evalmulti(e[2], scope, None)
        return self.call(f, args)

    def call(self, f, args):
        if isinstance(f, LuaFunction):
            inner = _Scope(f.closure)
            for i, p in enumerate(f.params):
                if p == "...":
                    break
                inner.vars[p] = args[i] if i < len(args) else None
            try:
                self.run(f.body, inner)
            except _Return as r:
                return r.values
            return []
        if callable(f):
            r = f(*args)
            return list(r) if isinstance(r, tuple) else [r]
        raise DeckError(f"attempt to call a {_type(f)} value")


def _eq(a, b):
    if isinstance(a, bool) or isinstance(b, bool):
        return a is b
    if isinstance(a, (int, float)) and isinstance(b, (int, float)):
        return a == b
    return a is b if isinstance(a, LuaTable) else a == b


# ---------------------------------------------------------------------------
# the deck
# ---------------------------------------------------------------------------
_PRESET_TABLES = ("ceq", "noise", "restart", "bc", "time", "viscosity", "buoyancy", "grid",
                  "mpi", "hdf5", "eos", "progress", "status")

_MODES = {"plain": abi.MODE_PLAIN_FP64, "fp64": abi.MODE_PLAIN_FP64,
          "mixed": abi.MODE_MIXED, "hybrid": abi.MODE_HYBRID}


def parse_bc(name):
    """parseBC (src/bc.cpp:251-270): case, '-', '_' and ' ' are ignored."""
    if not isinstance(name, str):
        raise DeckError(f"Unknown boundary condition '{name}'")
    key = name.lower().replace("-", "").replace("_", "").replace(" ", "")
    if key not in abi.BC_NAMES:
        raise DeckError(f"Unknown boundary condition '{name}'")
    return abi.BC_NAMES[key]


@dataclass
class Deck:
    """What FIESTA's input stage reads, for the right-hand-side path."""
    filename: str
    title: str = ""
    ndim: int = 2
    ni: list = field(default_factory=list)
    dx: list = field(default_factory=list)
    procs: list = field(default_factory=list)
    dt: float = 0.0
    nt: int = 0
    R: float = 8.314462
    species: list = field(default_factory=list)
    visc: bool = False
    ceq: bool = False
    kap: float = 0.0
    eps: float = 0.0
    alpha: float = 0.0
    beta: float = 0.0
    betae: float = 0.0
    buoyancy: bool = False
    g_accel: float = 0.0
    rho_ref: float = 0.0
    periodic: tuple = (False, False, False)
    bcs: tuple = (0, 0, 0, 0, 0, 0)
    noise: bool = False
    noise_dh: float = 0.0
    noise_eta: float = 0.0
    noise_coff: float = 0.0
    noise_nt: int = 1
    noise_mode: int = 1
    scheme: str = "weno5"
    grid: str = "cartesian"
    tdx: float = 0.0        # terrain: node spacing in x (fiesta.tdx)
    tdy: float = 0.0        # terrain: node spacing in y (fiesta.tdy)
    h: float = 0.0          # terrain: height of the domain top (fiesta.h)
    ng: int = 3
    mode: int = abi.MODE_PLAIN_FP64
    audit_every: int = 0
    classify_every: int = 1
    lua: LuaState | None = None

    def config(self):
        """The fst_config of this deck (abi.FstConfig)."""
        n = list(self.ni) + [1] * (3 - len(self.ni))
        gen = self.grid in ("generalized", "terrain")
        # generalized grids run in computational space: dx = dy = dz = 1
        # (src/input.cpp:344-350)
        dx = [1.0, 1.0, 1.0] if gen else list(self.dx) + [self.dx[0]] * (3 - len(self.dx))
        return abi.make_config(self.ndim, n, dt=self.dt, species=self.species, R=self.R,
                               visc=self.visc, ceq=self.ceq, kap=self.kap, eps=self.eps,
                               alpha=self.alpha, buoyancy=self.buoyancy, g=self.g_accel,
                               rho_ref=self.rho_ref, periodic=self.periodic,
                               bcs=self.bcs, mode=self.mode, audit_every=self.audit_every,
                               dx=dx, classify_every=self.classify_every,
                               grid_type=abi.GRID_GENERALIZED if gen else abi.GRID_CARTESIAN,
                               scheme=_SCHEMES.get(self.scheme, abi.SCHEME_WENO5))

    def noise_params(self):
        """abi.FstNoiseParams of fiesta.noise, or None when the filter is off
        (or the module has none: gen3d_func::postStep, src/gen3d.cpp:111-128)."""
        if not self.noise or (self.grid == "generalized" and self.ndim == 3):
            return None
        return abi.FstNoiseParams(dh=self.noise_dh, eta=self.noise_eta, coff=self.noise_coff,
                                  nt=self.noise_nt, mode=self.noise_mode)

    def _call_number(self, name, args):
        """luaReader::call (src/luaReader.cpp:317-345): fiesta.<name>(...)
        must exist and return a number."""
        fn = _fiesta(self.lua).get(name)
        if fn is None:
            raise DeckError(f"Could not find fiesta.{name} in '{self.filename}'")
        r = self.lua.call(fn, args)
        val = r[0] if r else None
        try:
            return float(_num(val, "conversion"))
        except DeckError:
            raise DeckError(f"function '{name}' should return a number") from None

    def grid_nodes(self, cfg=None, height=None):
        """Node coordinates of a generalized grid, (ni, nj, nk, 3) with
        ni = nci + 1: ``fiesta.initialize_grid(i, j, k, v)`` for v < ndim at
        every node, as loadGrid (src/input.cpp:529-560) on one rank.  A
        terrain grid is built from the ground heights ``height`` (ni, nj),
        which the reference reads from its restart file's "Height" dataset
        (HDF5, not readable here), and fiesta.tdx / tdy / h."""
        import numpy as np
        cfg = cfg or self.config()
        if self.grid == "terrain":
            from .grids import terrain_nodes
            if height is None:
                raise DeckError("a terrain grid needs the ground heights (the 'Height' dataset "
                                "of the restart file): pass height=")
            return terrain_nodes(cfg, height, self.tdx, self.tdy, self.h)
        ni, nj, nk, _ = abi.grid_dims(cfg)
        X = np.zeros((ni, nj, nk, 3), order="F")
        for v in range(cfg.ndim):
            for k in range(nk):
                for j in range(nj):
                    for i in range(ni):
                        X[i, j, k, v] = self._call_number(
                            "initialize_grid", [float(i), float(j), float(k), float(v)])
        return X

    def initial_conditions(self, cfg=None, nodes=None):
        """Evaluate ``fiesta.initial_conditions(x, y, z, v)`` at every interior
        cell centre, as loadInitialConditions (src/input.cpp:453-515): uniform
        grids, x = dx*(i-ng) + 0.5*dx; generalized grids, the mean of the
        cell's nodes (``nodes`` from grid_nodes(), computed when not given);
        conserved variables v < nv only; ghosts and C-variables stay zero.
        Interpreted Python: for modest grids."""
        import numpy as np
        cfg = cfg or self.config()
        gen = cfg.grid_type == abi.GRID_GENERALIZED
        if gen and nodes is None:
            nodes = self.grid_nodes(cfg)
        ngi, ngj, ngk, nvt = abi.dims(cfg)
        nv = abi.nv_of(cfg)
        ng = cfg.ng
        U = np.zeros((ngi, ngj, ngk, nvt), order="F")
        ks = range(ng, cfg.nck + ng) if cfg.ndim == 3 else [0]

        def centre(i, j, k):
            if not gen:
                x = cfg.dx * (i - ng) + 0.5 * cfg.dx
                y = cfg.dy * (j - ng) + 0.5 * cfg.dy
                z = cfg.dz * (k - ng) + 0.5 * cfg.dz if cfg.ndim == 3 else 0.0
                return x, y, z
            x = y = z = 0.0
            if cfg.ndim == 3:
                for ix in range(2):
                    for iy in range(2):
                        for iz in range(2):
                            a, b, c = i + ix - ng, j + iy - ng, k + iz - ng
                            x += nodes[a, b, c, 0]
                            y += nodes[a, b, c, 1]
                            z += nodes[a, b, c, 2]
                return x / 8.0, y / 8.0, z / 8.0
            for ix in range(2):
                for iy in range(2):
                    x += nodes[i + ix - ng, j + iy - ng, 0, 0]
                    y += nodes[i + ix - ng, j + iy - ng, 0, 1]
            return x / 4.0, y / 4.0, 0.0

        for v in range(nv):
            for k in ks:
                for j in range(ng, cfg.ncj + ng):
                    for i in range(ng, cfg.nci + ng):
                        x, y, z = centre(i, j, k)
                        U[i, j, k, v] = self._call_number("initial_conditions",
                                                          [x, y, z, float(v)])
        return U


_SCHEMES = {"weno5": abi.SCHEME_WENO5, "centered4": abi.SCHEME_CENTERED4,
            "quick": abi.SCHEME_QUICK}


def _fiesta(lua):
    t = lua.g.vars.get("fiesta")
    if not isinstance(t, LuaTable):
        raise DeckError("the deck replaced the table 'fiesta'")
    return t


class _Reader:
    """luaReader::get with and without defaults (src/luaReader.cpp:78-161)."""

    def __init__(self, lua, filename):
        self.root = _fiesta(lua)
        self.filename = filename

    def lookup(self, keys):
        t = self.root
        for k in keys:
            if not isinstance(t, LuaTable):
                return None
            t = t.get(k)
            if t is None:
                return None
        return t

    def get(self, keys, kind, default=...):
        v = self.lookup(keys)
        if v is None:
            if default is ...:
                raise DeckError(f"Could not find required parameter "
                                f"'fiesta.{'.'.join(keys)}' in '{self.filename}'")
            return default
        return _convert(v, kind)

    def array(self, keys, n, kind):
        v = self.lookup(keys)
        if v is None:
            raise DeckError(f"Could not find required parameter "
                            f"'fiesta.{'.'.join(keys)}' in '{self.filename}'")
        if not isinstance(v, LuaTable):
            raise DeckError(f"fiesta.{'.'.join(keys)} is not a table")
        return [_convert(v.get(i + 1), kind) for i in range(n)]


def _convert(v, kind):
    """getValue (src/luaReader.cpp:352-375): lua_toboolean for bool (0 is
    true, as in Lua), lua_tointegerx for int (0 unless integral), number for
    the rest, the string itself for str."""
    if kind is bool:
        return _truthy(v)
    if kind is str:
        return v if isinstance(v, str) else (_tostr(v) if isinstance(v, (int, float)) else "")
    try:
        x = _num(v)
    except DeckError:
        return 0 if kind is int else 0.0
    if kind is int:
        return int(x) if float(x).is_integer() else 0
    if kind == "size":
        return int(x)
    return float(x)


def load(path=None, text=None):
    """Run a deck and read its keys (src/input.cpp:136-284, 163-209)."""
    if text is None:
        with open(path) as f:
            text = f.read()
    filename = path or "<string>"
    lua = LuaState()
    root = LuaTable()
    for name in _PRESET_TABLES:
        root.set(name, LuaTable())
    lua.g.vars["fiesta"] = root
    try:
        lua.run(_Parser(text).chunk(), lua.g)
    except (_Return, _Break):
        pass
    except RecursionError:
        raise DeckError("deck nesting too deep")
    rd = _Reader(lua, filename)
    d = Deck(filename=filename, lua=lua)
    d.title = rd.get(["title"], str)
    d.nt = rd.get(["time", "nt"], int, 0)
    d.dt = rd.get(["time", "dt"], float)
    if d.nt == 0:
        rd.get(["time", "tend"], int, 0)
    d.R = rd.get(["eos", "R"], float, 8.314462)
    d.ndim = rd.get(["grid", "ndim"], int, 2)
    if d.ndim not in (2, 3):
        raise DeckError(f"fiesta.grid.ndim must be 2 or 3, got {d.ndim}")
    d.visc = rd.get(["viscosity", "enabled"], bool, False)
    d.ng = rd.get(["ng"], int, 3)
    xper = rd.get(["bc", "xperiodic"], bool, False)
    yper = rd.get(["bc", "yperiodic"], bool, False)
    d.scheme = rd.get(["advection_scheme"], str, "weno5")
    d.grid = rd.get(["grid", "type"], str, "cartesian")
    d.dx = rd.array(["grid", "dx"], d.ndim, float)
    if d.grid == "terrain" and d.ndim == 3:  # src/input.cpp:294-302
        d.tdx = rd.get(["tdx"], float)
        d.tdy = rd.get(["tdy"], float)
        d.h = rd.get(["h"], float)
    d.ni = rd.array(["grid", "ni"], d.ndim, "size")
    d.procs = rd.array(["mpi", "procs"], d.ndim, "size")
    bcs = [abi.BC_OUTFLOW] * 6
    if not xper:
        bcs[0] = parse_bc(rd.get(["bc", "xmin"], str))
        bcs[1] = parse_bc(rd.get(["bc", "xmax"], str))
    if not yper:
        bcs[2] = parse_bc(rd.get(["bc", "ymin"], str))
        bcs[3] = parse_bc(rd.get(["bc", "ymax"], str))
    d.buoyancy = rd.get(["buoyancy", "enabled"], bool, False)
    if d.buoyancy:
        d.g_accel = rd.get(["buoyancy", "acceleration"], float, 9.81)
        d.rho_ref = rd.get(["buoyancy", "rho_reference"], float, 0.0)
    d.ceq = rd.get(["ceq", "enabled"], bool, False)
    if d.ceq:
        d.kap = rd.get(["ceq", "kappa"], float, 1.23456)
        d.eps = rd.get(["ceq", "epsilon"], float)
        d.alpha = rd.get(["ceq", "alpha"], float)
        d.beta = rd.get(["ceq", "beta"], float)
        d.betae = rd.get(["ceq", "betae"], float)
    d.noise = rd.get(["noise", "enabled"], bool, False)
    if d.noise:  # src/input.cpp:270-277
        d.noise_dh = rd.get(["noise", "dh"], float)
        d.noise_eta = rd.get(["noise", "eta"], float)
        d.noise_coff = rd.get(["noise", "coff"], float)
        d.noise_nt = rd.get(["noise", "nt"], int, 1)
        d.noise_mode = rd.get(["noise", "mode"], int, 1)
    zper = False
    if d.ndim == 3:
        zper = rd.get(["bc", "zperiodic"], bool, False)
        if not zper:
            bcs[4] = parse_bc(rd.get(["bc", "zmin"], str))
            bcs[5] = parse_bc(rd.get(["bc", "zmax"], str))
    d.periodic = (xper, yper, zper)
    d.bcs = tuple(bcs)
    # species (src/luaReader.cpp:163-209)
    sp = rd.lookup(["species"])
    if sp is None:
        raise DeckError(f"Could not find fiesta.species in '{filename}'")
    if not isinstance(sp, LuaTable):
        raise DeckError("Error Reading Input File: Could not read blocks.")
    for s in range(sp.length()):
        e = sp.get(s + 1)
        if not isinstance(e, LuaTable):
            raise DeckError(f"fiesta.species[{s + 1}] is not a table")
        d.species.append({k: _convert(e.get(k), float) for k in ("gamma", "M", "mu")})
    # this library's keys
    gb = rd.lookup(["gb300"])
    if isinstance(gb, LuaTable):
        m = gb.get("mode")
        if m is not None:
            if not isinstance(m, str) or m.lower() not in _MODES:
                raise DeckError(f"fiesta.gb300.mode must be one of {sorted(_MODES)}, got {m!r}")
            d.mode = _MODES[m.lower()]
        d.audit_every = _convert(gb.get("audit_every"), int) if gb.get("audit_every") is not None \
            else 0
        d.classify_every = _convert(gb.get("classify_every"), int) \
            if gb.get("classify_every") is not None else 1
    _check_supported(d)
    return d


def _check_supported(d):
    """What the library's right-hand side covers: cartesian and generalized
    grids; the three 2D advection schemes (an unknown scheme name leaves
    WENO5, as src/input.cpp:317-323 does); the 3D modules use WENO5."""
    if d.grid == "terrain" and d.ndim != 3:
        raise DeckError("ndim must be equal to 3 for terrain")  # src/input.cpp:303-305
    if d.grid not in ("cartesian", "generalized", "terrain"):
        raise DeckError(f"unknown fiesta.grid.type '{d.grid}'")
    if d.grid in ("generalized", "terrain"):
        if d.mode == abi.MODE_HYBRID or (d.mode == abi.MODE_MIXED and d.ndim != 3):
            raise DeckError("generalized grids run in the plain FP64 mode (and mixed in 3D)")
        if any(d.periodic[:d.ndim]):
            raise DeckError("periodic axes are not supported on generalized grids")
    if (d.ndim == 2 and _SCHEMES.get(d.scheme, 1) != abi.SCHEME_WENO5
            and d.mode != abi.MODE_PLAIN_FP64):
        raise DeckError(f"fiesta.advection_scheme '{d.scheme}' runs in the plain FP64 mode")
    if d.ng != 3:
        raise DeckError("fiesta.ng must be 3")
    if not d.species:
        raise DeckError("fiesta.species is empty")
    if len(d.species) > abi.FST_MAX_SPECIES:
        raise DeckError(f"at most {abi.FST_MAX_SPECIES} species")


def export(path, prefix, height=None):
    """Write what a C++ host needs to start a run of the deck at ``path``:
    ``<prefix>.cfg`` (the raw fst_config, read by fst::load_config in
    include/fst_module.hpp), ``<prefix>.U0`` (the initial state, LayoutLeft
    FP64), ``<prefix>.X`` (generalized and terrain grids: the node
    coordinates), ``<prefix>.noise`` (fiesta.noise on: the raw
    fst_noise_params, read by fst::load_noise) and ``<prefix>.json`` (a
    readable summary)."""
    import ctypes as C
    import json

    import numpy as np
    d = load(path)
    cfg = d.config()
    X = None
    if cfg.grid_type == abi.GRID_GENERALIZED:
        X = d.grid_nodes(cfg, height=height)
    U0 = d.initial_conditions(cfg, X)
    with open(prefix + ".cfg", "wb") as f:
        f.write(bytes(C.string_at(C.addressof(cfg), C.sizeof(cfg))))
    np.asfortranarray(U0).ravel(order="F").astype("<f8").tofile(prefix + ".U0")
    if X is not None:
        np.asfortranarray(X).ravel(order="F").astype("<f8").tofile(prefix + ".X")
    noise = d.noise_params()
    if noise is not None:
        with open(prefix + ".noise", "wb") as f:
            f.write(bytes(C.string_at(C.addressof(noise), C.sizeof(noise))))
    summary = {"deck": path, "title": d.title, "nt": d.nt, "dt": d.dt,
               "state_shape": list(abi.dims(cfg)), "grid": d.grid,
               "grid_shape": list(abi.grid_dims(cfg)) if X is not None else None,
               "noise": noise is not None, "config": abi.config_to_dict(cfg)}
    with open(prefix + ".json", "w") as f:
        json.dump(summary, f, indent=1)
    return summary


if __name__ == "__main__":
    import sys
    if len(sys.argv) != 3:
        sys.exit("usage: python -m fiesta_gb300.deck <deck.lua> <output prefix>")
    print(export(sys.argv[1], sys.argv[2])["state_shape"])
