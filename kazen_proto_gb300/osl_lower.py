"""Lowering of OSL surface shaders to kz_material records.

The reference compiles its .osl shaders with OSL and runs them per shading
point; process_closure (src/shading/bsdf.cpp:183-320 in kazen_proto) then
flattens the closure tree into weighted lobes plus emitted radiance. For
shaders whose closure weights do not depend on the shading point, that
result is a constant per material, and this module computes it once on the
host: it parses the shader source and evaluates its body over constant
inputs, in a subset of OSL large enough for the reference's own shaders
(resource/shader/src/principle.osl, disney_brdf.osl, ward.osl, lambert.osl,
emissive.osl and the scene shaders):

* parameters `[output] type name = expr [[metadata]]`, overridden by the
  group's <Parameter> values;
* statements: declarations, `=` `+=` `-=` `*=` `/=`, `if` / `else`,
  blocks, `return`;
* expressions: float and color arithmetic, comparisons, `&&` `||` `!`,
  `?:`, casts, component access (c[i], v.x, c.r), color()/vector()/
  normal()/point(), luminance (Rec. 709 weights, OSL's default colour
  space), clamp, mix, min, max, pow, sqrt, inversesqrt, abs, exp, exp2, log,
  log2, log10, floor, ceil, round, trunc, sign, fmod, mod, step,
  smoothstep, linearstep, the trigonometric functions, radians, degrees,
  hypot, dot, cross, length, distance, normalize;
* closures: sums of closures times colours or floats, mix() of closures.

The global N is the shading normal, (0, 1, 0) in the local frame the lobes
are evaluated in; assigning it (`N = bump_normal`) is recorded as a warning
and has no effect: lobes shade with the geometric normal. Other globals
(P, I, u, v, ...) and texture lookups make the shader position-dependent
and are rejected with ValueError.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from . import api

_TYPES = {"float", "int", "color", "vector", "normal", "point", "string", "closure", "matrix", "void"}
_COMPONENTS = {"x": 0, "y": 1, "z": 2, "r": 0, "g": 1, "b": 2}
_VEC_TYPES = {"color", "vector", "normal", "point"}
_TOKEN = re.compile(r"""
    (?P<ws>\s+|//[^\n]*|/\*.*?\*/)
  | (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?)
  | (?P<str>"(?:[^"\\]|\\.)*")
  | (?P<id>[A-Za-z_]\w*)
  | (?P<op>&&|\|\||==|!=|<=|>=|\+=|-=|\*=|/=|\[\[|\]\]|[-+*/<>=!?:(),;{}\[\]^%&|~.])
""", re.S | re.X)
LUMA = np.array([0.2126, 0.7152, 0.0722])


def tokenize(src: str):
    out, pos = [], 0
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise ValueError(f"OSL: unexpected character {src[pos]!r} at offset {pos}")
        pos = m.end()
        kind = m.lastgroup
        if kind != "ws":
            out.append((kind, m.group(kind)))
    out.append(("eof", ""))
    return out


# ---------------------------------------------------------------- values
class Normal:
    """The shading normal N (local +y)."""


class Global:
    """A shading-point global the lowering keeps symbolic: u, v (texture
    coordinates) or I (the ray direction, for environment lookups)."""

    def __init__(self, name):
        self.name = name


@dataclass
class TexRef:
    """A colour that varies over the surface: scale times a texture lookup.
    spec: ("image", filename), ("checker", scale_s, scale_t, Ca, Cb) or
    ("environment", filename)."""
    spec: tuple
    scale: np.ndarray = field(default_factory=lambda: np.ones(3))


@dataclass
class Closure:
    terms: list = field(default_factory=list)  # (weight np3, name, args, TexRef spec or None)

    def scaled(self, w, tex=None):
        w = np.asarray(w, np.float64)
        out = []
        for t in self.terms:
            if tex is not None and t[3] is not None:
                raise ValueError("OSL: a closure weighted by two textures is not lowered")
            out.append((t[0] * w, t[1], t[2], t[3] if tex is None else tex))
        return Closure(out)


def _is_num(v):
    return isinstance(v, (float, int, np.ndarray)) and not isinstance(v, bool)


def _zero(v):
    return _is_num(v) and np.all(np.asarray(v) == 0)


def binop(op, a, b):
    if isinstance(a, TexRef) or isinstance(b, TexRef):
        if op == "*":
            t, o = (a, b) if isinstance(a, TexRef) else (b, a)
            if isinstance(o, Closure):
                return o.scaled(t.scale, t.spec)
            if _is_num(o):
                return TexRef(t.spec, t.scale * np.asarray(o, np.float64))
        elif op == "/" and isinstance(a, TexRef) and _is_num(b):
            return TexRef(a.spec, a.scale / np.asarray(b, np.float64))
        raise ValueError(f"OSL: operator {op} on a texture lookup is not lowered (only scaling and closure weights)")
    if isinstance(a, Global) or isinstance(b, Global):
        raise ValueError("OSL: arithmetic on u, v or I is not lowered (texture coordinates pass through unchanged)")
    if isinstance(a, Closure) or isinstance(b, Closure):
        if op == "+":
            if isinstance(a, Closure) and isinstance(b, Closure):
                return Closure(a.terms + b.terms)
            if isinstance(a, Closure) and _zero(b):
                return a
            if isinstance(b, Closure) and _zero(a):
                return b
        elif op == "*":
            if isinstance(a, Closure) and _is_num(b):
                return a.scaled(b)
            if isinstance(b, Closure) and _is_num(a):
                return b.scaled(a)
        elif op == "/" and isinstance(a, Closure) and _is_num(b):
            return a.scaled(1.0 / np.asarray(b, np.float64))
        raise ValueError(f"OSL: operator {op} is not defined for these closure operands")
    if isinstance(a, Normal) or isinstance(b, Normal):
        raise ValueError("OSL: arithmetic on the shading normal N is not lowered")
    if isinstance(a, str) or isinstance(b, str):
        if op == "==":
            return float(a == b)
        if op == "!=":
            return float(a != b)
        raise ValueError("OSL: arithmetic on strings")
    a = np.asarray(a, np.float64) if isinstance(a, np.ndarray) else float(a)
    b = np.asarray(b, np.float64) if isinstance(b, np.ndarray) else float(b)
    if op == "+":
        return a + b
    if op == "-":
        return a - b
    if op == "*":
        return a * b
    if op == "/":
        with np.errstate(divide="ignore", invalid="ignore"):
            r = np.divide(a, b)
        return r if np.ndim(r) else float(r)
    cmp = {"<": np.less, ">": np.greater, "<=": np.less_equal, ">=": np.greater_equal, "==": np.equal,
           "!=": np.not_equal}[op]
    r = cmp(a, b)
    return float(np.all(r)) if op != "!=" else float(np.any(r))


def truth(v) -> bool:
    if isinstance(v, Closure):
        return bool(v.terms)
    if isinstance(v, str):
        return bool(v)
    return bool(np.any(np.asarray(v) != 0))


def convert(kind: str, v):
    """Assignment conversion to a declared type."""
    if isinstance(v, Global) and kind in ("float", "vector", "point", "normal"):
        return v
    if isinstance(v, TexRef) and kind == "color":
        return v
    if kind in _VEC_TYPES:
        if isinstance(v, Normal):
            return v
        if isinstance(v, np.ndarray):
            return v.astype(np.float64)
        if _is_num(v):
            return np.full(3, float(v))
        raise ValueError(f"OSL: cannot assign {type(v).__name__} to {kind}")
    if kind in ("float", "int"):
        if isinstance(v, np.ndarray):
            raise ValueError(f"OSL: cannot assign a triple to {kind}")
        if not _is_num(v):
            raise ValueError(f"OSL: cannot assign {type(v).__name__} to {kind}")
        return float(int(v)) if kind == "int" else float(v)
    if kind == "closure":
        if isinstance(v, Closure):
            return v
        if _zero(v):
            return Closure()
        raise ValueError("OSL: a closure variable takes a closure or 0")
    if kind == "string":
        if not isinstance(v, str):
            raise ValueError("OSL: cannot assign a number to a string")
        return v
    raise ValueError(f"OSL: type {kind} is not lowered")


def _triple(*args):
    if len(args) == 1:
        if isinstance(args[0], TexRef):
            return args[0]
        return convert("color", args[0])
    if len(args) == 3:
        return np.array([float(a) for a in args])
    if len(args) == 4 and isinstance(args[0], str):  # color("space", r, g, b): only rgb is lowered
        if args[0] not in ("rgb", "common", "world", "object", "shader"):
            raise ValueError(f"OSL: colour space {args[0]!r} is not lowered")
        return np.array([float(a) for a in args[1:]])
    raise ValueError("OSL: triple constructor takes 1 or 3 values")


def _mix(a, b, t):
    return binop("+", binop("*", a, binop("-", 1.0, t)), binop("*", b, t))


def _elementwise(fn):
    def f(*args):
        if any(isinstance(a, (Closure, Normal, str, TexRef, Global)) for a in args):
            raise ValueError("OSL: math function on a non-numeric value")
        r = fn(*[np.asarray(a, np.float64) for a in args])
        return r if np.ndim(r) else float(r)
    return f


def _texture(filename, s, t, *opts):
    """texture(filename, u, v): an image lookup at the hit's texture coordinates."""
    if not (isinstance(s, Global) and s.name == "u" and isinstance(t, Global) and t.name == "v"):
        raise ValueError("OSL: texture() is lowered at (u, v) only")
    if not isinstance(filename, str):
        raise ValueError("OSL: texture() takes a file name")
    return TexRef(("image", filename))


def _environment(filename, d, *opts):
    """environment(filename, I): a latitude-longitude lookup along the ray; an
    empty file name looks up nothing (black), as OIIO does."""
    if not (isinstance(d, Global) and d.name == "I"):
        raise ValueError("OSL: environment() is lowered along I only")
    if not filename:
        return 0.0
    return TexRef(("environment", filename))


FUNCS = {
    "texture": _texture, "environment": _environment,
    "color": _triple, "vector": _triple, "normal": _triple, "point": _triple,
    "luminance": lambda c: float(np.dot(convert("color", c), LUMA)),
    "clamp": _elementwise(lambda x, lo, hi: np.minimum(np.maximum(x, lo), hi)),
    "mix": _mix,
    "min": _elementwise(np.minimum), "max": _elementwise(np.maximum),
    "pow": _elementwise(np.power), "sqrt": _elementwise(np.sqrt), "abs": _elementwise(np.abs),
    "fabs": _elementwise(np.abs), "exp": _elementwise(np.exp), "log": _elementwise(np.log),
    "floor": _elementwise(np.floor), "ceil": _elementwise(np.ceil), "fmod": _elementwise(np.fmod),
    "mod": _elementwise(lambda a, b: a - b * np.floor(a / b)),
    "sin": _elementwise(np.sin), "cos": _elementwise(np.cos), "tan": _elementwise(np.tan),
    "asin": _elementwise(np.arcsin), "acos": _elementwise(np.arccos), "atan": _elementwise(np.arctan),
    "atan2": _elementwise(np.arctan2), "radians": _elementwise(np.radians), "degrees": _elementwise(np.degrees),
    "exp2": _elementwise(np.exp2), "log2": _elementwise(np.log2), "log10": _elementwise(np.log10),
    "sign": _elementwise(np.sign), "round": _elementwise(np.round), "trunc": _elementwise(np.trunc),
    "hypot": _elementwise(np.hypot), "inversesqrt": _elementwise(lambda x: 1.0 / np.sqrt(x)),
    "step": _elementwise(lambda edge, x: (x >= edge).astype(np.float64)),
    "smoothstep": _elementwise(lambda e0, e1, x: np.where(
        x <= e0, 0.0, np.where(x >= e1, 1.0, ((x - e0) / np.where(e1 > e0, e1 - e0, 1.0)) ** 2
                               * (3.0 - 2.0 * (x - e0) / np.where(e1 > e0, e1 - e0, 1.0))))),
    "linearstep": _elementwise(lambda e0, e1, x: np.clip((x - e0) / np.where(e1 > e0, e1 - e0, 1.0), 0.0, 1.0)),
    "dot": _elementwise(lambda a, b: np.dot(a, b)),
    "cross": _elementwise(np.cross),
    "length": _elementwise(np.linalg.norm),
    "distance": _elementwise(lambda a, b: np.linalg.norm(a - b)),
    "normalize": _elementwise(lambda a: a / np.linalg.norm(a) if np.linalg.norm(a) > 0 else a),
}
CLOSURES = {
    "diffuse", "phong", "oren_nayar", "ward", "reflection", "refraction", "transparent", "translucent",
    "microfacet", "emission", "background", "kp_mirror", "kp_dielectric", "kp_microfacet", "kp_emitter",
    "kp_principle_diffuse", "kp_principle_retro", "kp_principle_fakess", "kp_principle_sheen",
    "kp_principle_specular_reflection", "kp_principle_clearcoat", "holdout", "debug",
}


# ---------------------------------------------------------------- parser
class Parser:
    def __init__(self, src: str):
        self.t = tokenize(src)
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, val):
        if self.peek()[1] == val and self.peek()[0] in ("op", "id"):
            self.i += 1
            return True
        return False

    def expect(self, val):
        tok = self.next()
        if tok[1] != val:
            raise ValueError(f"OSL: expected {val!r}, found {tok[1]!r}")
        return tok

    def skip_metadata(self):
        if self.peek()[1] == "[[":
            depth = 0
            while True:
                tok = self.next()
                if tok[0] == "eof":
                    raise ValueError("OSL: unterminated [[ metadata ]]")
                if tok[1] == "[[":
                    depth += 1
                elif tok[1] == "]]":
                    depth -= 1
                    if depth == 0:
                        return

    def type_name(self):
        tok = self.peek()
        if tok[0] == "id" and tok[1] in _TYPES:
            self.i += 1
            if tok[1] == "closure":
                self.expect("color")
            return tok[1]
        return None

    def shader(self, body: bool = True):
        kind = self.next()
        if kind[1] not in ("surface", "shader", "displacement", "volume"):
            raise ValueError(f"OSL: expected a shader declaration, found {kind[1]!r}")
        name = self.next()[1]
        self.skip_metadata()
        self.expect("(")
        params = []
        while not self.accept(")"):
            self.accept("output")
            ty = self.type_name()
            if ty is None:
                raise ValueError(f"OSL: parameter type expected, found {self.peek()[1]!r}")
            pname = self.next()[1]
            if self.accept("["):
                raise ValueError("OSL: array parameters are not lowered")
            self.expect("=")
            params.append((ty, pname, self.expr()))
            self.skip_metadata()
            self.accept(",")
        return name, params, (self.block() if body else None)

    def block(self):
        self.expect("{")
        out = []
        while not self.accept("}"):
            out.append(self.stmt())
        return ("block", out)

    def stmt(self):
        tok = self.peek()
        if tok[1] == "{" and tok[0] == "op":
            return self.block()
        if tok[1] == ";":
            self.next()
            return ("block", [])
        if tok == ("id", "if"):
            self.next()
            self.expect("(")
            c = self.expr()
            self.expect(")")
            a = self.stmt()
            b = self.stmt() if self.accept("else") else None
            return ("if", c, a, b)
        if tok == ("id", "return"):
            self.next()
            self.expect(";")
            return ("return",)
        if tok[0] == "id" and tok[1] in ("for", "while", "do"):
            raise ValueError(f"OSL: `{tok[1]}` loops are not lowered")
        ty = self.type_name()
        if ty is not None:
            decls = []
            while True:
                name = self.next()[1]
                init = self.expr() if self.accept("=") else None
                decls.append((name, init))
                if not self.accept(","):
                    break
            self.expect(";")
            return ("decl", ty, decls)
        if tok[0] == "id" and self.peek(1)[1] in ("=", "+=", "-=", "*=", "/="):
            self.next()
            op = self.next()[1]
            e = self.expr()
            self.expect(";")
            return ("assign", tok[1], op, e)
        e = self.expr()
        self.expect(";")
        return ("expr", e)

    def expr(self):
        c = self.binary(0)
        if self.accept("?"):
            a = self.expr()
            self.expect(":")
            b = self.expr()
            return ("?", c, a, b)
        return c

    _LEVELS = [("||",), ("&&",), ("==", "!="), ("<", ">", "<=", ">="), ("+", "-"), ("*", "/")]

    def binary(self, level):
        if level == len(self._LEVELS):
            return self.unary()
        lhs = self.binary(level + 1)
        while self.peek()[0] == "op" and self.peek()[1] in self._LEVELS[level]:
            op = self.next()[1]
            lhs = (op, lhs, self.binary(level + 1))
        return lhs

    def unary(self):
        if self.peek()[0] == "op" and self.peek()[1] in ("-", "+", "!"):
            op = self.next()[1]
            return ("u" + op, self.unary())
        # cast: (type) expr
        if self.peek()[1] == "(" and self.peek(1)[0] == "id" and self.peek(1)[1] in _TYPES \
                and self.peek(2)[1] == ")":
            self.next()
            ty = self.next()[1]
            self.next()
            return ("cast", ty, self.unary())
        return self.primary()

    def primary(self):
        kind, val = self.next()
        if kind == "num":
            return ("num", float(val))
        if kind == "str":
            return ("str", val[1:-1])
        if kind == "id":
            if self.accept("("):
                args = []
                while not self.accept(")"):
                    args.append(self.expr())
                    self.accept(",")
                return self.postfix(("call", val, args))
            return self.postfix(("var", val))
        if val == "(":
            e = self.expr()
            self.expect(")")
            return self.postfix(e)
        raise ValueError(f"OSL: unexpected token {val!r}")

    def postfix(self, e):
        """Component access: c[i], or v.x / v.y / v.z (p.r / p.g / p.b)."""
        while True:
            if self.peek()[1] == "[" and self.peek()[0] == "op":
                self.next()
                i = self.expr()
                self.expect("]")
                e = ("index", e, i)
            elif self.peek()[1] == "." and self.peek(1)[0] == "id" and self.peek(1)[1] in _COMPONENTS:
                self.next()
                e = ("index", e, ("num", float(_COMPONENTS[self.next()[1]])))
            else:
                return e


# ---------------------------------------------------------------- evaluation
class _Return(Exception):
    pass


@dataclass
class Lowered:
    lobes: list                 # kz_lobe records; params[11] = index into `textures` + 1
    Le: np.ndarray
    warnings: list
    textures: list = field(default_factory=list)   # TexRef specs the lobes reference
    background: np.ndarray = field(default_factory=lambda: np.zeros(3))  # background() weight
    background_texture: tuple = None                # its environment TexRef spec, or None
    outputs: dict = field(default_factory=dict)     # output parameters after the body ran


class Evaluator:
    def __init__(self, params):
        self.scopes = [dict(params)]
        self.types = [{}]
        self.warnings = []

    def lookup(self, name):
        for s in reversed(self.scopes):
            if name in s:
                return s[name]
        if name == "N" or name == "Ng":
            return Normal()
        if name in ("u", "v", "I"):
            return Global(name)
        raise ValueError(f"OSL: `{name}` is not a parameter or local (position-dependent globals are not lowered)")

    def declared_type(self, name):
        for t in reversed(self.types):
            if name in t:
                return t[name]
        return None

    def set(self, name, value):
        for s, t in zip(reversed(self.scopes), reversed(self.types)):
            if name in s:
                ty = t.get(name)
                s[name] = convert(ty, value) if ty else value
                return
        if name == "Ci":
            self.scopes[0]["Ci"] = convert("closure", value)
            return
        if name in ("N", "Ng"):
            self.warnings.append(f"assignment to {name} is ignored: lobes shade with the geometric normal")
            return
        raise ValueError(f"OSL: assignment to undeclared `{name}`")

    def run(self, node):
        kind = node[0]
        if kind == "block":
            self.scopes.append({})
            self.types.append({})
            try:
                for st in node[1]:
                    self.run(st)
            finally:
                self.scopes.pop()
                self.types.pop()
        elif kind == "if":
            if truth(self.eval(node[1])):
                self.run(node[2])
            elif node[3] is not None:
                self.run(node[3])
        elif kind == "decl":
            for name, init in node[2]:
                self.types[-1][name] = node[1]
                if init is None:
                    v = Closure() if node[1] == "closure" else ("" if node[1] == "string" else
                                                              np.zeros(3) if node[1] in _VEC_TYPES else 0.0)
                else:
                    v = convert(node[1], self.eval(init))
                self.scopes[-1][name] = v
        elif kind == "assign":
            _, name, op, e = node
            v = self.eval(e)
            if op != "=":
                v = binop(op[0], self.lookup(name) if name != "Ci" else self.scopes[0]["Ci"], v)
            self.set(name, v)
        elif kind == "expr":
            self.eval(node[1])
        elif kind == "return":
            raise _Return()

    def eval(self, e):
        kind = e[0]
        if kind == "num":
            return e[1]
        if kind == "str":
            return e[1]
        if kind == "var":
            if e[1] == "Ci":
                return self.scopes[0]["Ci"]
            return self.lookup(e[1])
        if kind == "?":
            return self.eval(e[2]) if truth(self.eval(e[1])) else self.eval(e[3])
        if kind == "u-":
            return binop("*", -1.0, self.eval(e[1]))
        if kind == "u+":
            return self.eval(e[1])
        if kind == "u!":
            return float(not truth(self.eval(e[1])))
        if kind == "cast":
            v = self.eval(e[2])
            return v if isinstance(v, Normal) else convert(e[1], v)
        if kind == "index":
            v, i = self.eval(e[1]), self.eval(e[2])
            if not isinstance(v, np.ndarray) or not _is_num(i) or isinstance(i, np.ndarray) or not 0 <= int(i) < 3:
                raise ValueError("OSL: component access needs a triple and an index 0-2")
            return float(v[int(i)])
        if kind == "&&":
            return float(truth(self.eval(e[1])) and truth(self.eval(e[2])))
        if kind == "||":
            return float(truth(self.eval(e[1])) or truth(self.eval(e[2])))
        if kind == "call":
            name, args = e[1], [self.eval(a) for a in e[2]]
            if name in CLOSURES:
                return Closure([(np.ones(3), name, args, None)])
            if name in FUNCS:
                return FUNCS[name](*args)
            raise ValueError(f"OSL: function `{name}` is not lowered")
        return binop(kind, self.eval(e[1]), self.eval(e[2]))


def _f(v, what):
    if not _is_num(v) or isinstance(v, np.ndarray):
        raise ValueError(f"OSL: {what} must be a float")
    return float(v)


# argument counts of the registered closures (bsdfs.h register_closure tables)
_ARITY = {
    "diffuse": (1,), "phong": (2,), "ward": (4,), "reflection": (1, 2), "refraction": (2,), "transparent": (0,),
    "translucent": (0, 1), "microfacet": (5, 7), "kp_mirror": (0,), "kp_dielectric": (0, 2), "kp_microfacet": (4,),
    "kp_principle_diffuse": (1,), "kp_principle_retro": (2,), "kp_principle_fakess": (1,),
    "kp_principle_sheen": (1,), "kp_principle_specular_reflection": (6,), "kp_principle_clearcoat": (2,),
}


def _lobe(name, args, w, warnings):
    """One closure call -> a kz_lobe record."""
    if name in _ARITY and len(args) not in _ARITY[name]:
        raise ValueError(f"OSL: {name} takes {' or '.join(map(str, _ARITY[name]))} arguments, got {len(args)}")
    wt = tuple(float(x) for x in w)
    if name == "diffuse":
        return api.diffuse(wt)
    if name == "ward":
        return api.ward(_f(args[2], "ward xalpha"), _f(args[3], "ward yalpha"), wt)
    if name == "reflection":
        return api.reflection(_f(args[1], "eta") if len(args) > 1 else 0.0, wt)
    if name == "refraction":
        return api.refraction(_f(args[1], "eta"), wt)
    if name == "microfacet":
        if len(args) == 7:  # (dist, N, U, xalpha, yalpha, eta, refract): the registered form
            dist, _, _, xa, ya, eta, refract = args
        elif len(args) == 5:  # (dist, N, alpha, eta, refract): stdosl.h's short form
            dist, _, xa, eta, refract = args
            ya = xa
        else:
            raise ValueError("OSL: microfacet takes 5 or 7 arguments")
        return api.microfacet(dist, _f(xa, "xalpha"), _f(ya, "yalpha"), _f(eta, "eta"), int(_f(refract, "refract")),
                              weight=wt)
    if name == "kp_mirror":
        return api.mirror(wt)
    if name == "kp_dielectric":
        return api.dielectric(*(_f(a, "ior") for a in args[:2]), weight=wt) if args else api.dielectric(weight=wt)
    if name == "kp_microfacet":
        a = [_f(x, "kp_microfacet argument") for x in args]
        return api.kp_microfacet(*a[:4], weight=wt)
    if name == "kp_principle_diffuse":
        return api.principle_diffuse(wt)
    if name == "kp_principle_retro":
        return api.principle_retro(_f(args[1], "roughness"), wt)
    if name == "kp_principle_fakess":
        return api.principle_fakess(_f(args[0], "roughness"), wt)
    if name == "kp_principle_sheen":
        return api.principle_sheen(1.0, wt)
    if name == "kp_principle_specular_reflection":
        F0 = convert("color", args[0])
        return api.principle_specular(tuple(F0), _f(args[2], "xalpha"), _f(args[4], "eta"), _f(args[5], "metallic"),
                                      weight=wt, yalpha=_f(args[3], "yalpha"))
    if name == "kp_principle_clearcoat":
        r = _f(args[1], "roughness")
        if not 0.0 < r < 1.0:
            rc = min(max(r, 1e-4), 0.9999)
            warnings.append(f"kp_principle_clearcoat roughness {r} clamped to {rc} (GTR1 needs (0, 1))")
            r = rc
        return api.principle_clearcoat(r, wt)
    if name in ("phong", "transparent", "translucent"):
        warnings.append(f"`{name}` is not registered with the reference's shading system "
                        "(bsdf.cpp:142-180); lowered to its closure all the same")
        if name == "phong":
            return api.phong(_f(args[1], "exponent"), wt)
        return api.transparent(wt) if name == "transparent" else api.translucent(wt)
    raise ValueError(f"OSL: closure `{name}` is not lowered")


def _param_env(params, overrides, ev):
    for ty, pname, default in params:
        ev.types[0][pname] = ty
        if overrides and pname in overrides:
            v = overrides[pname]
            if not isinstance(v, (str, TexRef, Global)):
                v = np.asarray(v, np.float64) if np.ndim(v) else float(v)
            ev.scopes[0][pname] = convert(ty, v)
        else:
            ev.scopes[0][pname] = convert(ty, ev.eval(default))


def shader_params(src: str, overrides: dict | None = None):
    """(shader name, {parameter: value}) at the defaults, with overrides."""
    name, params, _ = Parser(src).shader(body=False)
    ev = Evaluator({})
    _param_env(params, overrides, ev)
    return name, dict(ev.scopes[0])


def lower(src: str, overrides: dict | None = None) -> Lowered:
    """Evaluate a surface shader over constant inputs -> lobes, Le, the
    textures the lobes use, the background() weight and the output parameters."""
    name, params, body = Parser(src).shader()
    ev = Evaluator({})
    _param_env(params, overrides, ev)
    ev.scopes[0]["Ci"] = Closure()
    ev.types[0]["Ci"] = "closure"
    try:
        ev.run(body)
    except _Return:
        pass
    ci = ev.scopes[0]["Ci"]
    lobes, Le, warnings, textures = [], np.zeros(3), list(ev.warnings), []
    bg, bg_tex = np.zeros(3), None
    for w, cname, args, tex in ci.terms:
        w = np.asarray(w, np.float64)
        if cname == "background":
            if tex is not None:
                if bg_tex is not None and bg_tex != tex:
                    raise ValueError("OSL: a background weighted by two environment maps is not lowered")
                bg_tex = tex
            bg = bg + w
            continue
        if tex is not None and tex[0] == "environment":
            raise ValueError("OSL: environment() weights only background()")
        if cname in ("emission", "kp_emitter"):  # process_closure adds the weight to Le
            if tex is not None:
                raise ValueError("OSL: textured emission is not lowered")
            Le = Le + w
            continue
        if cname in ("holdout", "debug"):
            continue
        if np.all(w == 0):
            continue
        lb = _lobe(cname, args, w, warnings)
        if tex is not None:
            if tex not in textures:
                textures.append(tex)
            if len(textures) > 1:
                raise ValueError("OSL: lobes of one shader reference two textures (one per material is lowered)")
            lb = api.textured(lb, textures.index(tex))
        lobes.append(lb)
    if len(lobes) > N.KZ_MAX_LOBES:
        raise ValueError(f"shader yields {len(lobes)} lobes; the reference keeps at most {N.KZ_MAX_LOBES}")
    outputs = {k: ev.scopes[0][k] for _, k, _ in params}
    return Lowered(lobes, Le, warnings, textures, bg, bg_tex, outputs)


def checkerboard_output(params: dict) -> TexRef:
    """The OSL checkerboard shader (Cout = Ca or Cb by the parity of
    int(fmod(s * scale_s, 2)) ^ int(fmod(t * scale_t, 2)); the version shipped
    with OSL and with the reference's textured scenes) at s = u, t = v, as a
    texture. Its body uses integer operations the evaluator does not lower, so
    it is recognised by name and parameters."""
    s, t = params.get("s"), params.get("t")
    if not (isinstance(s, Global) and s.name == "u" and isinstance(t, Global) and t.name == "v"):
        raise ValueError("checkerboard is lowered at s = u, t = v only")
    ca, cb = convert("color", params["Ca"]), convert("color", params["Cb"])
    if isinstance(ca, TexRef) or isinstance(cb, TexRef):
        raise ValueError("checkerboard colours must be constant")
    return TexRef(("checker", float(params["scale_s"]), float(params["scale_t"]), tuple(float(x) for x in ca),
                   tuple(float(x) for x in cb)))
