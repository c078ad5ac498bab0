"""Arithmetic of MOOSE's distribution and Function expressions, evaluated
as the reference evaluates them.

MOOSE hands these strings to exprtk through ``moose::MooseParser``
(``builtins/MooseParser.cpp``: ``&&``/``||``/``!`` are rewritten to
``and``/``or``/``not`` before parsing; ``ln``, ``fmod`` and, in the
``Neuron``'s ``nuParser``, the Heaviside ``H`` are added).  exprtk is a
third-party library vendored under the reference's ``external/exprtk`` (the
copy there is the pinned version).  Two of its published behaviours decide
the last bit of a result, and are followed here:

* numbers are read digit by digit, not correctly rounded: integer digits
  as ``d = 10 d + digit``, fraction digits into a second such integer added
  as ``frac / 10^k``, and a decimal exponent applied last as ``d * 10^e`` or
  ``d / 10^-e`` with the exact power of ten (``string_to_real``,
  ``compute_pow10``);
* ``x ^ c`` with ``c`` an integer constant, ``|c| <= 60``, is a fixed
  product chain (``fast_exp``: squares for 2, 4, 6, 8, 10, the
  square-and-multiply loop otherwise), its reciprocal for ``c < 0`` and 1
  for ``c = 0``; any other power is ``pow``.

The grammar covered: numbers, variables, ``+ - * / %``, ``^`` (one power
per operand: ``a^b^c`` is refused), unary ``-``/``+`` (applied after a
power: ``-x^2`` is ``-(x^2)``), comparisons ``< <= > >= == = !=
<>`` (1 or 0), ``and``/``or``/``not``, ``c ? a : b``, parentheses and the
functions ``exp log ln log10 sqrt abs sin cos tan asin acos atan sinh cosh
tanh floor ceil min max pow fmod H``.  Constant sub-expressions are
computed in the same operation order as at run time; exprtk's algebraic
rewrites of chained constants (e.g. ``c0 + (x + c1)``) are not applied, so
such expressions may differ in the last bit.  Anything else raises
ValueError.
"""
import math
import re

_TOKEN = re.compile(r"\s*(?:(?P<num>(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)|(?P<name>[A-Za-z_][A-Za-z_0-9]*)"
                    r"|(?P<op><=|>=|==|!=|<>|&&|\|\||[-+*/%^()<>=!?:,]))")


def exprtk_number(text):
    """A numeric literal as exprtk's string_to_real computes it."""
    m = re.fullmatch(r"(\d*)(?:\.(\d*))?(?:[eE]([+-]?\d+))?", text)
    if not m or not (m.group(1) or m.group(2)):
        raise ValueError("bad number %r" % text)
    d = 0.0
    for ch in (m.group(1) or "").lstrip("0"):
        d = d * 10.0 + float(ord(ch) - 48)
    frac = m.group(2) or ""
    if frac:
        t = 0.0
        for ch in frac:
            t = t * 10.0 + float(ord(ch) - 48)
        d += t / float(10 ** len(frac))
    e = int(m.group(3)) if m.group(3) else 0
    if e > 0:
        d = d * float(10 ** e)
    elif e < 0:
        d = d / float(10 ** -e)
    return d


def _fast_exp(v, n):
    """exprtk's details::numeric::fast_exp<T, n>."""
    if n == 0:
        return 1.0
    if n == 1:
        return v
    if n == 2:
        return v * v
    if n == 3:
        return v * v * v
    if n == 4:
        v2 = v * v
        return v2 * v2
    if n == 5:
        return _fast_exp(v, 4) * v
    if n == 6:
        v3 = _fast_exp(v, 3)
        return v3 * v3
    if n == 7:
        return _fast_exp(v, 6) * v
    if n == 8:
        v4 = _fast_exp(v, 4)
        return v4 * v4
    if n == 9:
        return _fast_exp(v, 8) * v
    if n == 10:
        v5 = _fast_exp(v, 5)
        return v5 * v5
    k, r = n, 1.0
    while k:
        if k % 2 == 1:
            r *= v
            k -= 1
        v *= v
        k //= 2
    return r


def _pow(a, b):
    try:
        return math.pow(a, b)
    except (OverflowError, ValueError):
        return float("nan") if a < 0 else float("inf")


_FUNCS = {
    "exp": (1, math.exp), "log": (1, math.log), "ln": (1, math.log), "log10": (1, math.log10),
    "sqrt": (1, math.sqrt), "abs": (1, abs), "sin": (1, math.sin), "cos": (1, math.cos),
    "tan": (1, math.tan), "asin": (1, math.asin), "acos": (1, math.acos), "atan": (1, math.atan),
    "sinh": (1, math.sinh), "cosh": (1, math.cosh), "tanh": (1, math.tanh),
    "floor": (1, math.floor), "ceil": (1, math.ceil),
    "min": (2, min), "max": (2, max), "pow": (2, _pow), "fmod": (2, math.fmod),
    "H": (1, lambda a: 1.0 if a > 0.0 else 0.0),
}


def _tokens(expr):
    expr = expr.replace("&&", " and ").replace("||", " or ")
    out, pos = [], 0
    while pos < len(expr):
        if expr[pos:].strip() == "":
            break
        m = _TOKEN.match(expr, pos)
        if not m:
            raise ValueError("cannot read %r at %r" % (expr, expr[pos:]))
        pos = m.end()
        if m.group("num") is not None:
            out.append(("num", exprtk_number(m.group("num"))))
        elif m.group("name") is not None:
            out.append(("name", m.group("name")))
        else:
            out.append(("op", m.group("op")))
    out.append(("end", None))
    return out


class Expression:
    """A parsed expression: ``Expression("1200 * (p < 1e-4)")(p=5e-5)``."""

    def __init__(self, text):
        self.text = text
        self._t = _tokens(text)
        self._i = 0
        self._fn = self._ternary()
        if self._t[self._i][0] != "end":
            raise ValueError("unexpected %r in %r" % (self._t[self._i][1], text))

    def __call__(self, **var):
        return float(self._fn(var))

    # -- recursive descent, lowest precedence first
    def _peek(self):
        return self._t[self._i]

    def _take(self, kind=None, value=None):
        tok = self._t[self._i]
        if (kind and tok[0] != kind) or (value is not None and tok[1] != value):
            raise ValueError("expected %s in %r" % (value or kind, self.text))
        self._i += 1
        return tok

    def _ternary(self):
        cond = self._or()
        if self._peek() == ("op", "?"):
            self._take()
            a = self._ternary()
            self._take("op", ":")
            b = self._ternary()
            return lambda v: a(v) if cond(v) != 0.0 else b(v)
        return cond

    def _or(self):
        left = self._and()
        while self._peek() == ("name", "or"):
            self._take()
            right = self._and()
            left = (lambda l, r: lambda v: 1.0 if (l(v) != 0.0 or r(v) != 0.0) else 0.0)(left, right)
        return left

    def _and(self):
        left = self._cmp()
        while self._peek() == ("name", "and"):
            self._take()
            right = self._cmp()
            left = (lambda l, r: lambda v: 1.0 if (l(v) != 0.0 and r(v) != 0.0) else 0.0)(left, right)
        return left

    _CMP = {"<": lambda a, b: a < b, "<=": lambda a, b: a <= b, ">": lambda a, b: a > b,
            ">=": lambda a, b: a >= b, "==": lambda a, b: a == b, "=": lambda a, b: a == b,
            "!=": lambda a, b: a != b, "<>": lambda a, b: a != b}

    def _cmp(self):
        left = self._add()
        while self._peek()[0] == "op" and self._peek()[1] in self._CMP:
            f = self._CMP[self._take()[1]]
            right = self._add()
            left = (lambda l, r, f: lambda v: 1.0 if f(l(v), r(v)) else 0.0)(left, right, f)
        return left

    def _add(self):
        left = self._mul()
        while self._peek() in (("op", "+"), ("op", "-")):
            op = self._take()[1]
            right = self._mul()
            left = ((lambda l, r: lambda v: l(v) + r(v)) if op == "+" else
                    (lambda l, r: lambda v: l(v) - r(v)))(left, right)
        return left

    def _mul(self):
        left = self._unary()
        while self._peek() in (("op", "*"), ("op", "/"), ("op", "%")):
            op = self._take()[1]
            right = self._unary()
            if op == "*":
                left = (lambda l, r: lambda v: l(v) * r(v))(left, right)
            elif op == "/":
                left = (lambda l, r: lambda v: _div(l(v), r(v)))(left, right)
            else:
                left = (lambda l, r: lambda v: math.fmod(l(v), r(v)))(left, right)
        return left

    def _unary(self):
        tok = self._peek()
        if tok == ("op", "-"):
            self._take()
            x = self._unary()
            return lambda v: -x(v)
        if tok == ("op", "+"):
            self._take()
            return self._unary()
        if tok == ("name", "not") or tok == ("op", "!"):
            self._take()
            x = self._unary()
            return lambda v: 1.0 if x(v) == 0.0 else 0.0
        return self._power()

    def _power(self):
        f = self._power1()
        self._check_no_chain()
        return f

    def _power1(self):
        base = self._primary()
        if self._peek() == ("op", "^"):
            self._take()
            neg = False
            if self._peek() in (("op", "-"), ("op", "+")):
                neg = self._take()[1] == "-"
            if self._peek()[0] == "num":
                c = self._take()[1]
                c = -c if neg else c
                if abs(c) <= 60 and c == int(c):
                    n = int(abs(c))
                    if c >= 0:
                        return lambda v: _fast_exp(base(v), n)
                    return lambda v: _div(1.0, _fast_exp(base(v), n))
                return lambda v: _pow(base(v), c)
            ex = self._primary()
            if neg:
                return lambda v: _pow(base(v), -ex(v))
            return lambda v: _pow(base(v), ex(v))
        return base

    def _check_no_chain(self):
        if self._peek() == ("op", "^"):
            raise ValueError("chained powers a^b^c are not accepted: %r" % self.text)

    def _primary(self):
        kind, val = self._take()
        if kind == "num":
            return lambda v, c=val: c
        if kind == "op" and val == "(":
            x = self._ternary()
            self._take("op", ")")
            return x
        if kind == "name":
            if self._peek() == ("op", "("):
                if val not in _FUNCS:
                    raise ValueError("unknown function %s in %r" % (val, self.text))
                nargs, f = _FUNCS[val]
                self._take()
                args = [self._ternary()]
                while self._peek() == ("op", ","):
                    self._take()
                    args.append(self._ternary())
                self._take("op", ")")
                if len(args) != nargs:
                    raise ValueError("%s takes %d arguments" % (val, nargs))
                if nargs == 1:
                    a = args[0]
                    return lambda v: float(f(a(v)))
                a, b = args
                return lambda v: float(f(a(v), b(v)))
            name = val
            return lambda v: _var(v, name)
        raise ValueError("unexpected %r in %r" % (val, self.text))


def _var(v, name):
    if name not in v:
        raise ValueError("unknown variable %s" % name)
    return float(v[name])


def _div(a, b):
    if b == 0.0:
        if a == 0.0 or a != a:
            return float("nan")
        return math.copysign(float("inf"), a) * math.copysign(1.0, b)
    return a / b
