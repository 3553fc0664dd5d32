"""Registered external forces.

wendy accepts any Python callable F(x, t) as ``ext_force`` and calls it
through numba or a ctypes callback once per force evaluation
(wendy/wendy.py:389-418).  A GPU kernel cannot call back into Python, so
wendy_gb300 evaluates forces inside the fused force kernels instead: two
closed forms with fast paths (Harmonic, PulseTanh) and compiled expressions
(Expression), which play the part of wendy's numba compilation.  An
Expression is built from a Python function or lambda of (x, t) -- or from
a string -- whose body is one arithmetic expression; it is compiled into a
short register program that the kernels interpret.  Names other than x and
t are read once, when the force is compiled (as numba freezes globals), and
must be numbers.  Instances are ordinary callables too (the original
function, in numpy), so the same object can be handed to the reference's
``wendy.nbody`` for comparison.  ``resolve`` compiles a plain callable on
the fly; anything outside the supported subset raises ValueError.
"""
import ast
import builtins
import inspect
import math
import textwrap

import numpy

from ._lib import EXT_EXPR, EXT_HARMONIC, EXT_PULSE_TANH


class RegisteredForce:
    kind = None
    params = ()

    def __call__(self, x, t):  # pragma: no cover - overridden
        raise NotImplementedError


class Harmonic(RegisteredForce):
    """F(x, t) = -omega^2 x, the form of wendy's own external-force tests
    (tests/test_approx_external.py:12)."""

    kind = EXT_HARMONIC

    def __init__(self, omega):
        self.omega2 = float(omega) ** 2.
        self.params = (self.omega2,)

    def __call__(self, x, t):
        return -self.omega2 * x


class PulseTanh(RegisteredForce):
    """F(x, t) = A exp(-(t - t0)^2 / (2 tau^2)) tanh(x / h): a transient
    antisymmetric kick that peaks at t0."""

    kind = EXT_PULSE_TANH

    def __init__(self, A, t0, tau, h):
        if tau == 0 or h == 0:
            raise ValueError("tau and h must be non-zero")
        self.A, self.t0, self.tau, self.h = float(A), float(t0), float(tau), float(h)
        self.params = (self.A, self.t0, self.tau, self.h)

    def __call__(self, x, t):
        return self.A * numpy.exp(-(t - self.t0) ** 2 / (2 * self.tau ** 2)) * numpy.tanh(x / self.h)


# ---- compiled expressions -------------------------------------------------
# op codes and limits of the C ABI (include/wendy_gb300.h, WG_EXT_EXPR)
(OP_X, OP_T, OP_K, OP_MOV, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_POW, OP_EXP, OP_LOG,
 OP_SQRT, OP_SIN, OP_COS, OP_TAN, OP_TANH, OP_SINH, OP_COSH, OP_ATAN, OP_ABS) = range(21)
EXPR_MAX_OPS = 64
EXPR_REGS = 16

_FUNCS = {"exp": OP_EXP, "log": OP_LOG, "sqrt": OP_SQRT, "sin": OP_SIN, "cos": OP_COS,
          "tan": OP_TAN, "tanh": OP_TANH, "sinh": OP_SINH, "cosh": OP_COSH, "arctan": OP_ATAN,
          "atan": OP_ATAN, "abs": OP_ABS, "fabs": OP_ABS, "absolute": OP_ABS}
_BINOPS = {ast.Add: OP_ADD, ast.Sub: OP_SUB, ast.Mult: OP_MUL, ast.Div: OP_DIV, ast.Pow: OP_POW}
_UNARY = {OP_NEG: numpy.negative, OP_EXP: numpy.exp, OP_LOG: numpy.log, OP_SQRT: numpy.sqrt,
          OP_SIN: numpy.sin, OP_COS: numpy.cos, OP_TAN: numpy.tan, OP_TANH: numpy.tanh,
          OP_SINH: numpy.sinh, OP_COSH: numpy.cosh, OP_ATAN: numpy.arctan,
          OP_ABS: numpy.abs, OP_MOV: lambda a: a}
_BINARY = {OP_ADD: numpy.add, OP_SUB: numpy.subtract, OP_MUL: numpy.multiply,
           OP_DIV: numpy.divide, OP_POW: numpy.power}


def _number(v, what):
    if isinstance(v, (bool, numpy.bool_)) or not isinstance(v, (int, float, numpy.integer,
                                                                 numpy.floating)):
        raise ValueError("%s is not a number (only x, t and numeric constants may appear in an "
                         "expression force)" % what)
    v = float(v)
    if not math.isfinite(v):
        raise ValueError("%s is not finite" % what)
    return ("k", v)


class _Parser:
    """AST of one expression -> tree of ("x",), ("t",), ("k", value),
    ("un", code, node), ("bin", code, node, node), with constants folded."""

    def __init__(self, xname, tname, env, obj=None, selfname=None):
        self.xname, self.tname, self.env = xname, tname, env
        self.obj, self.selfname = obj, selfname

    def lookup(self, name):
        if name in self.env:
            return self.env[name]
        raise ValueError("name %r is not defined" % name)

    def func_code(self, node):
        """The op code of a called function: numpy.X / np.X / math.X or a
        bare name bound to one of them (or the builtin abs)."""
        if isinstance(node, ast.Name):
            f = self.lookup(node.id)
            name = getattr(f, "__name__", None)
            if f is abs:
                return OP_ABS
            if name in _FUNCS and (f is getattr(numpy, name, None) or f is getattr(math, name, None)):
                return _FUNCS[name]
        elif isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name):
            mod = self.lookup(node.value.id)
            if mod in (numpy, math) and node.attr in _FUNCS:
                return _FUNCS[node.attr]
        raise ValueError("unsupported function in expression force: %s" % ast.unparse(node))

    def __call__(self, node):
        if isinstance(node, ast.Constant):
            return _number(node.value, "constant %r" % (node.value,))
        if isinstance(node, ast.Name):
            if node.id == self.xname:
                return ("x",)
            if node.id == self.tname:
                return ("t",)
            return _number(self.lookup(node.id), "name %r" % node.id)
        if isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name):
            if self.selfname is not None and node.value.id == self.selfname:
                return _number(getattr(self.obj, node.attr), "attribute %r" % node.attr)
            base = self.lookup(node.value.id)
            if base in (numpy, math) and node.attr in ("pi", "e"):
                return ("k", float(getattr(base, node.attr)))
        if isinstance(node, ast.UnaryOp):
            c = self(node.operand)
            if isinstance(node.op, ast.UAdd):
                return c
            if isinstance(node.op, ast.USub):
                return _fold(("un", OP_NEG, c))
        if isinstance(node, ast.BinOp) and type(node.op) in _BINOPS:
            code = _BINOPS[type(node.op)]
            a, b = self(node.left), self(node.right)
            if code == OP_POW and b[0] == "k":
                # numpy's float power takes these exponents on fast paths
                if b[1] == 2.0:
                    return _fold(("bin", OP_MUL, a, a))
                if b[1] == 1.0:
                    return a
                if b[1] == 0.5:
                    return _fold(("un", OP_SQRT, a))
                if b[1] == -1.0:
                    return _fold(("bin", OP_DIV, ("k", 1.0), a))
            return _fold(("bin", code, a, b))
        if isinstance(node, ast.Call) and len(node.args) == 1 and not node.keywords:
            return _fold(("un", self.func_code(node.func), self(node.args[0])))
        raise ValueError("unsupported construct in expression force: %s" % ast.unparse(node))


def _fold(node):
    """Constant subtrees become one constant (numpy float64 arithmetic)."""
    if node[0] == "un" and node[2][0] == "k":
        with numpy.errstate(all="ignore"):
            return _number(_UNARY[node[1]](numpy.float64(node[2][1])), "a constant subexpression")
    if node[0] == "bin" and node[2][0] == "k" and node[3][0] == "k":
        with numpy.errstate(all="ignore"):
            return _number(_BINARY[node[1]](numpy.float64(node[2][1]), numpy.float64(node[3][1])),
                           "a constant subexpression")
    return node


def _has_x(node):
    if node[0] == "x":
        return True
    if node[0] in ("un", "bin"):
        return any(_has_x(c) for c in node[2:])
    return False


class _Codegen:
    """Tree -> register program: the subtrees free of x first (time phase,
    their registers kept), then the rest (space phase, per sheet)."""

    def __init__(self):
        self.ops = []
        self.free = list(range(EXPR_REGS))
        self.kept = {}  # id of a hoisted subtree -> its register

    def alloc(self):
        if not self.free:
            raise ValueError("expression force needs more than %d registers" % EXPR_REGS)
        return self.free.pop(0)

    def emit(self, code, dst, a=0, b=0, k=0.0):
        if len(self.ops) >= EXPR_MAX_OPS:
            raise ValueError("expression force needs more than %d operations" % EXPR_MAX_OPS)
        self.ops.append((code, dst, a, b, float(k)))

    def owned(self, r):
        return r not in self.kept.values()

    def gen(self, node):
        if id(node) in self.kept:
            return self.kept[id(node)]
        kind = node[0]
        if kind in ("x", "t", "k"):
            r = self.alloc()
            self.emit({"x": OP_X, "t": OP_T, "k": OP_K}[kind], r,
                      k=node[1] if kind == "k" else 0.0)
            return r
        if kind == "un":
            ra = self.gen(node[2])
            dst = ra if self.owned(ra) else self.alloc()
            self.emit(node[1], dst, ra, ra)
            return dst
        ra = self.gen(node[2])
        rb = self.gen(node[3])
        dst = ra if self.owned(ra) else (rb if self.owned(rb) else self.alloc())
        self.emit(node[1], dst, ra, rb)
        for r in (ra, rb):
            if r != dst and self.owned(r):
                self.free.insert(0, r)
        return dst

    def hoist(self, node):
        """Time phase: every maximal subtree without x, kept in a register."""
        if not _has_x(node):
            r = self.gen(node)
            self.kept[id(node)] = r
            return
        for c in node[2:]:
            self.hoist(c)

    def program(self, tree):
        if not _has_x(tree):
            self.gen(tree)
            return self.ops, len(self.ops)
        self.hoist(tree)
        n_time = len(self.ops)
        self.gen(tree)
        return self.ops, n_time


def _source_expression(fn):
    """(expression AST, x name, t name, names, bound object, self name) of a
    function, lambda or callable object whose body is a single expression."""
    obj, selfname = None, None
    target = fn
    if not inspect.isfunction(fn) and callable(fn) and not inspect.isbuiltin(fn):
        obj = fn
        target = type(fn).__call__
    try:
        src = textwrap.dedent(inspect.getsource(target))
    except (OSError, TypeError):
        raise ValueError("the source of %r is not available; pass the expression as a string"
                         % (fn,))
    try:
        mod = ast.parse(src)
    except SyntaxError:
        # a lambda in the middle of a statement: parse from the lambda on
        i = src.find("lambda")
        if i < 0:
            raise ValueError("cannot parse the source of %r" % (fn,))
        mod = None
        for j in range(len(src), i, -1):
            try:
                mod = ast.parse(src[i:j].strip().rstrip(",)"))
                break
            except SyntaxError:
                continue
        if mod is None:
            raise ValueError("cannot parse the source of %r" % (fn,))
    code = target.__code__
    cands = []
    for node in ast.walk(mod):
        if isinstance(node, ast.Lambda) and target.__name__ == "<lambda>":
            cands.append((node.args, node.body))
        elif isinstance(node, ast.FunctionDef) and node.name == target.__name__:
            body = [b for b in node.body
                    if not (isinstance(b, ast.Expr) and isinstance(b.value, ast.Constant))]
            if len(body) != 1 or not isinstance(body[0], ast.Return) or body[0].value is None:
                raise ValueError("expression force %r must consist of one return statement"
                                 % target.__name__)
            cands.append((node.args, body[0].value))
    cands = [c for c in cands if len(c[0].args) == code.co_argcount and not c[0].vararg]
    if len(cands) != 1:
        raise ValueError("cannot single out the expression of %r in its source; pass it as a "
                         "string" % (fn,))
    args, expr = cands[0]
    names = [a.arg for a in args.args]
    if obj is not None:
        selfname, names = names[0], names[1:]
    if len(names) != 2:
        raise ValueError("an expression force takes two arguments (x, t)")
    cv = inspect.getclosurevars(target)
    env = dict(vars(builtins))
    env.update(cv.builtins)
    env.update(target.__globals__)
    env.update(cv.nonlocals)
    return expr, names[0], names[1], env, obj, selfname


class Expression(RegisteredForce):
    """A force F(x, t) compiled for the GPU kernels (WG_EXT_EXPR).

    ``f`` is a function, lambda or callable object of (x, t) whose body is a
    single arithmetic expression -- +, -, *, /, ** and exp, log, sqrt, sin,
    cos, tan, tanh, sinh, cosh, arctan, abs from numpy or math -- or a string
    with such an expression in x and t; ``constants`` name extra numbers a
    string may use.  Other names are read when the force is compiled and must
    be numbers.  Everything else raises ValueError.
    """

    kind = EXT_EXPR

    def __init__(self, f, **constants):
        if isinstance(f, str):
            tree = ast.parse(f.strip(), mode="eval").body
            env = {"numpy": numpy, "np": numpy, "math": math}
            env.update({name: getattr(numpy, name) for name in _FUNCS if hasattr(numpy, name)})
            env.update(constants)
            self._parsed = _Parser("x", "t", env)(tree)
            self.fn = None
            self.source = f
        else:
            expr, xn, tn, env, obj, selfname = _source_expression(f)
            env.update(constants)
            self._parsed = _Parser(xn, tn, env, obj, selfname)(expr)
            self.fn = f
            self.source = ast.unparse(expr)
        ops, n_time = _Codegen().program(self._parsed)
        self.ops, self.n_time = ops, n_time
        self.params = tuple([float(len(ops)), float(n_time)] +
                            [float(v) for op in ops for v in op])

    def run_program(self, x, t):
        """The compiled program run in numpy (what the kernels compute)."""
        x = numpy.asarray(x, dtype=numpy.float64)
        r = [None] * EXPR_REGS
        with numpy.errstate(all="ignore"):
            for code, dst, a, b, k in self.ops:
                if code == OP_X:
                    r[dst] = x
                elif code == OP_T:
                    r[dst] = numpy.float64(t)
                elif code == OP_K:
                    r[dst] = numpy.float64(k)
                elif code in _BINARY:
                    r[dst] = _BINARY[code](r[a], r[b])
                else:
                    r[dst] = _UNARY[code](r[a])
        return numpy.broadcast_to(r[self.ops[-1][1]], x.shape).astype(numpy.float64)

    def __call__(self, x, t):
        if self.fn is not None:
            return self.fn(x, t)
        return self.run_program(x, t)


def evaluate_on_device(ext_force, x, t):
    """F(x, t) of a registered force evaluated on the GPU by the force
    kernels' own code (wg_ext_force_eval): the device counterpart of calling
    the force object itself."""
    from . import _lib
    kind, params = resolve(ext_force)
    x = numpy.ascontiguousarray(x, dtype=numpy.float64)
    out = numpy.empty(len(x))
    _lib.check(_lib.lib().wg_ext_force_eval(len(x), x, float(t), int(kind),
                                            _lib.ext_params(params), len(params), out),
               "wg_ext_force_eval")
    return out


def resolve(ext_force):
    """(kind, params) for the C ABI.  A registered force is passed as is; a
    plain callable or string is compiled into an Expression (ValueError when
    it is outside the supported subset)."""
    if ext_force is None:
        return 0, ()
    if isinstance(ext_force, RegisteredForce):
        return ext_force.kind, tuple(ext_force.params)
    if isinstance(ext_force, str) or callable(ext_force):
        f = Expression(ext_force)
        return f.kind, f.params
    raise ValueError("ext_force must be a registered force (wendy_gb300.extforce.Harmonic, "
                     "PulseTanh, Expression) or a function of (x, t) that compiles into an "
                     "Expression")
