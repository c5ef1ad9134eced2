"""Translate Python callbacks F, B, S into CUDA C++ device code.

Stands in for the numba step of the reference (pypde/cfuncs.py:30-75): the
user writes F(Q, d) / F(Q) / F(Q, DQ, d), B(Q, d) / B(Q) and S(Q) in Python
with numpy, and the kernels need device functions with the callback
signatures of pypde/cfuncs.py:6-8.  The translator reads the function
source (inspect + ast) and emits a `struct UserSystem` for the NVRTC
compilation of the kernel templates.

Supported subset (what the reference's example systems use):
  * scalars and fixed-length arrays of float64; Q (length V), DQ (ndim x V),
    d (int) as in the reference's signatures;
  * assignment, augmented assignment, subscript assignment a[i] = ...,
    a[i, j] = ..., if / elif / else, `for i in range(...)` with bounds known
    at translation time, return;
  * + - * / ** (x**2 -> x*x, x**0.5 -> sqrt), unary -, comparisons, and/or/
    not, `a if c else b`; arrays combine elementwise and broadcast scalars;
  * Q[i], Q[a:b], DQ[d][i], DQ[d, i], DQ[d]; zeros(n), zeros((n, m)),
    array([...]), array([[...], ...]), len(), abs/min/max, sqrt, exp, log,
    sin, cos, tan, tanh, pow, floor, sum, dot (with or without a numpy /
    math prefix);
  * calls to other plain Python functions (translated as device functions)
    and numeric constants from the callback's globals or closure.
Every expression is emitted in Python's evaluation order with no algebraic
rewriting, so a callback that a C restatement writes the same way gives the
same bits (the kernels are compiled without FMA contraction).
"""
import ast
import inspect
import math
import textwrap

MATH1 = {"sqrt": "sqrt", "exp": "exp", "log": "log", "sin": "sin", "cos": "cos",
         "tan": "tan", "tanh": "tanh", "floor": "floor", "fabs": "fabs", "abs": "fabs",
         "absolute": "fabs", "log10": "log10", "cbrt": "cbrt", "arctan": "atan",
         "atan": "atan", "sinh": "sinh", "cosh": "cosh", "expm1": "expm1", "log1p": "log1p"}


class TranslateError(ValueError):
    pass


class T:
    """Type of a translated expression: int, float, or an array shape."""
    INT, FLT, ARR = "int", "float", "arr"

    def __init__(self, kind, shape=()):
        self.kind, self.shape = kind, tuple(shape)

    @property
    def n(self):
        r = 1
        for s in self.shape:
            r *= s
        return r

    def __repr__(self):
        return f"T({self.kind},{self.shape})"


INT, FLT = T(T.INT), T(T.FLT)


def _arr(*shape):
    return T(T.ARR, shape)


class Fn:
    """Translation of one Python function body into C statements."""

    def __init__(self, tr, func, params):
        self.tr = tr
        self.func = func
        self.env = {}        # python name -> (c name, T)
        self.lines = []
        self.tmp = 0
        self.params = params
        self.node = self._function_node(func)
        g = dict(getattr(func, "__globals__", {}))
        if func.__closure__:
            for name, cell in zip(func.__code__.co_freevars, func.__closure__):
                try:
                    g[name] = cell.cell_contents
                except ValueError:
                    pass
        self.globals = g

    @staticmethod
    def _function_node(func):
        """The FunctionDef of func; a lambda becomes a one-statement
        function.  Source that cannot be read or parsed is an error."""
        try:
            src = textwrap.dedent(inspect.getsource(func))
        except (OSError, TypeError) as e:
            raise TranslateError(f"{getattr(func, '__name__', func)}: no source ({e})")
        try:
            mod = ast.parse(src)
        except SyntaxError:
            try:
                mod = ast.parse("(" + src.strip().rstrip(",") + ")")
            except SyntaxError as e:
                raise TranslateError(f"{func.__name__}: cannot parse its source ({e})")
        if func.__name__ != "<lambda>":
            for n in mod.body:
                if isinstance(n, ast.FunctionDef) and n.name == func.__name__:
                    return n
            raise TranslateError(f"{func.__name__}: function definition not found")
        nargs = func.__code__.co_argcount
        lams = [n for n in ast.walk(mod) if isinstance(n, ast.Lambda)
                and len(n.args.args) == nargs]
        if len(lams) != 1:
            raise TranslateError("lambda: cannot tell it apart from the other lambdas on "
                                 "its source line; define it with def")
        lam = lams[0]
        fn = ast.FunctionDef(name="lambda_", args=lam.args,
                             body=[ast.Return(value=lam.body, lineno=lam.lineno,
                                              col_offset=lam.col_offset)],
                             decorator_list=[], returns=None, type_params=[],
                             lineno=lam.lineno, col_offset=lam.col_offset)
        return fn

    # ----------------------------------------------------------- helpers
    def new(self, t, init=None):
        self.tmp += 1
        name = f"t{self.tmp}_"
        if t.kind == T.ARR:
            self.emit(f"double {name}[{t.n}];")
        elif t.kind == T.INT:
            self.emit(f"int {name}{' = ' + init if init else ''};")
        else:
            self.emit(f"double {name}{' = ' + init if init else ''};")
        return name

    def emit(self, s):
        self.lines.append("  " * self.depth + s)

    depth = 1
    base_depth = 1

    def err(self, node, msg):
        raise TranslateError(f"{self.func.__name__}: line {getattr(node, 'lineno', '?')}: {msg}")

    def const(self, node):
        """Value of an expression known at translation time, or None."""
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float, bool)):
            return node.value
        if isinstance(node, ast.Name):
            if node.id in self.env:
                return None
            if node.id in ("V",) and "V" not in self.globals:
                return self.tr.V
            v = self.globals.get(node.id)
            if isinstance(v, (int, float)) and not isinstance(v, bool):
                return v
            return None
        if isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name):
            if node.value.id in ("math", "np", "numpy") and node.attr in ("pi", "e"):
                return getattr(math, node.attr)
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
            v = self.const(node.operand)
            return None if v is None else -v
        if isinstance(node, ast.BinOp):
            a, b = self.const(node.left), self.const(node.right)
            if a is None or b is None:
                return None
            ops = {ast.Add: lambda x, y: x + y, ast.Sub: lambda x, y: x - y,
                   ast.Mult: lambda x, y: x * y, ast.FloorDiv: lambda x, y: x // y,
                   ast.Mod: lambda x, y: x % y}
            if type(node.op) in ops and isinstance(a, int) and isinstance(b, int):
                return ops[type(node.op)](a, b)
            return None
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and node.func.id == "len":
            _, t = self.expr(node.args[0])
            return t.shape[0] if t.kind == T.ARR else None
        return None

    @staticmethod
    def lit(v):
        if isinstance(v, bool):
            return "1" if v else "0"
        if isinstance(v, int):
            return str(v)
        r = repr(float(v))
        if "inf" in r or "nan" in r:
            raise TranslateError("non-finite constant")
        if "." not in r and "e" not in r:
            r += ".0"
        return r

    # ----------------------------------------------------------- expressions
    def expr(self, node):
        """Return (c_expr_or_array_name, T)."""
        c = self.const(node)
        if c is not None:
            return self.lit(c), (INT if isinstance(c, int) else FLT)
        if isinstance(node, ast.Name):
            if node.id in self.env:
                return self.env[node.id]
            g = self.globals.get(node.id)
            vals = None
            try:  # a numeric tuple / list / 1-D array from globals or closure
                if g is not None and not callable(g) and len(g) > 0 and \
                        all(isinstance(float(x), float) for x in g):
                    vals = [float(x) for x in g]
            except (TypeError, ValueError):
                vals = None
            if vals is not None:
                cn = f"g_{node.id}"
                pad = "  " * self.base_depth
                self.lines.insert(0, f"{pad}const double {cn}[{len(vals)}] = "
                                     f"{{{', '.join(self.lit(v) for v in vals)}}};")
                self.env[node.id] = (cn, _arr(len(vals)))
                return self.env[node.id]
            self.err(node, f"unknown name {node.id}")
        if isinstance(node, ast.UnaryOp):
            v, t = self.expr(node.operand)
            if isinstance(node.op, ast.USub):
                if t.kind == T.ARR:
                    out = self.new(t)
                    self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = -{v}[i_];")
                    return out, t
                return f"(-{v})", t
            if isinstance(node.op, ast.UAdd):
                return v, t
            if isinstance(node.op, ast.Not):
                return f"(!({v}))", INT
            self.err(node, "unsupported unary operator")
        if isinstance(node, ast.BinOp):
            return self.binop(node)
        if isinstance(node, ast.BoolOp):
            op = " && " if isinstance(node.op, ast.And) else " || "
            parts = [self.expr(v)[0] for v in node.values]
            return "(" + op.join(f"({p})" for p in parts) + ")", INT
        if isinstance(node, ast.Compare):
            ops = {ast.Lt: "<", ast.LtE: "<=", ast.Gt: ">", ast.GtE: ">=", ast.Eq: "==",
                   ast.NotEq: "!="}
            left, _ = self.expr(node.left)
            parts = []
            for op, right in zip(node.ops, node.comparators):
                r, _ = self.expr(right)
                if type(op) not in ops:
                    self.err(node, "unsupported comparison")
                parts.append(f"({left} {ops[type(op)]} {r})")
                left = r
            return "(" + " && ".join(parts) + ")", INT
        if isinstance(node, ast.IfExp):
            c, _ = self.expr(node.test)
            a, ta = self.expr(node.body)
            b, tb = self.expr(node.orelse)
            if ta.kind == T.ARR or tb.kind == T.ARR:
                self.err(node, "conditional arrays are not supported")
            t = INT if ta.kind == tb.kind == T.INT else FLT
            return f"(({c}) ? ({a}) : ({b}))", t
        if isinstance(node, ast.Subscript):
            return self.subscript(node)
        if isinstance(node, ast.Call):
            return self.call(node)
        if isinstance(node, (ast.List, ast.Tuple)):
            return self.array_literal(node.elts, node)
        self.err(node, f"unsupported expression {type(node).__name__}")

    def index_expr(self, node):
        c = self.const(node)
        if c is not None:
            if not isinstance(c, int):
                self.err(node, "index must be an integer")
            return str(c), c
        v, t = self.expr(node)
        if t.kind != T.INT:
            self.err(node, "index must be an integer expression")
        return v, None

    def subscript(self, node):
        base, bt = self.expr(node.value)
        if bt.kind != T.ARR:
            self.err(node, "subscript of a scalar")
        sl = node.slice
        if isinstance(sl, ast.Tuple):
            idx = sl.elts
        else:
            idx = [sl]
        if len(idx) == 1 and isinstance(idx[0], ast.Slice):
            s = idx[0]
            lo = 0 if s.lower is None else self.const(s.lower)
            hi = bt.shape[0] if s.upper is None else self.const(s.upper)
            if lo is None or hi is None or s.step is not None:
                self.err(node, "slices need constant bounds")
            if lo < 0:
                lo += bt.shape[0]
            if hi < 0:
                hi += bt.shape[0]
            if len(bt.shape) != 1:
                self.err(node, "slices of 2-D arrays are not supported")
            t = _arr(hi - lo)
            out = self.new(t)
            self.emit(f"for (int i_ = 0; i_ < {hi - lo}; i_++) {out}[i_] = {base}[{lo} + i_];")
            return out, t
        if len(idx) == 1 and len(bt.shape) == 2:
            r, _ = self.index_expr(idx[0])
            t = _arr(bt.shape[1])
            return f"({base} + ({r}) * {bt.shape[1]})", t  # row view
        if len(idx) == 1:
            i, _ = self.index_expr(idx[0])
            return f"{base}[{i}]", FLT
        if len(idx) == 2 and len(bt.shape) == 2:
            i, _ = self.index_expr(idx[0])
            j, _ = self.index_expr(idx[1])
            return f"{base}[({i}) * {bt.shape[1]} + ({j})]", FLT
        self.err(node, "unsupported subscript")

    def array_literal(self, elts, node):
        if elts and isinstance(elts[0], (ast.List, ast.Tuple)):
            rows = [self.array_literal(e.elts, e) for e in elts]
            ncol = rows[0][1].n
            t = _arr(len(rows), ncol)
            out = self.new(t)
            for r, (name, rt) in enumerate(rows):
                if rt.n != ncol:
                    self.err(node, "ragged 2-D array literal")
                self.emit(f"for (int i_ = 0; i_ < {ncol}; i_++) {out}[{r * ncol} + i_] = {name}[i_];")
            return out, t
        vals = []
        for e in elts:
            v, t = self.expr(e)
            if t.kind == T.ARR:
                self.err(node, "nested arrays must be rows of a 2-D literal")
            vals.append(f"(double)({v})" if t.kind == T.INT else v)
        t = _arr(len(vals))
        out = self.new(t)
        for i, v in enumerate(vals):
            self.emit(f"{out}[{i}] = {v};")
        return out, t

    def binop(self, node):
        op = node.op
        if isinstance(op, ast.Pow):
            b, tb = self.expr(node.left)
            e = self.const(node.right)
            if tb.kind == T.ARR:
                self.err(node, "array ** is not supported")
            if e == 2:
                tmp = self.new(FLT, b if tb.kind != T.INT else f"(double)({b})")
                return f"({tmp} * {tmp})", FLT
            if e == 0.5:
                return f"sqrt({b})", FLT
            if e == 1:
                return b, tb
            ex, te = self.expr(node.right)
            return f"pow((double)({b}), (double)({ex}))", FLT
        a, ta = self.expr(node.left)
        b, tb = self.expr(node.right)
        sym = {ast.Add: "+", ast.Sub: "-", ast.Mult: "*", ast.Div: "/", ast.FloorDiv: "/",
               ast.Mod: "%"}.get(type(op))
        if sym is None:
            self.err(node, "unsupported operator")
        if ta.kind != T.ARR and tb.kind != T.ARR:
            if isinstance(op, ast.Div):
                return f"((double)({a}) / (double)({b}))" if (ta.kind == T.INT and
                                                              tb.kind == T.INT) \
                    else f"({a} / {b})", FLT
            if isinstance(op, (ast.FloorDiv, ast.Mod)):
                if ta.kind == T.INT and tb.kind == T.INT:
                    return f"({a} {sym} {b})", INT
                self.err(node, "// and % need integers")
            t = INT if ta.kind == tb.kind == T.INT else FLT
            return f"({a} {sym} {b})", t
        # elementwise with broadcasting of scalars
        t = ta if ta.kind == T.ARR else tb
        if ta.kind == T.ARR and tb.kind == T.ARR and ta.n != tb.n:
            self.err(node, "arrays of different lengths")
        out = self.new(t)
        ai = f"{a}[i_]" if ta.kind == T.ARR else a
        bi = f"{b}[i_]" if tb.kind == T.ARR else b
        self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {ai} {sym} {bi};")
        return out, t

    def call(self, node):
        f = node.func
        if isinstance(f, ast.Attribute) and isinstance(f.value, ast.Name) and \
                f.value.id in ("np", "numpy", "math"):
            name = f.attr
        elif isinstance(f, ast.Name):
            name = f.id
        else:
            self.err(node, "unsupported call")
        args = node.args
        if name in ("zeros", "empty", "zeros_like"):
            if name == "zeros_like":
                _, t = self.expr(args[0])
                shape = t.shape
            else:
                a0 = args[0]
                if isinstance(a0, (ast.Tuple, ast.List)):
                    shape = tuple(self.const(e) for e in a0.elts)
                else:
                    shape = (self.const(a0),)
                if any(s is None for s in shape):
                    self.err(node, "zeros() needs a constant shape")
            t = _arr(*shape)
            out = self.new(t)
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = 0.0;")
            return out, t
        if name in ("array", "asarray"):
            a0 = args[0]
            if isinstance(a0, (ast.List, ast.Tuple)):
                return self.array_literal(a0.elts, a0)
            return self.expr(a0)
        if name in MATH1 and len(args) == 1:
            v, t = self.expr(args[0])
            if t.kind == T.ARR:
                out = self.new(t)
                self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {MATH1[name]}({v}[i_]);")
                return out, t
            if name == "abs" and t.kind == T.INT:
                return f"abs({v})", INT
            return f"{MATH1[name]}((double)({v}))", FLT
        if name in ("min", "max", "fmin", "fmax", "minimum", "maximum") and len(args) == 2:
            a, ta = self.expr(args[0])
            b, tb = self.expr(args[1])
            fn = "fmin" if name in ("min", "fmin", "minimum") else "fmax"
            if ta.kind == tb.kind == T.INT:
                return f"(({a}) {'<' if fn == 'fmin' else '>'} ({b}) ? ({a}) : ({b}))", INT
            return f"{fn}((double)({a}), (double)({b}))", FLT
        if name == "ldexp" and len(args) == 2:
            a, _ = self.expr(args[0])
            b, _ = self.expr(args[1])
            return f"ldexp((double)({a}), (int)({b}))", FLT
        if name in ("pow", "power") and len(args) == 2:
            a, _ = self.expr(args[0])
            b, _ = self.expr(args[1])
            return f"pow((double)({a}), (double)({b}))", FLT
        if name in ("sum",) and len(args) == 1:
            v, t = self.expr(args[0])
            acc = self.new(FLT, "0.0")
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {acc} += {v}[i_];")
            return acc, FLT
        if name in ("dot", "inner") and len(args) == 2:
            a, ta = self.expr(args[0])
            b, tb = self.expr(args[1])
            acc = self.new(FLT, "0.0")
            self.emit(f"for (int i_ = 0; i_ < {ta.n}; i_++) {acc} += {a}[i_] * {b}[i_];")
            return acc, FLT
        if name in ("float",):
            v, _ = self.expr(args[0])
            return f"(double)({v})", FLT
        if name in ("int",):
            v, _ = self.expr(args[0])
            return f"(int)({v})", INT
        target = self.globals.get(name)
        if callable(target) and hasattr(target, "__code__"):
            return self.tr.call_helper(self, target, args, node)
        # numba-jitted helpers expose the Python function as .py_func
        if target is not None and hasattr(target, "py_func"):
            return self.tr.call_helper(self, target.py_func, args, node)
        self.err(node, f"unsupported function {name}")

    # ----------------------------------------------------------- statements
    def assign_name(self, name, v, t, node):
        if name in self.env:
            cn, ct = self.env[name]
            if ct.kind == T.ARR:
                if t.kind != T.ARR or t.n != ct.n:
                    self.err(node, f"{name} changes shape")
                self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {cn}[i_] = {v}[i_];")
            else:
                if t.kind == T.ARR:
                    self.err(node, f"{name} changes from scalar to array")
                if ct.kind == T.INT and t.kind == T.FLT:
                    self.err(node, f"{name} changes from int to float")
                self.emit(f"{cn} = {v};")
            return
        # Python names live for the whole function: declare at the top so a
        # name first bound inside an if/for block is visible after it
        cn = f"v_{name}"
        pad = "  " * self.base_depth
        if t.kind == T.ARR:
            self.lines.insert(0, f"{pad}double {cn}[{t.n}];")
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {cn}[i_] = {v}[i_];")
        else:
            self.lines.insert(0, f"{pad}{'int' if t.kind == T.INT else 'double'} {cn};")
            self.emit(f"{cn} = {v};")
        self.env[name] = (cn, t)

    def stmt(self, node):
        if isinstance(node, ast.Expr) and isinstance(node.value, ast.Constant):
            return  # docstring
        if isinstance(node, ast.Assign):
            if len(node.targets) != 1:
                self.err(node, "chained assignment")
            tgt = node.targets[0]
            if isinstance(tgt, ast.Tuple):
                if not isinstance(node.value, ast.Tuple) or len(node.value.elts) != len(tgt.elts):
                    self.err(node, "tuple assignment needs a tuple of the same length")
                vals = [self.expr(e) for e in node.value.elts]
                tmps = []
                for v, t in vals:
                    if t.kind == T.ARR:
                        self.err(node, "tuple assignment of arrays")
                    tmps.append((self.new(t, v), t))
                for tg, (v, t) in zip(tgt.elts, tmps):
                    self.assign_name(tg.id, v, t, node)
                return
            v, t = self.expr(node.value)
            if isinstance(tgt, ast.Name):
                self.assign_name(tgt.id, v, t, node)
                return
            if isinstance(tgt, ast.Subscript):
                lhs, lt = self.subscript_target(tgt)
                if lt.kind == T.ARR:
                    if t.kind == T.ARR:
                        self.emit(f"for (int i_ = 0; i_ < {lt.n}; i_++) {lhs}[i_] = {v}[i_];")
                    else:
                        self.emit(f"for (int i_ = 0; i_ < {lt.n}; i_++) {lhs}[i_] = {v};")
                else:
                    self.emit(f"{lhs} = {v};")
                return
            self.err(node, "unsupported assignment target")
        if isinstance(node, ast.AugAssign):
            sym = {ast.Add: "+", ast.Sub: "-", ast.Mult: "*", ast.Div: "/"}.get(type(node.op))
            if sym is None:
                self.err(node, "unsupported augmented assignment")
            v, t = self.expr(node.value)
            if isinstance(node.target, ast.Name):
                cn, ct = self.env[node.target.id]
                if ct.kind == T.ARR:
                    vi = f"{v}[i_]" if t.kind == T.ARR else v
                    self.emit(f"for (int i_ = 0; i_ < {ct.n}; i_++) {cn}[i_] = {cn}[i_] {sym} {vi};")
                else:
                    self.emit(f"{cn} = {cn} {sym} {v};")
                return
            lhs, lt = self.subscript_target(node.target)
            if lt.kind == T.ARR:
                vi = f"{v}[i_]" if t.kind == T.ARR else v
                self.emit(f"for (int i_ = 0; i_ < {lt.n}; i_++) {lhs}[i_] = {lhs}[i_] {sym} {vi};")
            else:
                self.emit(f"{lhs} = {lhs} {sym} {v};")
            return
        if isinstance(node, ast.If):
            c, _ = self.expr(node.test)
            self.emit(f"if ({c}) {{")
            self.block(node.body)
            if node.orelse:
                self.emit("} else {")
                self.block(node.orelse)
            self.emit("}")
            return
        if isinstance(node, ast.For):
            if not (isinstance(node.iter, ast.Call) and isinstance(node.iter.func, ast.Name) and
                    node.iter.func.id == "range" and isinstance(node.target, ast.Name)):
                self.err(node, "only `for i in range(...)` loops")
            a = [self.const(x) for x in node.iter.args]
            if any(x is None for x in a):
                self.err(node, "range() bounds must be known at translation time")
            lo, hi = (0, a[0]) if len(a) == 1 else (a[0], a[1])
            step = a[2] if len(a) == 3 else 1
            if step == 0:
                self.err(node, "range() step of 0")
            var = node.target.id
            cn = f"v_{var}"
            cmp = "<" if step > 0 else ">"
            self.emit(f"for (int {cn} = {lo}; {cn} {cmp} {hi}; {cn} += {step}) {{")
            old = self.env.get(var)
            self.env[var] = (cn, INT)
            self.block(node.body)
            if old is None:
                del self.env[var]
            else:
                self.env[var] = old
            self.emit("}")
            return
        if isinstance(node, ast.Return):
            v, t = self.expr(node.value)
            self.tr.on_return(self, v, t, node)
            return
        if isinstance(node, ast.Pass):
            return
        self.err(node, f"unsupported statement {type(node).__name__}")

    def subscript_target(self, node):
        v, t = self.subscript(node)
        return v, t

    def block(self, body):
        # names first bound inside a block are hoisted so they outlive it
        self.depth += 1
        for s in body:
            self.stmt(s)
        self.depth -= 1

    def hoist(self):
        """Declare, before the body, every name assigned in a nested block."""
        pass


class Translator:
    def __init__(self, ndim, V):
        self.ndim, self.V = ndim, V
        self.helpers = {}
        self.helper_src = []

    # the callback's own return: write into `out`
    def on_return(self, fn, v, t, node):
        want = fn.ret_len
        if t.kind != T.ARR or t.n != want:
            fn.err(node, f"must return an array of {want} values")
        fn.emit(f"for (int i_ = 0; i_ < {want}; i_++) out[i_] = {v}[i_];")
        fn.emit("return;")

    def call_helper(self, fn, target, args, node):
        # arguments known at translation time (sizes, flags) specialise the
        # helper; the others become parameters
        consts = [fn.const(a) for a in args]
        vals = [None if c is not None else fn.expr(a) for a, c in zip(args, consts)]
        key = (target, tuple(("c", c) if c is not None else (v[1].kind, v[1].shape)
                             for c, v in zip(consts, vals)))
        if key not in self.helpers:
            self.helpers[key] = self.translate_helper(
                target, [None if v is None else v[1] for v in vals], consts)
        cname, rt = self.helpers[key]
        argv = ", ".join(v[0] for v in vals if v is not None)
        if rt.kind == T.ARR:
            out = fn.new(rt)
            fn.emit(f"{cname}({argv}{', ' if argv else ''}{out});")
            return out, rt
        return f"{cname}({argv})", rt

    def translate_helper(self, func, arg_types, consts):
        h = Fn(self, func, None)
        names = [a.arg for a in h.node.args.args]
        if len(names) != len(arg_types):
            raise TranslateError(f"{func.__name__}: wrong number of arguments")
        params = []
        for nm, t, c in zip(names, arg_types, consts):
            if c is not None:
                h.globals[nm] = c
                continue
            if t.kind == T.ARR:
                params.append(f"const double *p_{nm}")
            elif t.kind == T.INT:
                params.append(f"int p_{nm}")
            else:
                params.append(f"double p_{nm}")
            h.env[nm] = (f"p_{nm}", t)
        rtype = {}

        def on_ret(fn, v, t, node):
            if "t" not in rtype:
                rtype["t"] = t
            if t.kind == T.ARR:
                fn.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) ret_[i_] = {v}[i_];")
                fn.emit("return;")
            else:
                fn.emit(f"return {v};")
        saved = self.on_return
        self.on_return = on_ret
        try:
            for s in h.node.body:
                h.stmt(s)
        finally:
            self.on_return = saved
        rt = rtype.get("t", FLT)
        cname = f"h_{func.__name__.strip('<>')}_{len(self.helpers)}"
        if rt.kind == T.ARR:
            sig = f"__device__ __forceinline__ void {cname}({', '.join(params + ['double *ret_'])})"
        else:
            ctype = "int" if rt.kind == T.INT else "double"
            sig = f"__device__ __forceinline__ {ctype} {cname}({', '.join(params)})"
        self.helper_src.append(sig + " {\n" + "\n".join(h.lines) + "\n}\n")
        return cname, rt

    def callback(self, func, role):
        fn = Fn(self, func, None)
        names = [a.arg for a in fn.node.args.args]
        V, nd = self.V, self.ndim
        if role == "F":
            sig = "static __device__ void F(double *out, const double *Q, const double *dQ, int d)"
            fn.ret_len = V
            if len(names) == 1:
                fn.env[names[0]] = ("Q", _arr(V))
            elif len(names) == 2:
                fn.env[names[0]] = ("Q", _arr(V))
                fn.env[names[1]] = ("d", INT)
            elif len(names) == 3:
                fn.env[names[0]] = ("Q", _arr(V))
                fn.env[names[1]] = ("dQ", _arr(nd, V))
                fn.env[names[2]] = ("d", INT)
            else:
                raise TranslateError("F takes (Q), (Q, d) or (Q, DQ, d)")
        elif role == "B":
            sig = "static __device__ void B(double *out, const double *Q, int d)"
            fn.ret_len = V * V
            fn.env[names[0]] = ("Q", _arr(V))
            if len(names) == 2:
                fn.env[names[1]] = ("d", INT)
            elif len(names) != 1:
                raise TranslateError("B takes (Q) or (Q, d)")
        else:
            sig = "static __device__ void S(double *out, const double *Q)"
            fn.ret_len = V
            if len(names) != 1:
                raise TranslateError("S takes (Q)")
            fn.env[names[0]] = ("Q", _arr(V))
        fn.depth = fn.base_depth = 2
        for s in fn.node.body:
            fn.stmt(s)
        body = "\n".join(fn.lines)
        return f"  {sig} {{\n{body}\n  }}\n"


def translate(F, B, S, ndim, V):
    """CUDA C++ source of `struct UserSystem` for the given callbacks."""
    tr = Translator(ndim, V)
    parts = {}
    for role, f in (("F", F), ("B", B), ("S", S)):
        if f is not None:
            parts[role] = tr.callback(f, role)
    second = F is not None and len(inspect.signature(F).parameters) == 3
    lines = ["struct UserSystem {",
             f"  static constexpr int V = {V}, NDIM = {ndim};",
             f"  static constexpr bool HAS_F = {str(F is not None).lower()}, "
             f"HAS_B = {str(B is not None).lower()}, HAS_S = {str(S is not None).lower()};",
             f"  static constexpr bool SECOND_ORDER = {str(second).lower()};",
             "  static constexpr bool HAS_FP32 = false; // double callbacks only"]
    for role, sig in (("F", "static __device__ void F(double *, const double *, const double *, int) {}"),
                      ("B", "static __device__ void B(double *, const double *, int) {}"),
                      ("S", "static __device__ void S(double *, const double *) {}")):
        lines.append(parts.get(role, "  " + sig + "\n"))
    lines.append("};")
    helpers = "".join(tr.helper_src)
    return helpers + "\n".join(lines) + "\n"
