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
  * + - * / ** (x**2 -> x*x, x**0.5 -> sqrt; elementwise for an array with
    a constant exponent), unary -, comparisons, and/or/
    not, `a if c else b`; arrays combine elementwise and broadcast scalars;
  * Q[i], Q[a:b], DQ[d][i], DQ[d, i], DQ[d]; slices are views, as numpy's,
    so `ret[a:b] = x` and `ret[i, a:b] -= x` write into ret; slice bounds
    are constants or x + a : x + b around one expression (`5 + d:8 + d`);
  * zeros(n), zeros((n, m)), ones, full, eye(n), array([...]),
    array([[...], ...]), concatenate / hstack of vectors and scalars, len(),
    list comprehensions `[expr for i in range(...)]`, abs, min/max of two
    values (elementwise for arrays) or of one array,
    maximum/minimum, where, sign, square, clip, arctan2, hypot, copysign,
    fmod, sqrt, exp, log, sin, cos, tan,
    tanh, pow, floor, sum, prod, norm, outer, cross (3-vectors), trace,
    det (up to 3x3), dot / @ for vectors and matrices, and the
    array methods and attributes copy, reshape, ravel, flatten, sum, dot,
    transpose and .T (with or without a numpy / numpy.linalg / math prefix);
  * calls to other plain Python functions, also through a module attribute
    (translated as device functions; a numba-jitted helper contributes its
    Python function), including helpers that return a tuple, which unpacks
    at the call site: `rho, v, A = get_variables(Q)`;
  * numeric constants from the callback's globals, closure or an imported
    module; comparisons of constants fold, so a branch on a module flag
    (`if EOS == STIFFENED_GAS:`, `if tau == inf:`) keeps only its taken side
    and code after a return that always runs is not translated;
  * any Python identifier (Greek letters included): C names are ASCII;
  * integer // and % floor as Python's do, negative operands included;
    a negative index counts from the end (a computed index is checked for
    this when its expression contains a minus sign), and a constant index
    outside its dimension is refused.
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


def _cid(name):
    """An ASCII C identifier for a Python identifier (Python allows letters
    such as the Greek ones the reference's examples use; C++ compilers need
    not): other characters become _u<hex>_."""
    return "".join(c if (c.isascii() and (c.isalnum() or c == "_")) else f"_u{ord(c):x}_"
                   for c in name)


class T:
    """Type of a translated expression: int, float, an array shape, or the
    tuple a helper function returns (elems: the types of its items)."""
    INT, FLT, ARR, TUP = "int", "float", "arr", "tuple"

    def __init__(self, kind, shape=(), elems=()):
        self.kind, self.shape, self.elems = kind, tuple(shape), tuple(elems)

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
        self.rebinds = 0
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

    def copy(self, v, t):
        out = self.new(t)
        self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {v}[i_];")
        return out

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
            if isinstance(v, (int, float)):
                return v
            return None
        if isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name):
            if node.value.id in ("math", "np", "numpy") and node.attr in ("pi", "e", "inf"):
                return getattr(math, node.attr)
            mod = self.globals.get(node.value.id)
            if node.value.id not in self.env and inspect.ismodule(mod):
                v = getattr(mod, node.attr, None)
                if isinstance(v, (int, float)) and not isinstance(v, bool):
                    return v
            return None
        if isinstance(node, ast.Compare):
            # comparisons of translation-time constants fold, so branches on
            # module flags (an equation-of-state switch, an infinite
            # relaxation time) drop out with the code they guard
            vals = [self.const(node.left)] + [self.const(c) for c in node.comparators]
            if any(v is None for v in vals):
                return None
            cmp = {ast.Lt: lambda x, y: x < y, ast.LtE: lambda x, y: x <= y,
                   ast.Gt: lambda x, y: x > y, ast.GtE: lambda x, y: x >= y,
                   ast.Eq: lambda x, y: x == y, ast.NotEq: lambda x, y: x != y}
            if any(type(op) not in cmp for op in node.ops):
                return None
            return all(cmp[type(op)](a, b) for op, a, b in zip(node.ops, vals, vals[1:]))
        if isinstance(node, ast.BoolOp):
            vals = [self.const(v) for v in node.values]
            if any(v is None for v in vals):
                return None
            return all(vals) if isinstance(node.op, ast.And) else any(vals)
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.Not):
            v = self.const(node.operand)
            return None if v is None else (not v)
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
                cn = f"g_{_cid(node.id)}"
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
                if t.kind == T.ARR:
                    self.err(node, "`not` of an array (its truth value is ambiguous)")
                return f"(!({v}))", INT
            self.err(node, "unsupported unary operator")
        if isinstance(node, ast.BinOp):
            return self.binop(node)
        if isinstance(node, ast.BoolOp):
            op = " && " if isinstance(node.op, ast.And) else " || "
            parts = []
            for v in node.values:
                pv, pt = self.expr(v)
                if pt.kind == T.ARR:
                    self.err(node, "and/or of an array (its truth value is ambiguous)")
                parts.append(pv)
            return "(" + op.join(f"({p})" for p in parts) + ")", INT
        if isinstance(node, ast.Compare):
            ops = {ast.Lt: "<", ast.LtE: "<=", ast.Gt: ">", ast.GtE: ">=", ast.Eq: "==",
                   ast.NotEq: "!="}
            left, tl = self.expr(node.left)
            if len(node.ops) == 1 and type(node.ops[0]) in ops:
                r, tr = self.expr(node.comparators[0])
                if T.ARR in (tl.kind, tr.kind):  # elementwise: 1.0 / 0.0 per item
                    t = tl if tl.kind == T.ARR else tr
                    if tl.kind == tr.kind == T.ARR and tl.n != tr.n:
                        self.err(node, "arrays of different lengths")
                    out = self.new(t)
                    li = f"{left}[i_]" if tl.kind == T.ARR else left
                    ri = f"{r}[i_]" if tr.kind == T.ARR else r
                    self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) "
                              f"{out}[i_] = ({li} {ops[type(node.ops[0])]} {ri}) ? 1.0 : 0.0;")
                    return out, t
                return f"(({left}) {ops[type(node.ops[0])]} ({r}))", INT
            parts = []
            for op, right in zip(node.ops, node.comparators):
                r, _ = self.expr(right)
                if type(op) not in ops:
                    self.err(node, "unsupported comparison")
                parts.append(f"({left} {ops[type(op)]} {r})")
                left = r
            return "(" + " && ".join(parts) + ")", INT
        if isinstance(node, ast.IfExp):
            c, tc = self.expr(node.test)
            if tc.kind == T.ARR:
                self.err(node, "the condition is an array (its truth value is ambiguous)")
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
        if isinstance(node, ast.Attribute) and node.attr == "T":
            v, t = self.expr(node.value)
            return self.transpose(v, t, node)
        if isinstance(node, (ast.List, ast.Tuple)):
            return self.array_literal(node.elts, node)
        if isinstance(node, ast.ListComp):
            return self.list_comp(node)
        self.err(node, f"unsupported expression {type(node).__name__}")

    def list_comp(self, node):
        """[expr for i in range(...)] with bounds known at translation time
        and a scalar expr: a loop that fills an array."""
        if len(node.generators) != 1 or node.generators[0].ifs or \
                node.generators[0].is_async:
            self.err(node, "list comprehensions need one `for i in range(...)` and no if")
        gen = node.generators[0]
        if not (isinstance(gen.iter, ast.Call) and isinstance(gen.iter.func, ast.Name) and
                gen.iter.func.id == "range" and isinstance(gen.target, ast.Name)):
            self.err(node, "list comprehensions need `for i in range(...)`")
        a = [self.const(x) for x in gen.iter.args]
        if any(not isinstance(x, int) for x in a):
            self.err(node, "range() bounds must be known at translation time")
        lo, hi = (0, a[0]) if len(a) == 1 else (a[0], a[1])
        step = a[2] if len(a) == 3 else 1
        if step == 0:
            self.err(node, "range() step of 0")
        count = len(range(lo, hi, step))
        if count < 1:
            self.err(node, "empty list comprehension")
        t = _arr(count)
        out = self.new(t)
        var = gen.target.id
        cn = f"v_{_cid(var)}"
        cmp = "<" if step > 0 else ">"
        self.emit(f"for (int {cn} = {lo}, k_ = 0; {cn} {cmp} {hi}; {cn} += {step}, k_++) {{")
        old = self.env.get(var)
        self.env[var] = (cn, INT)
        self.depth += 1
        v, vt = self.expr(node.elt)
        if vt.kind == T.ARR:
            self.err(node, "list comprehension items must be scalars")
        self.emit(f"{out}[k_] = {v};")
        self.depth -= 1
        if old is None:
            del self.env[var]
        else:
            self.env[var] = old
        self.emit("}")
        return out, t

    def index_expr(self, node, size=None):
        """C expression of an integer index.  A constant index into a
        dimension of the given size wraps from the end when negative, as in
        Python, and must lie inside it."""
        c = self.const(node)
        if c is not None:
            if not isinstance(c, int) or isinstance(c, bool):
                self.err(node, "index must be an integer")
            if size is not None:
                if c < 0:
                    c += size
                if not 0 <= c < size:
                    self.err(node, f"index out of range for a dimension of {size}")
            return str(c), c
        v, t = self.expr(node)
        if t.kind != T.INT:
            self.err(node, "index must be an integer expression")
        if size is not None:
            # a negative index counts from the end, as in Python, whether it
            # is written with a minus sign or held in a name (k = -1; Q[k],
            # a loop over range(-3, 0)); a compare and select per access.
            # The expression stays where it is written (not hoisted into a
            # temporary), so that one under a conditional expression is not
            # evaluated when its branch is not taken
            v = f"(({v}) < 0 ? ({v}) + {size} : ({v}))"
        return v, None

    def _offset(self, node):
        """Split node into (x, a) with node == x + a for a constant integer
        a (a = 0 when there is none)."""
        if isinstance(node, ast.BinOp) and isinstance(node.op, (ast.Add, ast.Sub)):
            c = self.const(node.right)
            if isinstance(c, int) and not isinstance(c, bool):
                return node.left, (c if isinstance(node.op, ast.Add) else -c)
            c = self.const(node.left)
            if isinstance(c, int) and not isinstance(c, bool) and isinstance(node.op, ast.Add):
                return node.right, c
        return node, 0

    def _slice(self, s, size, node):
        """(C expression of the start, length) of a step-1 slice whose length
        is known at translation time: constant bounds (numpy's negative and
        clipped bounds included), or bounds x + a : x + b around one
        expression x."""
        if s.step is not None and self.const(s.step) != 1:
            self.err(node, "slices need step 1")
        lo = 0 if s.lower is None else self.const(s.lower)
        hi = size if s.upper is None else self.const(s.upper)
        if lo is not None and hi is not None:
            lo = max(lo + size, 0) if lo < 0 else min(lo, size)
            hi = max(hi + size, 0) if hi < 0 else min(hi, size)
            if hi <= lo:
                self.err(node, "empty slice")
            return str(lo), hi - lo
        if s.lower is None or s.upper is None:
            self.err(node, "slices need constant bounds or bounds x + a : x + b")
        xl, al = self._offset(s.lower)
        xu, au = self._offset(s.upper)
        if ast.dump(xl) != ast.dump(xu) or au <= al:
            self.err(node, "slices need constant bounds or bounds x + a : x + b")
        lo_c, _ = self.index_expr(s.lower)
        return lo_c, au - al

    def subscript(self, node, target=False):
        """Elements, rows and slices.  Slices and rows of contiguous memory
        are views (a pointer into the array), as numpy's are, so they can be
        assigned to; a column slice of a 2-D array is a copy and cannot."""
        base, bt = self.expr(node.value)
        if bt.kind != T.ARR:
            self.err(node, "subscript of a scalar")
        sl = node.slice
        idx = sl.elts if isinstance(sl, ast.Tuple) else [sl]
        if len(idx) == 1 and isinstance(idx[0], ast.Slice):
            lo, n = self._slice(idx[0], bt.shape[0], node)
            if len(bt.shape) == 1:
                return f"({base} + {lo})", _arr(n)
            return f"({base} + ({lo}) * {bt.shape[1]})", _arr(n, bt.shape[1])
        if len(idx) == 1 and len(bt.shape) == 2:
            r, _ = self.index_expr(idx[0], bt.shape[0])
            return f"({base} + ({r}) * {bt.shape[1]})", _arr(bt.shape[1])  # row view
        if len(idx) == 1:
            i, _ = self.index_expr(idx[0], bt.shape[0])
            return f"{base}[{i}]", FLT
        if len(idx) == 2 and len(bt.shape) == 2:
            ncol = bt.shape[1]
            rs, cs = isinstance(idx[0], ast.Slice), isinstance(idx[1], ast.Slice)
            if not rs and not cs:
                i, _ = self.index_expr(idx[0], bt.shape[0])
                j, _ = self.index_expr(idx[1], ncol)
                return f"{base}[({i}) * {ncol} + ({j})]", FLT
            if not rs:  # part of one row: contiguous
                i, _ = self.index_expr(idx[0], bt.shape[0])
                lo, n = self._slice(idx[1], ncol, node)
                return f"({base} + ({i}) * {ncol} + ({lo}))", _arr(n)
            if target:
                self.err(node, "assignment to a column slice of a 2-D array")
            rlo, nr = self._slice(idx[0], bt.shape[0], node)
            if not cs:
                j, _ = self.index_expr(idx[1], ncol)
                t = _arr(nr)
                out = self.new(t)
                self.emit(f"for (int i_ = 0; i_ < {nr}; i_++) "
                          f"{out}[i_] = {base}[(({rlo}) + i_) * {ncol} + ({j})];")
                return out, t
            clo, nc = self._slice(idx[1], ncol, node)
            t = _arr(nr, nc)
            out = self.new(t)
            self.emit(f"for (int i_ = 0; i_ < {nr * nc}; i_++) {out}[i_] = "
                      f"{base}[(({rlo}) + i_ / {nc}) * {ncol} + ({clo}) + i_ % {nc}];")
            return out, t
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
        if isinstance(op, ast.MatMult):
            return self.dot(*self.expr(node.left), *self.expr(node.right), node)
        if isinstance(op, ast.Pow):
            b, tb = self.expr(node.left)
            e = self.const(node.right)
            if tb.kind == T.ARR:  # elementwise, with the scalar rules below
                if e is None:
                    self.err(node, "array ** needs a constant exponent")
                out = self.new(tb)
                x = f"{b}[i_]"
                item = f"{x} * {x}" if e == 2 else (f"sqrt({x})" if e == 0.5 else
                                                    (x if e == 1 else
                                                     f"pow({x}, (double)({self.lit(e)}))"))
                self.emit(f"for (int i_ = 0; i_ < {tb.n}; i_++) {out}[i_] = {item};")
                return out, tb
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
                    # Python floors: when the remainder is non-zero and the
                    # operands' signs differ, C's truncated quotient is one
                    # too large and its remainder lacks one divisor
                    adj = f"((({a}) % ({b})) != 0 && ((({a}) < 0) != (({b}) < 0)))"
                    if isinstance(op, ast.FloorDiv):
                        return f"((({a}) / ({b})) - {adj})", INT
                    return f"((({a}) % ({b})) + ({adj} ? ({b}) : 0))", INT
                self.tr.py_divmod_helpers()
                fn = "py_floordiv_" if isinstance(op, ast.FloorDiv) else "py_mod_"
                return f"{fn}((double)({a}), (double)({b}))", FLT
            t = INT if ta.kind == tb.kind == T.INT else FLT
            return f"({a} {sym} {b})", t
        # elementwise with broadcasting of scalars
        t = ta if ta.kind == T.ARR else tb
        if ta.kind == T.ARR and tb.kind == T.ARR and ta.n != tb.n:
            self.err(node, "arrays of different lengths")
        out = self.new(t)
        ai = f"{a}[i_]" if ta.kind == T.ARR else a
        bi = f"{b}[i_]" if tb.kind == T.ARR else b
        if isinstance(op, (ast.FloorDiv, ast.Mod)):  # numpy floors, as Python does
            self.tr.py_divmod_helpers()
            fn = "py_floordiv_" if isinstance(op, ast.FloorDiv) else "py_mod_"
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) "
                      f"{out}[i_] = {fn}((double)({ai}), (double)({bi}));")
            return out, t
        self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {ai} {sym} {bi};")
        return out, t

    def transpose(self, v, t, node):
        if t.kind != T.ARR or len(t.shape) > 2:
            self.err(node, "transpose of a scalar")
        if len(t.shape) == 1:
            return v, t
        m, n = t.shape
        rt = _arr(n, m)
        out = self.new(rt)
        self.emit(f"for (int i_ = 0; i_ < {m * n}; i_++) "
                  f"{out}[i_] = {v}[(i_ % {m}) * {n} + i_ / {m}];")
        return out, rt

    def dot(self, a, ta, b, tb, node):
        """numpy's dot / @ for 1-D and 2-D operands; each sum runs over the
        shared index in increasing order."""
        if ta.kind != T.ARR or tb.kind != T.ARR:
            self.err(node, "dot of a scalar")
        sa, sb = ta.shape, tb.shape
        if sa[-1] != sb[0]:
            self.err(node, f"dot of shapes {sa} and {sb}")
        k = sa[-1]
        if len(sa) == 1 and len(sb) == 1:
            acc = self.new(FLT, "0.0")
            self.emit(f"for (int i_ = 0; i_ < {k}; i_++) {acc} += {a}[i_] * {b}[i_];")
            return acc, FLT
        m = sa[0] if len(sa) == 2 else 1
        n = sb[1] if len(sb) == 2 else 1
        shape = tuple(x for x, keep in ((m, len(sa) == 2), (n, len(sb) == 2)) if keep)
        rt = _arr(*shape)
        out = self.new(rt)
        self.emit(f"for (int i_ = 0; i_ < {m}; i_++) for (int j_ = 0; j_ < {n}; j_++) {{")
        self.emit(f"  double s_ = 0.0;")
        self.emit(f"  for (int k_ = 0; k_ < {k}; k_++) "
                  f"s_ += {a}[i_ * {k} + k_] * {b}[k_ * {n} + j_];")
        self.emit(f"  {out}[i_ * {n} + j_] = s_;")
        self.emit("}")
        return out, rt

    def det(self, v, t, node):
        """Determinant of a 1x1, 2x2 or 3x3 matrix by cofactor expansion
        along the first row."""
        if t.kind != T.ARR or len(t.shape) != 2 or t.shape[0] != t.shape[1] or t.shape[0] > 3:
            self.err(node, "det() of a 1x1, 2x2 or 3x3 matrix only")
        n = t.shape[0]
        a = [[f"{v}[{i * n + j}]" for j in range(n)] for i in range(n)]
        if n == 1:
            return a[0][0], FLT
        if n == 2:
            return f"({a[0][0]} * {a[1][1]} - {a[0][1]} * {a[1][0]})", FLT
        m = [f"({a[1][1]} * {a[2][2]} - {a[1][2]} * {a[2][1]})",
             f"({a[1][0]} * {a[2][2]} - {a[1][2]} * {a[2][0]})",
             f"({a[1][0]} * {a[2][1]} - {a[1][1]} * {a[2][0]})"]
        return f"({a[0][0]} * {m[0]} - {a[0][1]} * {m[1]} + {a[0][2]} * {m[2]})", FLT

    def method(self, node, obj, attr, args):
        """Array methods: copy, reshape, ravel/flatten, transpose, sum, dot."""
        v, t = self.expr(obj)
        if t.kind != T.ARR:
            self.err(node, f".{attr}() of a scalar")
        if attr == "copy":
            return self.copy(v, t), t
        if attr == "reshape":
            dims = args[0].elts if len(args) == 1 and isinstance(args[0], (ast.Tuple, ast.List)) \
                else args
            shape = [self.const(x) for x in dims]
            if any(not isinstance(x, int) for x in shape):
                self.err(node, "reshape() needs a constant shape")
            if -1 in shape:
                rest = 1
                for x in shape:
                    rest *= x if x != -1 else 1
                shape[shape.index(-1)] = t.n // rest
            nt = _arr(*shape)
            if nt.n != t.n:
                self.err(node, f"cannot reshape {t.shape} to {tuple(shape)}")
            return v, nt
        if attr in ("ravel", "flatten"):
            return (self.copy(v, t) if attr == "flatten" else v), _arr(t.n)
        if attr == "transpose":
            return self.transpose(v, t, node)
        if attr == "sum" and not args:
            acc = self.new(FLT, "0.0")
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {acc} += {v}[i_];")
            return acc, FLT
        if attr == "dot" and len(args) == 1:
            return self.dot(v, t, *self.expr(args[0]), node)
        self.err(node, f"unsupported array method .{attr}()")

    def call(self, node):
        f = node.func
        args = node.args
        name = None
        if isinstance(f, ast.Attribute):
            # np.f, numpy.linalg.f, math.f, a module's function, or a method
            chain, base = [f.attr], f.value
            while isinstance(base, ast.Attribute):
                chain.append(base.attr)
                base = base.value
            root = base.id if isinstance(base, ast.Name) else None
            mod = None if root is None or root in self.env else self.globals.get(root)
            if root in ("np", "numpy", "math") or (inspect.ismodule(mod) and
                                                   mod.__name__.split(".")[0] in
                                                   ("numpy", "math")):
                name = f.attr
            elif inspect.ismodule(mod):
                target = mod
                for a in reversed(chain):
                    target = getattr(target, a, None)
                if target is not None and hasattr(target, "py_func"):
                    target = target.py_func
                if callable(target) and hasattr(target, "__code__"):
                    return self.tr.call_helper(self, target, args, node)
                self.err(node, f"unsupported function {'.'.join([root] + chain[::-1])}")
            else:
                return self.method(node, f.value, f.attr, args)
        elif isinstance(f, ast.Name):
            name = f.id
        else:
            self.err(node, "unsupported call")
        if name in ("eye", "identity"):
            n = self.const(args[0])
            if not isinstance(n, int):
                self.err(node, f"{name}() needs a constant size")
            t = _arr(n, n)
            out = self.new(t)
            self.emit(f"for (int i_ = 0; i_ < {n * n}; i_++) "
                      f"{out}[i_] = (i_ % {n + 1} == 0) ? 1.0 : 0.0;")
            return out, t
        if name == "transpose" and len(args) == 1:
            return self.transpose(*self.expr(args[0]), node)
        if name == "trace" and len(args) == 1:
            v, t = self.expr(args[0])
            if t.kind != T.ARR or len(t.shape) != 2:
                self.err(node, "trace() of a matrix only")
            acc = self.new(FLT, "0.0")
            self.emit(f"for (int i_ = 0; i_ < {min(t.shape)}; i_++) "
                      f"{acc} += {v}[i_ * {t.shape[1] + 1}];")
            return acc, FLT
        if name == "det" and len(args) == 1:
            return self.det(*self.expr(args[0]), node)
        if name in ("matmul",) and len(args) == 2:
            return self.dot(*self.expr(args[0]), *self.expr(args[1]), node)
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
        if name in ("ones", "full", "ones_like", "full_like"):
            if name.endswith("_like"):
                shape = self.expr(args[0])[1].shape
            else:
                a0 = args[0]
                shape = tuple(self.const(e) for e in a0.elts) \
                    if isinstance(a0, (ast.Tuple, ast.List)) else (self.const(a0),)
                if any(not isinstance(x, int) for x in shape):
                    self.err(node, f"{name}() needs a constant shape")
            fill = "1.0"
            if name.startswith("full"):
                fv, ft = self.expr(args[1])
                if ft.kind == T.ARR:
                    self.err(node, f"{name}() needs a scalar fill value")
                fill = f"(double)({fv})"
            t = _arr(*shape)
            out = self.new(t)
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {fill};")
            return out, t
        if name in ("max", "min", "amax", "amin") and len(args) == 1:
            # the largest / smallest element, found in index order
            v, t = self.expr(args[0])
            if t.kind != T.ARR:
                self.err(node, f"{name}() of one scalar")
            acc = self.new(FLT, f"{v}[0]")
            cmp = ">" if name in ("max", "amax") else "<"
            self.emit(f"for (int i_ = 1; i_ < {t.n}; i_++) "
                      f"if ({v}[i_] {cmp} {acc}) {acc} = {v}[i_];")
            return acc, FLT
        if name in ("sign", "square", "clip"):
            v, t = self.expr(args[0])
            if name == "clip":
                lo, _ = self.expr(args[1])
                hi, _ = self.expr(args[2])

            def one(x):
                if name == "sign":
                    return f"(({x}) > 0.0 ? 1.0 : (({x}) < 0.0 ? -1.0 : 0.0))"
                if name == "square":
                    return f"(({x}) * ({x}))"
                return f"fmin(fmax((double)({x}), (double)({lo})), (double)({hi}))"
            if t.kind == T.ARR:
                out = self.new(t)
                self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {one(f'{v}[i_]')};")
                return out, t
            return one(v), (FLT if name != "square" or t.kind != T.INT else INT)
        if name in ("arctan2", "atan2", "hypot", "copysign", "fmod") and len(args) == 2:
            fn = {"arctan2": "atan2"}.get(name, name)
            a, ta = self.expr(args[0])
            b, tb = self.expr(args[1])
            if T.ARR in (ta.kind, tb.kind):
                t = ta if ta.kind == T.ARR else tb
                out = self.new(t)
                ai = f"{a}[i_]" if ta.kind == T.ARR else f"(double)({a})"
                bi = f"{b}[i_]" if tb.kind == T.ARR else f"(double)({b})"
                self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {fn}({ai}, {bi});")
                return out, t
            return f"{fn}((double)({a}), (double)({b}))", FLT
        if name == "where" and len(args) == 3:
            c, tc = self.expr(args[0])
            a, ta = self.expr(args[1])
            b, tb = self.expr(args[2])
            if T.ARR in (tc.kind, ta.kind, tb.kind):  # elementwise, scalars broadcast
                t = next(x for x in (tc, ta, tb) if x.kind == T.ARR)
                out = self.new(t)
                ci, ai, bi = ((f"{v}[i_]" if tv.kind == T.ARR else f"({v})")
                              for v, tv in ((c, tc), (a, ta), (b, tb)))
                self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) "
                          f"{out}[i_] = ({ci}) ? (double){ai} : (double){bi};")
                return out, t
            return f"(({c}) ? (double)({a}) : (double)({b}))", FLT
        if name == "prod" and len(args) == 1:
            v, t = self.expr(args[0])
            acc = self.new(FLT, "1.0")
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {acc} *= {v}[i_];")
            return acc, FLT
        if name == "norm" and len(args) == 1:
            # 2-norm of a vector, Frobenius norm of a matrix
            v, t = self.expr(args[0])
            acc = self.new(FLT, "0.0")
            self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {acc} += {v}[i_] * {v}[i_];")
            return f"sqrt({acc})", FLT
        if name == "outer" and len(args) == 2:
            a, ta = self.expr(args[0])
            b, tb = self.expr(args[1])
            t = _arr(ta.n, tb.n)
            out = self.new(t)
            self.emit(f"for (int i_ = 0; i_ < {ta.n * tb.n}; i_++) "
                      f"{out}[i_] = {a}[i_ / {tb.n}] * {b}[i_ % {tb.n}];")
            return out, t
        if name == "cross" and len(args) == 2:
            a, ta = self.expr(args[0])
            b, tb = self.expr(args[1])
            if ta.shape != (3,) or tb.shape != (3,):
                self.err(node, "cross() of two 3-vectors only")
            t = _arr(3)
            out = self.new(t)
            for i in range(3):
                j, k = (i + 1) % 3, (i + 2) % 3
                self.emit(f"{out}[{i}] = {a}[{j}] * {b}[{k}] - {a}[{k}] * {b}[{j}];")
            return out, t
        if name in ("concatenate", "hstack") and len(args) == 1 and \
                isinstance(args[0], (ast.Tuple, ast.List)):
            parts = [self.expr(e) for e in args[0].elts]
            n = sum(pt.n if pt.kind == T.ARR else 1 for _, pt in parts)
            t = _arr(n)
            out = self.new(t)
            off = 0
            for pv, pt in parts:
                if pt.kind == T.ARR:
                    self.emit(f"for (int i_ = 0; i_ < {pt.n}; i_++) {out}[{off} + i_] = {pv}[i_];")
                    off += pt.n
                else:
                    self.emit(f"{out}[{off}] = (double)({pv});")
                    off += 1
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
            if T.ARR in (ta.kind, tb.kind):  # elementwise, scalars broadcast
                t = ta if ta.kind == T.ARR else tb
                if ta.kind == tb.kind == T.ARR and ta.n != tb.n:
                    self.err(node, "arrays of different lengths")
                out = self.new(t)
                ai = f"{a}[i_]" if ta.kind == T.ARR else f"(double)({a})"
                bi = f"{b}[i_]" if tb.kind == T.ARR else f"(double)({b})"
                self.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) {out}[i_] = {fn}({ai}, {bi});")
                return out, t
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
            return self.dot(*self.expr(args[0]), *self.expr(args[1]), node)
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
        if name in self.env and self.env[name][0] in ("Q", "dQ") or \
                self.env.get(name, ("",))[0].startswith("p_"):
            # rebinding an input (Q = Q * 2, or a helper's parameter) makes
            # the name refer to a new array, as in Python; the caller's
            # array is left as it was
            del self.env[name]
            self.rebinds += 1
            name_c = f"{name}_r{self.rebinds}"
            self._declare(name, name_c, v, t)
            return
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
        self._declare(name, name, v, t)

    def _declare(self, name, cname, v, t):
        # Python names live for the whole function: declare at the top so a
        # name first bound inside an if/for block is visible after it
        cn = f"v_{_cid(cname)}"
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
                if not all(isinstance(e, ast.Name) for e in tgt.elts):
                    self.err(node, "tuple assignment to names only")
                nt = len(tgt.elts)
                if isinstance(node.value, ast.Tuple):
                    if len(node.value.elts) != nt:
                        self.err(node, "tuple assignment needs a tuple of the same length")
                    vals = [self.expr(e) for e in node.value.elts]
                else:
                    # a helper's tuple, or the items of a 1-D array
                    v, t = self.expr(node.value)
                    if t.kind == T.TUP and len(t.elems) == nt:
                        vals = list(zip(v, t.elems))
                    elif t.kind == T.ARR and len(t.shape) == 1 and t.shape[0] == nt:
                        vals = [(f"{v}[{k}]", FLT) for k in range(nt)]
                    else:
                        self.err(node, "tuple assignment needs a tuple of the same length")
                # evaluate every item before binding any name (a, b = b, a)
                tmps = [(self.copy(v, t) if t.kind == T.ARR else self.new(t, v), t)
                        for v, t in vals]
                for tg, (v, t) in zip(tgt.elts, tmps):
                    self.assign_name(tg.id, v, t, node)
                return
            v, t = self.expr(node.value)
            if isinstance(tgt, ast.Name):
                self.assign_name(tgt.id, v, t, node)
                return
            if isinstance(tgt, ast.Subscript):
                if t.kind == T.ARR and v.startswith("("):  # a view: may overlap
                    v = self.copy(v, t)
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
            if t.kind == T.ARR and v.startswith("("):  # a view: may overlap
                v = self.copy(v, t)
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
            k = self.const(node.test)
            if k is not None:  # known at translation time: only the taken side
                return self.run(node.body if k else node.orelse)
            c, tc = self.expr(node.test)
            if tc.kind == T.ARR:
                self.err(node, "the condition is an array (its truth value is ambiguous)")
            self.emit(f"if ({c}) {{")
            ends = self.block(node.body)
            if node.orelse:
                self.emit("} else {")
                ends = self.block(node.orelse) and ends
            else:
                ends = False
            self.emit("}")
            return ends
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
            cn = f"v_{_cid(var)}"
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
            if getattr(self, "is_helper", False) and isinstance(node.value, ast.Tuple):
                vals = [self.expr(e) for e in node.value.elts]
                self.tr.on_return(self, [v for v, _ in vals],
                                  T(T.TUP, elems=[t for _, t in vals]), node)
                return True
            v, t = self.expr(node.value)
            self.tr.on_return(self, v, t, node)
            return True
        if isinstance(node, ast.Pass):
            return
        self.err(node, f"unsupported statement {type(node).__name__}")

    def subscript_target(self, node):
        base = node.value
        while isinstance(base, ast.Subscript):
            base = base.value
        if isinstance(base, ast.Name) and self.env.get(base.id, ("",))[0] in ("Q", "dQ"):
            self.err(node, f"assignment into the callback's input {base.id}; "
                           f"copy it first ({base.id}.copy())")
        v, t = self.subscript(node, target=True)
        return v, t

    def run(self, body):
        """Translate statements until one that always returns (the rest is
        dead code, which may name things that exist only on other paths);
        True when the body always returns."""
        for s in body:
            if self.stmt(s):
                return True
        return False

    def block(self, body):
        # names first bound inside a block are hoisted so they outlive it
        self.depth += 1
        ends = self.run(body)
        self.depth -= 1
        return ends

    def hoist(self):
        """Declare, before the body, every name assigned in a nested block."""
        pass


# Python's float floor division and remainder (the semantics numpy's //
# and % follow): a % b takes the sign of b, a // b is (a - a % b) / b made
# an exact integer.  fmod is exact, so the quotient is off an integer only
# by the rounding of that one division.
PY_DIVMOD_SRC = """__device__ __forceinline__ double py_mod_(double a, double b) {
  double r = fmod(a, b);
  if (r != 0.0) {
    if ((r < 0.0) != (b < 0.0))
      r += b;
  } else {
    r = copysign(0.0, b);
  }
  return r;
}
__device__ __forceinline__ double py_floordiv_(double a, double b) {
  double r = fmod(a, b);
  double q = (a - r) / b;
  if (r != 0.0 && ((r < 0.0) != (b < 0.0)))
    q -= 1.0;
  if (q == 0.0)
    return copysign(0.0, a / b);
  double f = floor(q);
  if (q - f > 0.5)
    f += 1.0;
  return f;
}
"""


class Translator:
    def __init__(self, ndim, V):
        self.ndim, self.V = ndim, V
        self.helpers = {}
        self.helper_src = []
        self.divmod_emitted = False

    def py_divmod_helpers(self):
        if not self.divmod_emitted:
            self.divmod_emitted = True
            self.helper_src.insert(0, PY_DIVMOD_SRC)

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
        if rt.kind == T.TUP:
            outs, refs = [], []
            for et in rt.elems:
                o = fn.new(et)
                outs.append(o)
                refs.append(o if et.kind == T.ARR else f"&{o}")
            fn.emit(f"{cname}({argv}{', ' if argv else ''}{', '.join(refs)});")
            return outs, rt
        if rt.kind == T.ARR:
            out = fn.new(rt)
            fn.emit(f"{cname}({argv}{', ' if argv else ''}{out});")
            return out, rt
        return f"{cname}({argv})", rt

    def translate_helper(self, func, arg_types, consts):
        h = Fn(self, func, None)
        h.is_helper = True
        names = [a.arg for a in h.node.args.args]
        if len(names) != len(arg_types):
            raise TranslateError(f"{func.__name__}: wrong number of arguments")
        params = []
        for nm, t, c in zip(names, arg_types, consts):
            if c is not None:
                h.globals[nm] = c
                continue
            if t.kind == T.ARR:
                params.append(f"const double *p_{_cid(nm)}")
            elif t.kind == T.INT:
                params.append(f"int p_{_cid(nm)}")
            else:
                params.append(f"double p_{_cid(nm)}")
            h.env[nm] = (f"p_{_cid(nm)}", t)
        rtype = {}

        def same(a, b):
            return a.kind == b.kind and a.shape == b.shape or \
                (a.kind != T.ARR and b.kind != T.ARR and T.TUP not in (a.kind, b.kind))

        def on_ret(fn, v, t, node):
            # every return of a helper gives the same kind of value; a scalar
            # helper returns double when any of its returns is a float
            first = rtype.setdefault("t", t)
            if t.kind == T.TUP:
                if first.kind != T.TUP or len(first.elems) != len(t.elems) or \
                        not all(same(a, b) for a, b in zip(first.elems, t.elems)):
                    fn.err(node, "returns of different shapes")
                rtype["t"] = first = T(T.TUP, elems=[
                    FLT if FLT in (a, b) or T.FLT in (a.kind, b.kind) and a.kind != T.ARR
                    else a for a, b in zip(first.elems, t.elems)])
                for k, (vk, tk) in enumerate(zip(v, first.elems)):
                    if tk.kind == T.ARR:
                        fn.emit(f"for (int i_ = 0; i_ < {tk.n}; i_++) ret{k}_[i_] = {vk}[i_];")
                    else:
                        fn.emit(f"*ret{k}_ = {vk};")
                fn.emit("return;")
                return
            if not same(first, t):
                fn.err(node, "returns of different shapes")
            if t.kind == T.ARR:
                fn.emit(f"for (int i_ = 0; i_ < {t.n}; i_++) ret_[i_] = {v}[i_];")
                fn.emit("return;")
            else:
                if t.kind == T.FLT:
                    rtype["t"] = FLT
                fn.emit(f"return {v};")
        saved = self.on_return
        self.on_return = on_ret
        try:
            h.run(h.node.body)
        finally:
            self.on_return = saved
        rt = rtype.get("t", FLT)
        cname = f"h_{_cid(func.__name__.strip('<>'))}_{len(self.helpers)}"
        if rt.kind == T.TUP:
            outs = [f"{'int' if et.kind == T.INT else 'double'} *ret{k}_"
                    for k, et in enumerate(rt.elems)]
            sig = f"__device__ __forceinline__ void {cname}({', '.join(params + outs)})"
        elif rt.kind == T.ARR:
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
        fn.run(fn.node.body)
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
