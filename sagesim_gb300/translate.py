"""Translator from SAGESim's Python step dialect to a CUDA C++ step.

SAGESim step functions are CuPy-JIT Python (`@jit.rawkernel(device="cuda")`)
with the signature

    step(tick, agent_index, <globals...>, agent_ids, breeds, locations, <properties...>)

(the call the reference generates, sagesim/model.py:2312-2330: globals in
registration order, then the agent ids, then every property in property order,
starting with the breed and the neighbour rows). The reference rewrites the body
before compiling it: neighbour rows become CSR reads (`_CSRBodyTransformer`,
sagesim/model.py:1643-1902), the seed and the agent's logical id are injected into
`rand_uniform_philox` / `rand_normal` (`_inject_seed`, model.py:1903-1953), and
property writes go to the write buffer (model.py:2085-2222). This module applies
the same meaning while emitting C++ for `sg_compile_step`, whose `sg_ctx` already
implements those three rewrites (reads from the read buffer, writes to the write
buffer, `ctx.rand_uniform(i, salt)` with seed and logical id filled in).

Supported subset (what the reference's own step functions use): assignments and
augmented assignments to locals and to property elements, `if` / `elif` / `else`,
`while`, `for ... in range(...)`, `break`, `continue`, bare `return`; arithmetic,
comparisons, `and` / `or` / `not`; `int()`, `float()`, `bool()`, `abs()`, `min()`,
`max()` (of two or more values), `math` / `cp` `pi` and `e`, `len(row)`, `cp.float32()`, `cp.float64()`, `cp.int32()`, `cp.isnan()`,
`math` / `cp` `exp log sqrt sin cos tan tanh floor ceil fabs`;
`rand_uniform_philox(tick, agent, salt)` and `rand_normal(tick, agent, salt)`;
the helpers of sagesim/utils.py (`get_num_neighbors`, `get_neighbor`,
`get_this_agent_data_from_tensor`, `set_this_agent_data_from_tensor`);
`locations[a]` (a neighbour row), `row[k]`, `len(row)`; property reads `p[a]`,
`p[a][c]`, a local bound to a list property's row (`r = p[a]`, read as `r[c]`,
`len(r)`; also `len(p[a])`), writes `p[a] = v`, `p[a][c] = v`; breed-local
arrays `a[r][j]` (reads and writes) and their index maps; globals `g` and `g[k]`.

Types follow numpy's scalar rules as CuPy-JIT does: Python int and float
locals are int64 and float64, `cp.float32(...)` values are float32, a float32 with
an int64 or float64 operand becomes float64, Python number literals take the other
operand's type, `/` is true division, float `%` takes the divisor's sign (the
helpers for it are emitted only into steps that use it). Integer `//` and `%` keep Python's flooring
semantics. Anything outside the subset raises `StepTranslationError` naming the
line.
"""
import ast
import inspect
import os
import textwrap

__all__ = ["StepTranslationError", "translate_step", "find_step_source"]


class StepTranslationError(ValueError):
    pass


# types: "i" int64, "f" float32, "d" float64, "b" bool, "row" neighbour row,
# "wi" / "wf" weak (literal) int / float
_CT = {"i": "long long", "f": "float", "d": "double", "b": "bool"}
_CONSTS = {"pi": "3.141592653589793", "e": "2.718281828459045"}
_MATH = {"exp", "log", "sqrt", "sin", "cos", "tan", "tanh", "floor", "ceil", "fabs", "log10", "log2"}
_PRELUDE = r"""
__device__ __forceinline__ long long sg_py_floordiv(long long a, long long b)
{
    long long q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}
__device__ __forceinline__ long long sg_py_mod(long long a, long long b)
{
    long long m = a % b;
    if (m != 0 && ((m < 0) != (b < 0))) m += b;
    return m;
}
"""
# emitted only for steps that take a float remainder
_PRELUDE_FMOD = r"""
__device__ __forceinline__ double sg_py_fmod(double a, double b)
{
    double m = fmod(a, b);
    if (m != 0.0 && ((m < 0.0) != (b < 0.0))) m += b;
    return m;
}
__device__ __forceinline__ float sg_py_fmodf(float a, float b)
{
    float m = fmodf(a, b);
    if (m != 0.0f && ((m < 0.0f) != (b < 0.0f))) m += b;
    return m;
}
"""


def find_step_source(step_func, module_fpath=None):
    """(source of the module, function name) for a step function: its module file
    (the path given to register_step_func, as the reference reads it) or, for a plain
    Python function, inspect.getsource. A CuPy-JIT rawkernel object needs no CuPy
    here: only its __name__ and the module path are used."""
    name = getattr(step_func, "__name__", None) or getattr(getattr(step_func, "_func", None), "__name__", None)
    if name is None:
        raise StepTranslationError("step function %r has no __name__" % (step_func,))
    if module_fpath and os.path.isfile(str(module_fpath)):
        with open(module_fpath) as f:
            return f.read(), name
    try:
        return textwrap.dedent(inspect.getsource(step_func)), name
    except (OSError, TypeError) as exc:
        raise StepTranslationError("cannot read the source of %s: %s" % (name, exc))


def _promote(a, b):
    if a == "row" or b == "row":
        raise TypeError("a neighbour row is not a number")
    a = "i" if a == "b" else a
    b = "i" if b == "b" else b
    strong = [t for t in (a, b) if t in ("i", "f", "d")]
    if not strong:
        return "d" if "wf" in (a, b) else "i"
    if len(strong) == 1:
        s, w = strong[0], (b if a == strong[0] else a)
        if s == "i" and w == "wf":
            return "d"
        return s
    if a == b:
        return a
    return "d"  # f with i, f with d, i with d


class _Translator:
    def __init__(self, fn, globals_, props, prop_dtypes, entry, arrays=(), prop_widths=None):
        self.fn = fn
        self.entry = entry
        args = [a.arg for a in fn.args.args]
        ng = len(globals_)
        if len(args) < 2 + ng + 1:
            raise StepTranslationError("%s: expected (tick, agent_index, %d globals, agent_ids, breeds, "
                                       "locations, properties...), got %d parameters"
                                       % (fn.name, ng, len(args)))
        self.tick = args[0]
        self.agent = args[1]
        self.globals = dict(zip(args[2:2 + ng], globals_))
        rest = args[2 + ng:]
        self.agent_ids = rest[0]
        pnames = ["breed", "locations"] + list(props)
        self.props = {}
        self.breeds = self.locations = None
        for a, p in zip(rest[1:], pnames):
            if p == "breed":
                self.breeds = a
            elif p == "locations":
                self.locations = a
            else:
                self.props[a] = p
        # breed-local arrays: (array, index map) parameter pairs after the
        # properties, in registration order (sagesim/model.py:1994-2008)
        self.arrays = {}  # parameter -> (array name, shape per agent)
        self.array_idx = {}  # parameter -> array name
        tail = rest[1 + len(pnames):]
        arrays = list(arrays)
        if len(tail) != 2 * len(arrays):
            raise StepTranslationError("%s: expected %d breed-local array parameters after the properties, got %d"
                                       % (fn.name, 2 * len(arrays), len(tail)))
        for k, (aname, shape) in enumerate(arrays):
            self.arrays[tail[2 * k]] = (aname, tuple(int(d) for d in shape))
            self.array_idx[tail[2 * k + 1]] = aname
        self.prop_dtypes = prop_dtypes
        self.locals = {}  # name -> type
        self.row_of = {}  # row local -> agent expression
        self.widths = dict(prop_widths or {})  # list property -> values per agent
        self.prow_of = {}  # local alias of a list property's row -> (property, agent expression)
        self.writes = set()
        self.need_fmod = False
        self.out = []

    def err(self, node, msg):
        raise StepTranslationError("%s line %d: %s" % (self.fn.name, getattr(node, "lineno", 0), msg))

    # ---- expressions ----------------------------------------------------------------
    def expr(self, n):
        """(C++ text, type) of an expression."""
        if isinstance(n, ast.Constant):
            v = n.value
            if isinstance(v, bool):
                return ("true" if v else "false"), "b"
            if isinstance(v, int):
                return ("%dLL" % v), "wi"
            if isinstance(v, float):
                return repr(v) if "e" in repr(v) or "." in repr(v) else repr(v) + ".0", "wf"
            self.err(n, "unsupported constant %r" % (v,))
        if isinstance(n, ast.Name):
            if n.id == self.tick:
                return "ctx.tick", "i"
            if n.id == self.agent:
                return "sg_agent", "i"
            if n.id in self.globals:
                return "ctx.g[G_%s]" % self.globals[n.id], "d"
            if n.id in ("True", "False"):
                return n.id.lower(), "b"
            if n.id in self.prow_of:
                self.err(n, "a property row is used only as row[k] or len(row)")
            if n.id in self.row_of:
                return self.row_of[n.id], "row"
            if n.id in self.locals:
                return "u_" + n.id, self.locals[n.id]
            self.err(n, "unknown name %r" % n.id)
        if isinstance(n, ast.BinOp):
            return self.binop(n)
        if isinstance(n, ast.UnaryOp):
            s, t = self.expr(n.operand)
            if isinstance(n.op, ast.Not):
                return "(!(%s))" % s, "b"
            if isinstance(n.op, ast.USub):
                return "(-(%s))" % s, ("i" if t == "b" else t)
            if isinstance(n.op, ast.UAdd):
                return s, t
            self.err(n, "unsupported unary operator")
        if isinstance(n, ast.BoolOp):
            op = " && " if isinstance(n.op, ast.And) else " || "
            return "(" + op.join("(%s)" % self.expr(v)[0] for v in n.values) + ")", "b"
        if isinstance(n, ast.Compare):
            parts = []
            left, lt = self.expr(n.left)
            for op, comp in zip(n.ops, n.comparators):
                right, rt = self.expr(comp)
                sym = {ast.Lt: "<", ast.LtE: "<=", ast.Gt: ">", ast.GtE: ">=", ast.Eq: "==",
                       ast.NotEq: "!="}.get(type(op))
                if sym is None:
                    self.err(n, "unsupported comparison")
                parts.append("((%s) %s (%s))" % (left, sym, right))
                left = right
            return "(" + " && ".join(parts) + ")", "b"
        if isinstance(n, ast.IfExp):
            c, _ = self.expr(n.test)
            a, at = self.expr(n.body)
            b, bt = self.expr(n.orelse)
            t = _promote(at, bt)
            t = "i" if t == "wi" else ("d" if t == "wf" else t)
            return "((%s) ? (%s)(%s) : (%s)(%s))" % (c, _CT[t], a, _CT[t], b), t
        if isinstance(n, ast.Attribute) and isinstance(n.value, ast.Name) and \
                n.value.id in ("math", "cp", "np", "numpy", "cupy") and n.attr in _CONSTS:
            return _CONSTS[n.attr], "wf"  # a Python float: weak in numpy's promotion
        if isinstance(n, ast.Subscript):
            return self.subscript(n)
        if isinstance(n, ast.Call):
            return self.call(n)
        self.err(n, "unsupported expression %s" % type(n).__name__)

    def binop(self, n):
        a, at = self.expr(n.left)
        b, bt = self.expr(n.right)
        op = n.op
        if isinstance(op, ast.Div):
            t = _promote(at, bt)
            t = "d" if t in ("i", "wi", "wf") else t
            return "((%s)(%s) / (%s)(%s))" % (_CT[t], a, _CT[t], b), t
        t = _promote(at, bt)
        if isinstance(op, (ast.FloorDiv, ast.Mod)):
            if t in ("i", "wi"):
                f = "sg_py_floordiv" if isinstance(op, ast.FloorDiv) else "sg_py_mod"
                return "%s((long long)(%s), (long long)(%s))" % (f, a, b), "i"
            if isinstance(op, ast.FloorDiv):
                t = "d" if t == "wf" else t
                return "floor((%s)(%s) / (%s)(%s))" % (_CT[t], a, _CT[t], b), t
            # Python / numpy float remainder: the sign of the divisor
            t = "d" if t == "wf" else t
            self.need_fmod = True
            f = "sg_py_fmodf" if t == "f" else "sg_py_fmod"
            return "%s((%s)(%s), (%s)(%s))" % (f, _CT[t], a, _CT[t], b), t
        if isinstance(op, ast.Pow):
            e = n.right
            if (t in ("i", "wi") and isinstance(e, ast.Constant) and isinstance(e.value, int)
                    and not isinstance(e.value, bool) and 0 <= e.value <= 8):
                # Python int ** small int literal: an exact integer product
                return "(" + " * ".join(["(long long)(%s)" % a] * e.value or ["1LL"]) + ")", "i"
            return "pow((double)(%s), (double)(%s))" % (a, b), "d"
        sym = {ast.Add: "+", ast.Sub: "-", ast.Mult: "*", ast.BitAnd: "&", ast.BitOr: "|",
               ast.BitXor: "^", ast.LShift: "<<", ast.RShift: ">>"}.get(type(op))
        if sym is None:
            self.err(n, "unsupported operator %s" % type(op).__name__)
        if t in ("wi", "wf"):
            return "((%s) %s (%s))" % (a, sym, b), t
        return "((%s)(%s) %s (%s)(%s))" % (_CT[t], a, sym, _CT[t], b), t

    def prop_read(self, node, pname, agent, comp=None):
        dt = self.prop_dtypes[pname]
        fn = "i32" if dt == "i" else "f32"
        if comp is None:
            return "ctx.%s(PROP_%s, (int)(%s))" % (fn, pname, agent), ("i" if dt == "i" else "f")
        return "ctx.%s(PROP_%s, (int)(%s), (int)(%s))" % (fn, pname, agent, comp), ("i" if dt == "i" else "f")

    def array_element(self, n):
        """(array name, row C++, column C++) when n is a full element of a
        breed-local array (a[r][j], a[r, j], a[r][j][k], a[r, j, k]), else None."""
        subs = []
        b = n
        while isinstance(b, ast.Subscript):
            sl = b.slice
            subs[:0] = list(sl.elts) if isinstance(sl, ast.Tuple) else [sl]
            b = b.value
        if not (isinstance(b, ast.Name) and b.id in self.arrays):
            return None
        aname, shape = self.arrays[b.id]
        if len(subs) != 1 + len(shape):
            self.err(n, "breed-local array %r needs %d indices" % (aname, 1 + len(shape)))
        row, _ = self.expr(subs[0])
        col = "0LL"
        for d, sub in zip(shape, subs[1:]):
            c, _ = self.expr(sub)
            col = "(%s) * %dLL + (long long)(%s)" % (col, d, c)
        return aname, row, col

    def subscript(self, n):
        el = self.array_element(n)
        if el is not None:
            aname, row, col = el
            return "ctx.arr_f32(PROP_sgbla_%s, (long long)(%s), %s)" % (aname, row, col), "f"
        base, idx = n.value, n.slice
        if isinstance(base, ast.Name) and base.id in self.array_idx:
            a, _ = self.expr(idx)
            return "(long long)ctx.i32(PROP_sgbla_%s_idx, (int)(%s))" % (self.array_idx[base.id], a), "i"
        # p[a][c]
        if isinstance(base, ast.Subscript) and isinstance(base.value, ast.Name) and base.value.id in self.props:
            a, _ = self.expr(base.slice)
            c, _ = self.expr(idx)
            return self.prop_read(n, self.props[base.value.id], a, c)
        if isinstance(base, ast.Name):
            if base.id in self.props:
                if isinstance(idx, ast.Tuple) and len(idx.elts) == 2:
                    a, _ = self.expr(idx.elts[0])
                    c, _ = self.expr(idx.elts[1])
                    return self.prop_read(n, self.props[base.id], a, c)
                a, _ = self.expr(idx)
                return self.prop_read(n, self.props[base.id], a)
            if base.id == self.locations:
                a, _ = self.expr(idx)
                return a, "row"
            if base.id in self.globals:
                k, _ = self.expr(idx)
                return "ctx.g[G_%s + (int)(%s)]" % (self.globals[base.id], k), "d"
            if base.id in self.prow_of:
                pname, a = self.prow_of[base.id]
                c, _ = self.expr(idx)
                return self.prop_read(n, pname, a, c)
            if base.id in self.row_of:
                k, _ = self.expr(idx)
                return "(long long)ctx.neighbor((int)(%s), (int)(%s))" % (self.row_of[base.id], k), "i"
        if isinstance(base, ast.Subscript) and isinstance(base.value, ast.Name) and base.value.id == self.locations:
            a, _ = self.expr(base.slice)
            k, _ = self.expr(idx)
            return "(long long)ctx.neighbor((int)(%s), (int)(%s))" % (a, k), "i"
        self.err(n, "unsupported subscript")

    def call(self, n):
        f = n.func
        name = f.id if isinstance(f, ast.Name) else (f.attr if isinstance(f, ast.Attribute) else None)
        mod = f.value.id if isinstance(f, ast.Attribute) and isinstance(f.value, ast.Name) else None
        args = n.args
        # sagesim/utils.py device helpers
        if name == "get_this_agent_data_from_tensor" and len(args) == 2:
            sub = ast.Subscript(value=args[1], slice=args[0], ctx=ast.Load())
            ast.copy_location(sub, n)
            return self.subscript(sub)
        if name == "get_num_neighbors" and len(args) == 2:
            a, _ = self.expr(args[0])
            return "(long long)ctx.degree((int)(%s))" % a, "i"
        if name == "get_neighbor" and len(args) == 4:
            a, _ = self.expr(args[0])
            k, _ = self.expr(args[1])
            return "(long long)ctx.neighbor((int)(%s), (int)(%s))" % (a, k), "i"
        if name in ("rand_uniform_philox", "rand_normal"):
            if len(args) != 3:
                self.err(n, "%s takes (tick, agent, salt)" % name)
            if not (isinstance(args[0], ast.Name) and args[0].id == self.tick):
                self.err(n, "%s must be drawn at the current tick" % name)
            a, _ = self.expr(args[1])
            s, _ = self.expr(args[2])
            m = "rand_uniform" if name == "rand_uniform_philox" else "rand_normal"
            return "ctx.%s((int)(%s), (long long)(%s))" % (m, a, s), "d"
        if name == "len" and mod is None:
            if len(args) == 1:
                a0 = args[0]
                if isinstance(a0, ast.Name) and a0.id in self.prow_of:
                    return "(long long)ctx.width(PROP_%s)" % self.prow_of[a0.id][0], "i"
                if self._list_prop_row(a0):
                    return "(long long)ctx.width(PROP_%s)" % self.props[a0.value.id], "i"
                r, t = self.expr(a0)
                if t == "row":
                    return "(long long)ctx.degree((int)(%s))" % r, "i"
            self.err(n, "len() of a neighbour row or a list property's row only")
        if name == "isnan":
            a0 = args[0]
            if isinstance(a0, ast.Subscript) and self._is_row_element(a0):
                return "false", "b"  # CSR rows hold no padding
            s, _ = self.expr(a0)
            return "isnan((double)(%s))" % s, "b"
        if name in ("int", "int32", "int64") and (mod in (None, "cp", "np", "numpy", "cupy")):
            s, _ = self.expr(args[0])
            return "(long long)(%s)" % s, "i"
        if name in ("float", "float64") and (mod in (None, "cp", "np", "numpy", "cupy")):
            s, _ = self.expr(args[0])
            return "(double)(%s)" % s, "d"
        if name == "float32" and mod in ("cp", "np", "numpy", "cupy"):
            s, _ = self.expr(args[0])
            return "(float)(%s)" % s, "f"
        if name == "bool" and mod is None:
            s, _ = self.expr(args[0])
            return "((bool)(%s))" % s, "b"
        if name == "abs" and mod is None or name == "fabs":
            s, t = self.expr(args[0])
            if t in ("f",):
                return "fabsf(%s)" % s, "f"
            if t in ("i", "wi", "b"):
                return "llabs((long long)(%s))" % s, "i"
            return "fabs((double)(%s))" % s, "d"
        if name in ("min", "max") and mod is None:
            if len(args) < 2:
                self.err(n, "min/max of two or more values only")
            a, at = self.expr(args[0])
            op = "<" if name == "min" else ">"
            for arg in args[1:]:  # left to right, as Python folds them
                b, bt = self.expr(arg)
                t = _promote(at, bt)
                t = "i" if t == "wi" else ("d" if t == "wf" else t)
                a, at = "((%s)(%s) %s (%s)(%s) ? (%s)(%s) : (%s)(%s))" % (
                    _CT[t], a, op, _CT[t], b, _CT[t], a, _CT[t], b), t
            return a, at
        if name in _MATH and mod in ("math", "cp", "np", "numpy", "cupy"):
            s, t = self.expr(args[0])
            if t == "f" and mod != "math":
                return "%sf(%s)" % (name, s), "f"
            return "%s((double)(%s))" % (name, s), "d"
        self.err(n, "unsupported call %s" % (ast.unparse(f) if hasattr(ast, "unparse") else name))

    @staticmethod
    def _helper_name(call):
        f = call.func
        return f.id if isinstance(f, ast.Name) else (f.attr if isinstance(f, ast.Attribute) else None)

    def _list_prop_row(self, n):
        """Whether n is p[a] for a list property p (one agent's row)."""
        return (isinstance(n, ast.Subscript) and isinstance(n.value, ast.Name) and n.value.id in self.props
                and self.widths.get(self.props[n.value.id], 1) > 1 and not isinstance(n.slice, ast.Tuple))

    def _is_row_element(self, n):
        b = n.value
        if isinstance(b, ast.Name) and b.id in self.row_of:
            return True
        return isinstance(b, ast.Subscript) and isinstance(b.value, ast.Name) and b.value.id == self.locations

    # ---- statements ------------------------------------------------------------------
    def declare(self, name, t, node):
        t = "i" if t == "wi" else ("d" if t == "wf" else t)
        if (name in (self.tick, self.agent) or name in self.globals or name in self.props
                or name in self.arrays or name in self.array_idx):
            self.err(node, "cannot assign to parameter %r" % name)
        old = self.locals.get(name)
        if old is None:
            self.locals[name] = t
        elif old != t and "row" not in (old, t):
            # numpy rebinding: keep the wider type for the C++ declaration
            self.locals[name] = "d" if "d" in (old, t) else ("f" if "f" in (old, t) else old)

    def scan(self, body):
        """First pass: local variable types (assignments in program order)."""
        for s in body:
            for node in ast.walk(s):
                if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
                    name = node.targets[0].id
                    v = node.value
                    if isinstance(v, ast.Subscript) and isinstance(v.value, ast.Name) and v.value.id == self.locations:
                        self.locals[name] = "row"
                        self.row_of[name] = self.expr(v.slice)[0]
                        continue
                    if self._list_prop_row(v):
                        # alias of one agent's row of a list property (read through row[k])
                        self.locals[name] = "row"
                        self.prow_of[name] = (self.props[v.value.id], self.expr(v.slice)[0])
                        continue
                    try:
                        _, t = self.expr(v)
                    except StepTranslationError:
                        continue  # depends on a local not typed yet; second pass below
                    self.declare(name, t, node)
                elif isinstance(node, ast.For) and isinstance(node.target, ast.Name):
                    self.declare(node.target.id, "i", node)
        # second pass for assignments that referenced later-typed locals
        for s in body:
            for node in ast.walk(s):
                if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
                    name = node.targets[0].id
                    if name not in self.locals:
                        _, t = self.expr(node.value)
                        self.declare(name, t, node)

    def emit(self, line, depth):
        self.out.append("    " * depth + line)

    def block(self, body, depth):
        for s in body:
            self.stmt(s, depth)

    def stmt(self, s, d):
        if isinstance(s, ast.Expr):
            if isinstance(s.value, ast.Constant) and isinstance(s.value.value, str):
                return  # docstring
            v = s.value
            if (isinstance(v, ast.Call) and self._helper_name(v) == "set_this_agent_data_from_tensor"
                    and len(v.args) == 3):
                # sagesim/utils.py: set_this_agent_data_from_tensor(a, p, x) is p[a] = x
                tgt = ast.Subscript(value=v.args[1], slice=v.args[0], ctx=ast.Store())
                ast.copy_location(tgt, s)
                return self.assign(tgt, v.args[2], d, s)
            self.err(s, "expression statements are not supported")
        if isinstance(s, ast.Pass):
            return
        if isinstance(s, ast.Assign):
            if len(s.targets) != 1:
                self.err(s, "one assignment target only")
            return self.assign(s.targets[0], s.value, d, s)
        if isinstance(s, ast.AugAssign):
            tgt = s.target
            val = ast.BinOp(left=_load(tgt), op=s.op, right=s.value)
            ast.copy_location(val, s)
            return self.assign(tgt, val, d, s)
        if isinstance(s, ast.If):
            c, _ = self.expr(s.test)
            self.emit("if (%s) {" % c, d)
            self.block(s.body, d + 1)
            if s.orelse:
                self.emit("} else {", d)
                self.block(s.orelse, d + 1)
            self.emit("}", d)
            return
        if isinstance(s, ast.While):
            if s.orelse:
                self.err(s, "while ... else is not supported")
            c, _ = self.expr(s.test)
            self.emit("while (%s) {" % c, d)
            self.block(s.body, d + 1)
            self.emit("}", d)
            return
        if isinstance(s, ast.For):
            it = s.iter
            if not (isinstance(it, ast.Call) and isinstance(it.func, ast.Name) and it.func.id == "range"
                    and isinstance(s.target, ast.Name) and not s.orelse):
                self.err(s, "for loops over range() only")
            a = [self.expr(x)[0] for x in it.args]
            lo, hi, st = ("0LL", a[0], "1LL") if len(a) == 1 else (a[0], a[1], a[2] if len(a) == 3 else "1LL")
            v = "u_" + s.target.id
            self.emit("for (%s = (long long)(%s); ((long long)(%s) > 0) ? (%s < (long long)(%s)) : "
                      "(%s > (long long)(%s)); %s += (long long)(%s)) {" % (v, lo, st, v, hi, v, hi, v, st), d)
            self.block(s.body, d + 1)
            self.emit("}", d)
            return
        if isinstance(s, ast.Break):
            return self.emit("break;", d)
        if isinstance(s, ast.Continue):
            return self.emit("continue;", d)
        if isinstance(s, ast.Return):
            if s.value is not None:
                self.err(s, "a step returns nothing")
            return self.emit("return;", d)
        self.err(s, "unsupported statement %s" % type(s).__name__)

    def assign(self, tgt, value, d, node):
        if isinstance(tgt, ast.Name):
            if self.locals.get(tgt.id) == "row":
                return  # declared as a row alias; nothing to emit
            v, _ = self.expr(value)
            t = self.locals[tgt.id]
            return self.emit("u_%s = (%s)(%s);" % (tgt.id, _CT[t], v), d)
        if isinstance(tgt, ast.Subscript):
            el = self.array_element(tgt)
            if el is not None:
                aname, row, col = el
                v, _ = self.expr(value)
                self.writes.add("sgbla_" + aname)
                return self.emit("ctx.set_arr_f32(PROP_sgbla_%s, (long long)(%s), (float)(%s), %s);"
                                 % (aname, row, v, col), d)
            base, idx = tgt.value, tgt.slice
            if isinstance(base, ast.Name) and base.id in self.prow_of:
                self.err(node, "write a list property through the property (p[a][k] = v), not a row alias")
            comp = None
            if isinstance(base, ast.Subscript) and isinstance(base.value, ast.Name) and base.value.id in self.props:
                pname = self.props[base.value.id]
                agent, _ = self.expr(base.slice)
                comp, _ = self.expr(idx)
            elif isinstance(base, ast.Name) and base.id in self.props:
                pname = self.props[base.id]
                if isinstance(idx, ast.Tuple) and len(idx.elts) == 2:
                    agent, _ = self.expr(idx.elts[0])
                    comp, _ = self.expr(idx.elts[1])
                else:
                    agent, _ = self.expr(idx)
            else:
                self.err(node, "assignment to a subscript of a property only")
            v, _ = self.expr(value)
            self.writes.add(pname)
            fn = "set_i32" if self.prop_dtypes[pname] == "i" else "set_f32"
            cast = "int" if self.prop_dtypes[pname] == "i" else "float"
            if comp is None:
                return self.emit("ctx.%s(PROP_%s, (int)(%s), (%s)(%s));" % (fn, pname, agent, cast, v), d)
            return self.emit("ctx.%s(PROP_%s, (int)(%s), (%s)(%s), (int)(%s));" % (fn, pname, agent, cast, v, comp), d)
        self.err(node, "unsupported assignment target")

    def run(self):
        self.scan(self.fn.body)
        decls = ["    %s u_%s = 0;" % (_CT[t], name) for name, t in self.locals.items() if t != "row"]
        self.block(self.fn.body, 1)
        prelude = _PRELUDE + (_PRELUDE_FMOD if self.need_fmod else "")
        src = [prelude, "__device__ void %s(const sg_ctx &ctx, int sg_agent)" % self.entry, "{"]
        src += decls
        src += self.out
        src.append("}")
        return "\n".join(src)


def _load(t):
    n = ast.parse(ast.unparse(t), mode="eval").body if hasattr(ast, "unparse") else t
    return n


def translate_step(source, name, globals_, props, prop_dtypes, entry=None, arrays=(), prop_widths=None):
    """CUDA C++ for step `name` defined in `source`.

    globals_: the model's global property names in registration order.
    props: the model's agent property names in property order (without the
    breed and the neighbour rows). prop_dtypes: name -> "i" (int32) or "f"
    (float32). arrays: the model's breed-local arrays in registration order as
    (name, shape per agent); each is read and written as the float32 engine
    array PROP_sgbla_<name> (row-major, one row per agent of its breed) with the
    int32 index map PROP_sgbla_<name>_idx. prop_widths: name -> values per
    agent of list properties (a local bound to p[a] of such a property is an
    alias of that row: row[k], len(row)). Returns (C++ source, entry name,
    properties and arrays written, the arrays as sgbla_<name>)."""
    tree = ast.parse(source)
    fn = None
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == name:
            fn = node
            break
    if fn is None:
        raise StepTranslationError("no function %r in the step's source" % name)
    entry = entry or ("sg_py_" + name)
    tr = _Translator(fn, list(globals_), list(props), dict(prop_dtypes), entry, arrays, prop_widths)
    return tr.run(), entry, sorted(tr.writes)
