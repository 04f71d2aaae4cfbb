"""Pure-Python stand-in for numba, used ONLY by make_golden.py to run the
reference ion_gym solver unmodified in a container where numba is absent.

``njit`` does not compile anything.  It re-executes the decorated function's
own source with numba's literal typing restored: every float literal is a
float64 and every int literal an int64 (numba types ``1.0`` and ``1`` that
way, so ``1.0 / th_f32`` and ``1 / th_f32`` are float64 divisions).  Under
NumPy 2 scalar promotion (NEP 50) a bare Python number is "weak" and
``1.0 / np.float32(x)`` would round to float32 instead, which is not what the
compiled reference computes.  Wrapping each literal in ``np.float64`` /
``np.int64`` makes the interpreted arithmetic follow the compiled typing:
float32 op float32 stays float32, anything with a float64 or int64 operand is
float64.

Arguments are typed the same way: numba types a Python ``float`` argument
as float64 and a Python ``int`` as int64, so the wrapper passes them on as
``np.float64`` / ``np.int64`` (``(a_f32 - b_f32) / h`` with ``h`` a Python
float divides in float64 when compiled).

``prange`` is ``range``: within one red-black colour the updates are
independent and the row maxima are order-free, so serial execution gives the
same bits as numba's parallel execution.
"""
import ast
import inspect
import textwrap

import numpy as np

__version__ = "0.0-stub"


class _F64Literals(ast.NodeTransformer):
    """numba types a float literal as float64 and an int literal as int64;
    under NEP 50 both would be "weak" and take the other operand's type
    (``1 / th_f32`` would be a float32 division instead of float64)."""

    def visit_Constant(self, node):
        v = node.value
        if isinstance(v, bool) or not isinstance(v, (int, float)):
            return node
        name = "__stub_f64" if isinstance(v, float) else "__stub_i64"
        call = ast.Call(func=ast.Name(id=name, ctx=ast.Load()),
                        args=[ast.Constant(v)], keywords=[])
        return ast.copy_location(call, node)


def _interpret(fn):
    src = textwrap.dedent(inspect.getsource(fn))
    tree = ast.parse(src)
    fdef = tree.body[0]
    fdef.decorator_list = []
    tree = ast.fix_missing_locations(_F64Literals().visit(tree))
    # keep original line numbers for tracebacks
    ast.increment_lineno(tree, fn.__code__.co_firstlineno - 1)
    code = compile(tree, inspect.getsourcefile(fn), "exec")
    g = fn.__globals__
    g["__stub_f64"] = np.float64
    g["__stub_i64"] = np.int64
    ns = {}
    exec(code, g, ns)
    inner = ns[fn.__name__]

    def _arg(v):
        if isinstance(v, (bool, np.generic, np.ndarray)):
            return v
        if isinstance(v, float):
            return np.float64(v)
        if isinstance(v, int):
            return np.int64(v)
        return v

    def out(*args, **kwargs):
        return inner(*[_arg(v) for v in args],
                     **{k: _arg(v) for k, v in kwargs.items()})
    out.__name__ = fn.__name__
    out.__wrapped_source__ = src
    out.__interpreted__ = inner
    return out


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return _interpret(args[0])

    def deco(fn):
        return _interpret(fn)
    return deco


jit = njit
prange = range
