"""The identity of the code that produces a solved field, for the field-cache
keys (drop-in for ion_gym physics/solve_code.py:36-51, 116-122).

The reference hashes its Python solver modules into every field-cache key,
so that any change to the solve path re-solves each cached geometry once.
Here the solve path is mostly CUDA: solve_code_key() hashes

  * the CUDA sources and headers of libigsolve.so (csrc/*.cu, *.cuh, *.h)
    and the C-ABI header include/igsolve.h, with C and C++ comments removed
    (a comment edit changes nothing; any code change does);
  * the Python drop-ins on the solve path (solvers, the mixed session, the
    mask providers, the C-ABI binding), as docstring-free syntax trees;
  * the precision the basis door runs in ("fp64": the reference's V-cycle
    bits; "mixed": the batched FP32-multigrid / FP64-refinement session)
    and, for "mixed", its cycle parameters.

A listed source that no longer exists raises, so a rename cannot drop code
from the key unnoticed.  In the reference, build_stl3d.py:753-754 and
io/basis_cache.py:200-201 call solve_code_key(); pointing them at this
module (the same name) keys the cache on this library.
"""
import ast
import hashlib
import os
from functools import lru_cache

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)

# Python modules on the solve path (relative to the package)
SOLVE_MODULES = (
    "_lib.py", "physics/solver3d.py", "physics/multigrid3d.py",
    "physics/mixed.py", "physics/_device.py", "physics/rasterize3d.py",
    "physics/shapes3d.py", "physics/scene3d.py",
)
# native sources (relative to the repository root); the csrc folder is
# listed whole, so a new translation unit joins the key by itself
NATIVE_DIRS = ("ion_gym_gb300/csrc",)
NATIVE_FILES = ("include/igsolve.h",)
NATIVE_SUFFIXES = (".cu", ".cuh", ".h", ".cc", ".cpp")


def strip_c_comments(src):
    """C/C++/CUDA source without its // and /* */ comments (string and
    character literals kept), whitespace runs collapsed, so that comment
    and layout edits do not change the key."""
    out = []
    i, n = 0, len(src)
    while i < n:
        c = src[i]
        if c in "\"'":
            j = i + 1
            while j < n and src[j] != c:
                j += 2 if src[j] == "\\" else 1
            out.append(src[i:j + 1])
            i = j + 1
        elif src.startswith("//", i):
            j = src.find("\n", i)
            i = n if j < 0 else j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            i = n if j < 0 else j + 2
            out.append(" ")
        else:
            out.append(c)
            i += 1
    return " ".join("".join(out).split())


def python_code_part(src):
    """A Python module as a syntax-tree dump without docstrings."""
    tree = ast.parse(src)
    for node in ast.walk(tree):
        body = getattr(node, "body", None)
        if (isinstance(node, (ast.Module, ast.ClassDef, ast.FunctionDef,
                              ast.AsyncFunctionDef)) and body
                and isinstance(body[0], ast.Expr)
                and isinstance(body[0].value, ast.Constant)
                and isinstance(body[0].value.value, str)):
            node.body = body[1:] or [ast.Pass()]
    return ast.dump(tree, include_attributes=False)


def key_of_sources(native, python, precision="fp64", cycle=None):
    """16 hex digits over {path: C/CUDA source}, {path: Python source}, the
    precision and (mixed only) the cycle parameters."""
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"unknown basis precision {precision!r}")
    h = hashlib.sha256()
    for kind, table, part in (("native", native, strip_c_comments),
                              ("python", python, python_code_part)):
        for path in sorted(table):
            h.update(f"{kind}|{path}|".encode())
            h.update(part(table[path]).encode())
    h.update(f"precision|{precision}".encode())
    if precision == "mixed":
        h.update(repr(sorted((cycle or {}).items())).encode())
    return h.hexdigest()[:16]


def _read(path):
    with open(path, encoding="utf-8") as f:
        return f.read()


def solve_sources():
    """({native path: source}, {python path: source}) of this installation;
    raises LookupError when a listed source is missing."""
    native, python = {}, {}
    missing = []
    for d in NATIVE_DIRS:
        full = os.path.join(ROOT, d)
        if not os.path.isdir(full):
            missing.append(d)
            continue
        for f in sorted(os.listdir(full)):
            if f.endswith(NATIVE_SUFFIXES):
                native[f"{d}/{f}"] = _read(os.path.join(full, f))
    for f in NATIVE_FILES:
        p = os.path.join(ROOT, f)
        if os.path.exists(p):
            native[f] = _read(p)
        else:
            missing.append(f)
    for f in SOLVE_MODULES:
        p = os.path.join(PKG, f)
        if os.path.exists(p):
            python[f"ion_gym_gb300/{f}"] = _read(p)
        else:
            missing.append(f)
    if missing:
        raise LookupError(
            f"solve_code: listed solve-path sources are missing: {missing}; "
            f"update the lists so the field-cache key covers the solve path")
    return native, python


@lru_cache(maxsize=4)
def _key(precision, cycle_items):
    native, python = solve_sources()
    return key_of_sources(native, python, precision, dict(cycle_items))


def solve_code_key(precision=None):
    """The key of the solve-path code of this installation for the basis
    door's precision (None: the door's default, multigrid3d.BASIS_PRECISION)."""
    from ion_gym_gb300.physics import multigrid3d
    from ion_gym_gb300.physics.mixed import CYCLE_SINGLE, CYCLE_BATCH, BATCH_MIN
    p = multigrid3d.basis_precision(precision)
    cyc = ()
    if p == "mixed":
        cyc = tuple(sorted({**{f"single_{k}": v for k, v in CYCLE_SINGLE.items()},
                            **{f"batch_{k}": v for k, v in CYCLE_BATCH.items()},
                            "batch_min": BATCH_MIN}.items()))
    return _key(p, cyc)
