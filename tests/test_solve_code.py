"""The field-cache key of the solve-path code (solve_code.solve_code_key,
the reference's physics/solve_code.py:36-51, 116-122): a code change in a
CUDA source or a Python drop-in changes it, a comment or docstring edit
does not, and the basis door's precision is part of it.  The basis door's
precision switch refuses unknown values and the mixed form refuses theta
before any GPU work."""
import numpy as np
import pytest

from ion_gym_gb300 import solve_code as SC

CU = """// kernel
__global__ void k(float* a) { a[threadIdx.x] *= 2.f; /* twice */ }
"""
PY = '''"""module doc"""
def f(x):
    """doc"""
    return x + 1
'''


def test_key_follows_code_not_comments():
    base = SC.key_of_sources({"a.cu": CU}, {"m.py": PY})
    assert len(base) == 16 and int(base, 16) >= 0
    # comments, docstrings and layout do not count
    cu2 = CU.replace("// kernel", "// the kernel, renamed comment").replace(
        "/* twice */", "")
    py2 = PY.replace('"""doc"""', '"""another doc"""')
    assert SC.key_of_sources({"a.cu": cu2}, {"m.py": py2}) == base
    assert SC.key_of_sources({"a.cu": CU.replace("{ a", "{\n   a")},
                             {"m.py": PY}) == base
    # code does, and so does a string literal inside it
    assert SC.key_of_sources({"a.cu": CU.replace("2.f", "3.f")},
                             {"m.py": PY}) != base
    assert SC.key_of_sources({"a.cu": CU}, {"m.py": PY.replace("+ 1", "+ 2")}) != base
    assert SC.key_of_sources({"a.cu": 'char* s = "//";'}, {}) != \
        SC.key_of_sources({"a.cu": 'char* s = "";'}, {})
    # a file added or renamed counts
    assert SC.key_of_sources({"b.cu": CU}, {"m.py": PY}) != base
    # the precision and the mixed cycle are part of the key
    mixed = SC.key_of_sources({"a.cu": CU}, {"m.py": PY}, "mixed", {"nu1": 2})
    assert mixed != base
    assert SC.key_of_sources({"a.cu": CU}, {"m.py": PY}, "mixed",
                             {"nu1": 3}) != mixed
    with pytest.raises(ValueError):
        SC.key_of_sources({}, {}, "fp32")


def test_installation_key_covers_the_cuda_sources():
    native, python = SC.solve_sources()
    assert any(p.endswith("ig_f64.cu") for p in native)
    assert any(p.endswith("ig_mixed.cu") for p in native)
    assert "include/igsolve.h" in native
    assert any(p.endswith("multigrid3d.py") for p in python)
    k64, kmx = SC.solve_code_key("fp64"), SC.solve_code_key("mixed")
    assert k64 != kmx and len(k64) == len(kmx) == 16
    assert SC.solve_code_key() == k64          # the door's default precision


def test_precision_switch_refuses_before_gpu_work():
    from ion_gym_gb300.physics import multigrid3d as M
    masks = {1: np.zeros((9, 9, 9), bool), 2: np.zeros((9, 9, 9), bool)}
    masks[1][0] = True
    masks[2][-1] = True
    with pytest.raises(ValueError, match="known precisions"):
        M.solve_bases_mg(masks, precision="fp32")
    th = np.ones((6, 9, 9, 9), np.float32)
    with pytest.raises(ValueError, match="theta None"):
        M.solve_bases_mg(masks, theta=th, precision="mixed")
    with pytest.raises(ValueError, match="known stencils"):
        M.solve_bases_mg(masks, stencil="node", precision="mixed")
