"""Quadrature tables shared by the library and the oracle (CPU)."""
import math

import numpy as np
import pytest

import oracle
from beastgpu_gb300.csrc import gen_trirules


def _table():
    import re
    txt = open(gen_trirules.__file__.replace("gen_trirules.py", "trirules.h")).read()
    rows = re.findall(r"\{([-0-9.e]+), ([-0-9.e]+), ([-0-9.e]+)\}", txt)
    return np.array(rows, dtype=float)


@pytest.mark.parametrize("npts,degree,offset", [(1, 1, 0), (3, 2, 1), (4, 3, 4), (6, 4, 8), (7, 5, 14),
                                                (12, 6, 21), (13, 7, 33)])
def test_triangle_rule_exact_to_degree(npts, degree, offset):
    t = _table()[offset:offset + npts]
    assert np.isclose(t[:, 2].sum(), 1.0, atol=1e-15)
    for i in range(degree + 1):
        for j in range(degree + 1 - i):
            exact = 2 * math.factorial(i) * math.factorial(j) / math.factorial(i + j + 2)
            got = np.sum(t[:, 2] * t[:, 0] ** i * t[:, 1] ** j)
            assert abs(got - exact) < 2e-16 * 8, (i, j, got, exact)
    # points inside the triangle
    assert np.all(t[:, 0] > 0) and np.all(t[:, 1] > 0) and np.all(t[:, 0] + t[:, 1] < 1)


def test_library_and_oracle_tables_identical():
    a = open(gen_trirules.__file__.replace("gen_trirules.py", "trirules.h")).read()
    b = open(oracle.__file__.replace("__init__.py", "trirules.h")).read()
    norm = lambda s: s.replace("bgb_", "X").replace("BGB_", "X").replace("orc_", "X").replace("ORC_", "X")  # noqa
    assert norm(a) == norm(b)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 10, 16])
def test_gauss_legendre01(n):
    x, w = oracle.gauss_legendre01(n)
    t, v = np.polynomial.legendre.leggauss(n)
    np.testing.assert_allclose(x, (t + 1) / 2, rtol=0, atol=2e-16)
    np.testing.assert_allclose(w, v / 2, rtol=0, atol=1e-15)
    for k in range(2 * n):
        assert abs(np.sum(w * x ** k) - 1.0 / (k + 1)) < 1e-14
