"""Host tiling of the far kernel (no GPU): the order in which tiles take the functions is a
permutation of the requested range, deterministic, and its tiles stage fewer triangles than
tiles cut from index order or from a Morton order of the functions' first triangles (the
tiling only decides which tile computes an entry, never its value)."""
import numpy as np
import pytest

import beastgpu_gb300 as bg
from beastgpu_gb300 import _lib
from beastgpu_gb300.api import tile_order


def _supports(X):
    t, loc = np.nonzero(X.fn_index >= 0)
    f = X.fn_index[t, loc]
    sup = [[] for _ in range(X.nfun)]
    for ti, fi in zip(t.tolist(), f.tolist()):
        sup[fi].append(ti)
    return sup


def _slots(sup, order, width):
    return sum(len({t for f in order[b:b + width] for t in sup[f]}) for b in range(0, len(order), width))


def _morton_first(X, sup):
    c = X.mesh.vertices[X.mesh.triangles].mean(axis=1)
    q = np.minimum((c - c.min(0)) / np.ptp(c, axis=0).max() * 1023, 1023).astype(np.int64)
    code = np.zeros(len(c), np.int64)
    for bit in range(10):
        for k in range(3):
            code |= ((q[:, k] >> bit) & 1) << (3 * bit + k)
    rank = np.empty(len(c), np.int64)
    rank[np.argsort(code, kind="stable")] = np.arange(len(c))
    first = np.array([rank[s].min() for s in sup])
    return np.lexsort((np.arange(X.nfun), first))


@pytest.fixture(scope="module")
def spaces():
    plates = bg.two_plates(24, jitter=0.3, seed=1, gap=0.01)
    return {"rwg_sphere": bg.raviartthomas(bg.icosphere(3)), "rwg_plates": bg.raviartthomas(plates),
            "hats_plates": bg.lagrangec0d1(plates)}


@pytest.mark.parametrize("name", ["rwg_sphere", "rwg_plates", "hats_plates"])
@pytest.mark.parametrize("width", [24, 32, 64])
def test_tile_order_is_a_compact_permutation(spaces, name, width):
    X = spaces[name]
    sup = _supports(X)
    order, slots = tile_order(X, width)
    assert sorted(order.tolist()) == list(range(X.nfun))
    assert slots == _slots(sup, order.tolist(), width)
    again, slots2 = tile_order(X, width)
    assert np.array_equal(order, again) and slots == slots2
    # fewer staged triangles than index-order tiles and than Morton-order tiles
    assert slots < _slots(sup, list(range(X.nfun)), width)
    assert slots < _slots(sup, _morton_first(X, sup).tolist(), width)
    # each tile is one leaf of the bisection: its functions in index order
    for b in range(0, X.nfun, width):
        tile = order[b:b + width]
        assert np.all(np.diff(tile) > 0)


def test_tile_order_of_a_function_range_and_unsupported_functions(spaces):
    X = spaces["rwg_sphere"]
    order, _ = tile_order(X, 32, functions=(100, 917))
    assert sorted(order.tolist()) == list(range(100, 917))
    # three functions without supports (indices past the used ones) come last, in index order
    Y = bg.Space(X.mesh, X.refspace, X.fn_index, X.fn_coef, X.nfun + 3)
    order, _ = tile_order(Y, 64)
    assert order[-3:].tolist() == [X.nfun, X.nfun + 1, X.nfun + 2]
    assert sorted(order.tolist()) == list(range(Y.nfun))


def test_tile_order_rejects_bad_arguments(spaces):
    X = spaces["rwg_sphere"]
    with pytest.raises(_lib.BGBError, match="range"):
        tile_order(X, 64, functions=(10, X.nfun + 1))
    with pytest.raises(_lib.BGBError, match="invalid"):
        tile_order(X, 0)


def _with(X, vertices=None, triangles=None, fn_index=None, fn_coef=None, nfun=None, refspace=None):
    m = X.mesh
    mesh = bg.Mesh(m.vertices if vertices is None else vertices, m.triangles if triangles is None else triangles)
    return bg.Space(mesh, X.refspace if refspace is None else refspace, X.fn_index if fn_index is None else fn_index,
                    X.fn_coef if fn_coef is None else fn_coef, X.nfun if nfun is None else nfun)


def test_space_validation_on_the_host(spaces):
    """The library's space checks (the same for every entry point) fail cleanly with a message."""
    X = spaces["rwg_sphere"]
    v = X.mesh.vertices.copy()
    v[5, 1] = np.nan
    t_bad = X.mesh.triangles.copy()
    t_bad[7, 2] = X.mesh.vertices.shape[0]
    t_deg = X.mesh.triangles.copy()
    t_deg[3, 1] = t_deg[3, 0]
    f_big = X.fn_index.copy()
    f_big[2, 0] = X.nfun
    f_dup = X.fn_index.copy()
    f_dup[4, 1] = f_dup[4, 0]
    c_bad = X.fn_coef.copy()
    c_bad[9, 2] = np.inf
    cases = [(dict(vertices=v), "non-finite vertex"), (dict(triangles=t_bad), "vertex index"),
             (dict(triangles=t_deg), "degenerate"), (dict(fn_index=f_big), "function index"),
             (dict(fn_index=f_dup), "two local shapes"), (dict(fn_coef=c_bad), "non-finite coefficient"),
             (dict(refspace=7), "refspace")]
    for kw, msg in cases:
        with pytest.raises(_lib.BGBError, match=msg):
            tile_order(_with(X, **kw), 64)
    tile_order(X, 64)  # the original space still passes
