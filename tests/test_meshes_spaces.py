"""Synthetic meshes and function spaces (CPU)."""
import numpy as np
import pytest

import beastgpu_gb300 as bg


@pytest.mark.parametrize("level", [0, 1, 2, 3])
def test_icosphere_counts_and_orientation(level):
    m = bg.icosphere(level)
    assert m.nt == 20 * 4 ** level
    assert m.nv == 10 * 4 ** level + 2
    np.testing.assert_allclose(np.linalg.norm(m.vertices, axis=1), 1.0, atol=1e-15)
    v = m.vertices[m.triangles]
    n = np.cross(v[:, 0] - v[:, 2], v[:, 1] - v[:, 2])
    assert np.all(np.einsum("ij,ij->i", n, v.mean(1)) > 0)  # outward


def test_rwg_on_closed_surface(ico2):
    X = bg.raviartthomas(ico2)
    assert X.nfun == 30 * 4 ** 2
    off, tri, loc, coef = X.supports()
    assert np.all(np.diff(off) == 2)
    assert np.all(coef[0::2] == 1.0) and np.all(coef[1::2] == -1.0)
    # the shared edge is opposite the local shape on both sides
    t = ico2.triangles
    for f in range(0, X.nfun, 37):
        a, b = tri[off[f]], tri[off[f] + 1]
        ea = {t[a][(loc[off[f]] + 1) % 3], t[a][(loc[off[f]] + 2) % 3]}
        eb = {t[b][(loc[off[f] + 1] + 1) % 3], t[b][(loc[off[f] + 1] + 2) % 3]}
        assert ea == eb


def test_lagrange_closed_and_plate():
    m = bg.icosphere(1)
    L = bg.lagrangec0d1(m)
    assert L.nfun == m.nv
    p = bg.plate(8, jitter=0.3, seed=1)
    Lp = bg.lagrangec0d1(p)
    assert p.nt == 2 * 8 * 8 and Lp.nfun == 7 * 7  # interior vertices only
    Xp = bg.raviartthomas(p)
    assert Xp.nfun == 3 * 8 * 8 - 2 * 8  # interior edges


def test_plate_jitter_seeded_and_bounded():
    a = bg.plate(16, jitter=0.3, seed=1)
    b = bg.plate(16, jitter=0.3, seed=1)
    c = bg.plate(16, jitter=0.0)
    np.testing.assert_array_equal(a.vertices, b.vertices)
    d = np.abs(a.vertices - c.vertices)
    assert d.max() <= 0.3 / 16 + 1e-15 and d[:, 2].max() == 0.0
    assert np.all(a.areas() > 0)


def test_two_plates_gap():
    m = bg.two_plates(8, gap=0.01)
    assert m.nt == 2 * 128
    x = m.vertices[:, 0]
    assert np.isclose(x[m.triangles[128:]].min() - x[m.triangles[:128]].max(), 0.01)


def test_ellipsoid_batch_seeded():
    a = bg.ellipsoid_batch(8, seed=2)
    b = bg.ellipsoid_batch(8, seed=2)
    assert [m.nt for m, _ in a] == [m.nt for m, _ in b]
    for (m, k), (m2, k2) in zip(a, b):
        assert k == k2 and 1 <= k <= 10
        np.testing.assert_array_equal(m.vertices, m2.vertices)
        assert m.nt in (80, 320, 1280, 5120)
