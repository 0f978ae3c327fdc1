"""The curve (2-D) oracle pinned to independent references (no GPU).

* The kernel (oracle.green2d) against scipy's Hankel functions.
* The graded rule against integrals of ln z.
* Local matrices of coincident, common-vertex, near and far segment pairs against the nested
  adaptive (QUADPACK) integrals of tests/golden/curve_pairs.npz (made by
  tests/golden/make_curve_fixtures.py): the singular rules converge exponentially in their order
  to 1e-12, near and far pairs to the rule's accuracy.
* Identities on closed polygons: Gauss's law for the static double layer, W 1 = 0 for the static
  hypersingular operator, K' = K^T, symmetry of the single layer, and the single layer of a
  constant density on a circle (-(i pi a / 2) J0(ka) H0^(2)(ka)) at second order in h.
"""
import os

import numpy as np
import pytest
from scipy import special

import beastgpu_gb300 as bg
import oracle
from beastgpu_gb300.curves import Operator2D, QuadStrat2D

FIX = os.path.join(os.path.dirname(__file__), "golden", "curve_pairs.npz")


def test_green_function_matches_scipy():
    for k, R in [(1.0, 0.3), (5.0, 2.0), (30.0, 1e-3), (0.2, 40.0), (12.0, 7.5)]:
        G, g1 = oracle.green2d(k, R)
        assert abs(G - (-0.25j * special.hankel2(0, k * R))) <= 1e-14 * abs(G)
        assert abs(g1 - 0.25j * k * special.hankel2(1, k * R) / R) <= 1e-14 * abs(g1)
    G, g1 = oracle.green2d(0.0, 0.7)
    assert abs(G + np.log(0.7) / (2 * np.pi)) < 1e-16 and abs(g1 + 1 / (2 * np.pi * 0.49)) < 1e-15


def test_graded_rule_integrates_logarithms():
    errs = []
    for n in (4, 8, 10, 12):
        x, w = oracle.graded01(n)
        assert np.all(np.diff(x) > 0) and 0 < x[0] and x[-1] < 1
        assert abs(w.sum() - 1) < 1e-14
        errs.append(max(abs(w @ np.log(x) + 1), abs(w @ (x * np.log(x)) + 0.25)))
    assert errs[1] < 1e-10 and errs[2] < 1e-12 and errs[3] < 1e-14, errs


@pytest.fixture(scope="module")
def fx():
    d = dict(np.load(FIX))
    V = d["vertices"]
    T = bg.curve_lagrangec0d1(bg.CurveMesh(V, d["test_segments"]), dirichlet=False)
    B = bg.curve_lagrangec0d1(bg.CurveMesh(V, d["trial_segments"]), dirichlet=False)
    return d, T, B


def test_fixture_machinery_against_closed_form(fx):
    # sum of the static hat matrix of a coincident pair = -(l^2 / 2 pi)(ln l - 3/2)
    assert float(fx[0]["closed_form_check"]) < 1e-14


def _rel(L, ref):
    out = []
    for p in range(len(ref)):
        nr = np.abs(ref[p]).max()
        out.append(np.abs(L[p] - ref[p]).max() / nr if nr > 0 else np.abs(L[p]).max())
    return np.array(out)


def _ref(d, kind, k, alpha=1.0, beta=1.0, T=None, B=None):
    """Reference local matrices of the fixture pairs for operator `kind` (hats)."""
    if kind in ("sl", "dl", "dlt"):
        return alpha * d[f"{kind}_k{int(k)}"]
    # hypersingular: alpha (n_x . n_y) SL + beta f' g' sum(SL)
    sl = d[f"sl_k{int(k)}"]
    out = np.empty_like(sl)
    for p, (t, s) in enumerate(zip(d["tau"], d["sigma"])):
        a, b = T.mesh.segments[t], B.mesh.segments[s]
        dA = T.mesh.vertices[a[1]] - T.mesh.vertices[a[0]]
        dB = B.mesh.vertices[b[1]] - B.mesh.vertices[b[0]]
        lA, lB = np.linalg.norm(dA), np.linalg.norm(dB)
        nn = (dA[1] * dB[1] + dA[0] * dB[0]) / (lA * lB)
        der = np.outer([-1 / lA, 1 / lA], [-1 / lB, 1 / lB])
        out[p] = alpha * nn * sl[p] + beta * der * sl[p].sum()
    return out


KINDS = {"sl": 0, "dl": 1, "dlt": 2, "hs": 3}


@pytest.mark.parametrize("k", [0.0, 3.0])
@pytest.mark.parametrize("kind", list(KINDS))
def test_oracle_converges_to_adaptive_references(fx, kind, k):
    d, T, B = fx
    alpha, beta = (0.7 - 0.2j), (1.3 + 0.4j)
    op = Operator2D(KINDS[kind], k, alpha, beta)
    ref = _ref(d, kind, k, alpha, beta, T, B)
    sing = d["cls"] != 0
    sing &= d["cls"] != 4
    errs = []
    for n in (4, 6, 8, 10, 12):
        L, cls = oracle.local_matrices_curve(op, T, B, QuadStrat2D(singular=n), d["tau"], d["sigma"])
        assert (cls == d["cls"]).all()
        errs.append(_rel(L, ref)[sing].max())
    assert errs[0] < 1e-3 and errs[-1] < 1e-12, errs
    assert all(a > b for a, b in zip(errs[:3], errs[1:4])), errs
    # near pairs (0.03 apart on 0.5-long segments) by the bisected rule, far pairs by Gauss-Legendre
    L, _ = oracle.local_matrices_curve(op, T, B, QuadStrat2D(), d["tau"], d["sigma"])
    e = _rel(L, ref)
    assert e[d["cls"] == 4].max() < 1e-12, e
    assert e[d["cls"] == 0].max() < 1e-6, e  # 4 x 4 points, k l = 1.5 per segment
    L, _ = oracle.local_matrices_curve(op, T, B, QuadStrat2D(far_test=12, far_trial=12), d["tau"], d["sigma"])
    assert _rel(L, ref)[d["cls"] == 0].max() < 1e-13


def test_piecewise_constants_are_sums_of_hat_matrices(fx):
    d, T, B = fx
    Tc = bg.curve_lagrangecxd0(T.mesh)
    Bc = bg.curve_lagrangecxd0(B.mesh)
    for kind in ("sl", "dl", "dlt"):
        op = Operator2D(KINDS[kind], 3.0, 1.0)
        L, _ = oracle.local_matrices_curve(op, Tc, Bc, QuadStrat2D(singular=12, far_test=12, far_trial=12), d["tau"],
                                           d["sigma"])
        ref = d[f"{kind}_k3"].sum(axis=(1, 2))
        nz = np.abs(ref) > 0
        assert np.all(np.abs(L[:, 0, 0] - ref)[nz] < 1e-12 * np.abs(ref)[nz])
        assert np.all(L[:, 0, 1] == 0) and np.all(L[:, 1, :] == 0)


def test_classes_on_a_polygon():
    X = bg.curve_lagrangec0d1(bg.circle(32))
    for k2 in (0.0, 100.0):
        c = oracle.classify_block_curve(X, X, k2)
        assert np.all(np.diag(c) == 3)
        n = 32
        for t in range(n):
            assert c[t, (t + 1) % n] == 1 and c[t, (t - 1) % n] == 1
        assert set(np.unique(c)) <= {0, 1, 3, 4}
    # k = 0: near pairs are those with the least vertex distance below sqrt(0.64 l)
    c0 = oracle.classify_block_curve(X, X, 0.0)
    assert (c0 == 4).sum() > 0
    assert ((oracle.classify_block_curve(X, X, 1e4)) == 4).sum() < (c0 == 4).sum()


def test_spaces():
    assert bg.lagrangec0d1(bg.circle(10)).nfun == 10
    assert bg.lagrangec0d1(bg.arc(10)).nfun == 9
    assert bg.lagrangec0d1(bg.arc(10), dirichlet=False).nfun == 11
    X = bg.lagrangecxd0(bg.arc(10))
    assert X.nfun == 10 and np.all(X.fn_index[:, 1] == -1)
    with pytest.raises(NotImplementedError):
        bg.lagrangecxd0(bg.icosphere(0))


def _full(op, X, qs=QuadStrat2D()):
    return oracle.assemble_curve(op, X, X, qs)


def test_gauss_law_and_hypersingular_nullspace():
    X = bg.curve_lagrangec0d1(bg.ellipse(40, 1.0, 0.6, jitter=0.3, seed=3))
    # int f_m over the curve (hats: half the lengths of the two segments)
    lens = X.mesh.lengths()
    mass = np.zeros(X.nfun)
    for e, (a, b) in enumerate(X.fn_index):
        mass[a] += lens[e] / 2
        mass[b] += lens[e] / 2
    K = _full(Operator2D(1, 0.0, 1.0), X)
    assert np.abs(K.sum(axis=1) + 0.5 * mass).max() < 1e-8 * mass.max()  # default 4 x 4 far rule
    K = _full(Operator2D(1, 0.0, 1.0), X, QuadStrat2D(far_test=10, far_trial=10, near=20, singular=14))
    assert np.abs(K.sum(axis=1) + 0.5 * mass).max() < 1e-14 * mass.max()
    W = _full(bg.Helmholtz2D.hypersingular(wavenumber=0.0), X)
    assert np.abs(W.sum(axis=1)).max() < 1e-13 * np.abs(W).max()


def test_transpose_and_symmetry():
    X = bg.curve_lagrangec0d1(bg.ellipse(30, 1.0, 0.5, jitter=0.3, seed=4))
    k = 4.0
    K = _full(bg.Helmholtz2D.doublelayer(wavenumber=k), X)
    Kt = _full(bg.Helmholtz2D.doublelayer_transposed(wavenumber=k), X)
    assert np.abs(Kt - K.T).max() < 1e-11 * np.abs(K).max()
    for op in (bg.Helmholtz2D.singlelayer(wavenumber=k), bg.Helmholtz2D.hypersingular(wavenumber=k)):
        Z = _full(op, X)
        assert np.abs(Z - Z.T).max() < 1e-11 * np.abs(Z).max()


def test_single_layer_of_a_constant_on_a_circle():
    """S 1 = -(i pi a / 2) J0(ka) H0^(2)(ka) on the circle of radius a; the polygon's error is O(h^2)."""
    a, k = 0.8, 5.0
    exact = -0.5j * np.pi * a * special.jv(0, k * a) * special.hankel2(0, k * a)
    errs = []
    for n in (64, 128):
        X = bg.curve_lagrangecxd0(bg.circle(n, a))
        Z = _full(bg.Helmholtz2D.singlelayer(wavenumber=k), X)
        l = X.mesh.lengths()
        errs.append(np.abs(Z.sum(axis=1) / l - exact).max() / abs(exact))
    assert errs[0] < 5e-3 and 3.5 < errs[0] / errs[1] < 4.5, errs


def test_oracle_rejects_bad_rules():
    X = bg.curve_lagrangec0d1(bg.circle(8))
    with pytest.raises(RuntimeError):
        oracle.local_matrices_curve(Operator2D(0, 1.0), X, X, QuadStrat2D(singular=17), [0], [0])
    with pytest.raises(RuntimeError):  # a common-vertex rule forced on a far pair
        oracle.local_matrices_curve(Operator2D(0, 1.0), X, X, QuadStrat2D(), [0], [4], force_class=1)


def _besselfit():
    import re
    txt = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "beastgpu_gb300", "csrc",
                            "besselfit.h")).read()
    return {m.group(1): np.array([float(v.rstrip("f")) for v in m.group(2).split(",")], dtype=np.float32)
            for m in re.finditer(r"#define BGB_BESSEL_(\w\w) \{([^}]*)\}", txt)}


def _horner32(c, u):
    v = np.full_like(u, c[-1])
    for a in c[-2::-1]:
        v = (v * u + a).astype(np.float32)
    return v


def test_fp32_hankel_approximations_of_the_mixed_kernels():
    """besselfit.h evaluated in FP32 as the mixed kernels do (phase x mod 2 pi carried in FP64)
    against scipy's Hankel functions: relative error below 1e-6 for 1e-4 <= x <= 1e5."""
    c = _besselfit()
    with np.errstate(all="ignore"):  # both branches are evaluated everywhere; np.where keeps the valid one
        x = np.logspace(-4, 5, 20001)
        xf = x.astype(np.float32)
        phi = np.mod(x, 2 * np.pi).astype(np.float32)
        for nu in (0, 1):
            ref = special.hankel2(nu, x)
            small = x < 3
            u = (xf * xf * np.float32(1 / 9)).astype(np.float32)
            lg = np.log(np.float32(0.5) * xf).astype(np.float32)
            if nu == 0:
                j = _horner32(c["P0"], u)
                y = (np.float32(2 / np.pi) * lg * j + _horner32(c["Q0"], u)).astype(np.float32)
            else:
                j = (xf * _horner32(c["P1"], u)).astype(np.float32)
                y = ((np.float32(2 / np.pi) * xf * lg * j + _horner32(c["Q1"], u)) / xf).astype(np.float32)
            t = (np.float32(3) / xf).astype(np.float32)
            F, G = _horner32(c[f"F{nu}"], t), _horner32(c[f"G{nu}"], t)
            th = (phi - np.float32(np.pi / 4 * (1 + 2 * nu)) + G).astype(np.float32)
            amp = (F / np.sqrt(xf)).astype(np.float32)
            big = amp * (np.cos(th) - 1j * np.sin(th))
            H = np.where(small, j - 1j * y, big)
            err = np.abs(H - ref) / np.abs(ref)
            assert err.max() < 1e-6, (nu, err.max(), x[np.argmax(err)])
