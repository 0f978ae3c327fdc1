"""Parity of the curve (2-D) path on the GPU with the FP64 oracle (bgb_assemble_curve,
bgb_local_matrices_curve through the C ABI).

Bar: FP64 outputs within 1e-12 (relative Frobenius norm, and every local matrix within 1e-12
of the oracle's), complex-float outputs within 1e-6; the mixed path (FP32 far pairs) within 1e-5
of the oracle with its coincident, common-vertex (double-float) and near (FP64) pairs within 1e-12
of the FP64 path's;
classes and class counts identical; results bit-identical from run to run and across column
blocks.
"""
import os

import numpy as np
import pytest

import beastgpu_gb300 as bg
import oracle
from beastgpu_gb300.curves import Operator2D, QuadStrat2D

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "curve_pairs.npz")


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _ops(k):
    return [bg.Helmholtz2D.singlelayer(wavenumber=k), bg.Helmholtz2D.doublelayer(wavenumber=k, alpha=0.5 - 1j),
            bg.Helmholtz2D.doublelayer_transposed(wavenumber=k), bg.Helmholtz2D.hypersingular(wavenumber=k)]


CURVES = {
    "ellipse": lambda: bg.ellipse(48, 1.0, 0.6, jitter=0.3, seed=5),
    "arc": lambda: bg.arc(24, 1.0, 1.5 * np.pi),
    "two_close": lambda: bg.union(bg.circle(24, 0.5), bg.circle(20, 0.45, center=(1.0, 0.02))),
}


@pytest.mark.parametrize("curve", list(CURVES))
@pytest.mark.parametrize("k", [0.0, 3.7])
def test_full_matrices_match_the_oracle(curve, k):
    m = CURVES[curve]()
    for X in (bg.curve_lagrangec0d1(m), bg.curve_lagrangecxd0(m)):
        for op in _ops(k):
            Z = bg.assemble_gpu(op, X, X)
            Zo = oracle.assemble_curve(op, X, X, QuadStrat2D())
            assert Z.dtype == np.complex128 and Z.flags.f_contiguous
            assert rel(Z, Zo) < 1e-12, (curve, X, op)


def test_classes_and_stats_match_the_oracle():
    X = bg.curve_lagrangec0d1(CURVES["two_close"]())
    op = bg.Helmholtz2D.singlelayer(wavenumber=2.0)
    _, st = bg.assemble_gpu(op, X, X, return_stats=True)
    c = oracle.classify_block_curve(X, X, 4.0)
    assert st["pairs_total"] == c.size
    for cls in (0, 1, 3, 4):
        assert st["pairs_class"][cls] == int((c == cls).sum()), cls
    assert st["pairs_class"][4] > 0


def test_distinct_test_and_trial_curves_rows_and_outputs():
    A = bg.curve_lagrangec0d1(bg.ellipse(40, 1.0, 0.7, jitter=0.2, seed=1))
    B = bg.curve_lagrangecxd0(bg.union(bg.arc(12, 1.05, np.pi), bg.circle(10, 0.2, center=(0.2, 0.1))))
    op = bg.Helmholtz2D.doublelayer(wavenumber=5.0)
    Zo = oracle.assemble_curve(op, A, B, QuadStrat2D())
    Z = bg.assemble_gpu(op, A, B)
    assert rel(Z, Zo) < 1e-12
    Zr = bg.assemble_gpu(op, A, B, rows=(7, 20))
    assert rel(Zr, Zo[7:27]) < 1e-12
    Z32 = bg.assemble_gpu(op, A, B, dtype=np.complex64)
    assert Z32.dtype == np.complex64 and rel(Z32, Zo) < 1e-6
    Zd = bg.assemble_gpu(op, A, B, out="device").cpu().numpy()
    assert np.array_equal(Zd, Z)
    # host output with a leading dimension larger than the row count keeps the other rows
    big = np.full((35, B.nfun), 7 + 7j, dtype=np.complex128, order="F")
    view = big[3:23]
    import ctypes as C
    from beastgpu_gb300 import _lib, api
    h = api.get_handle(0)
    keep = api._Keep()
    st = _lib.Stats()
    _lib.check(_lib.load().bgb_assemble_curve(h.ptr, C.byref(api.c_operator2d(op)), C.byref(api.c_curve_space(A, keep)),
                                              C.byref(api.c_curve_space(B, keep)),
                                              C.byref(api.c_quadstrat2d(QuadStrat2D())), _lib.PREC_FP64,
                                              C.c_void_p(view.ctypes.data),
                                              _lib.OUT_HOST_C64, 35, 7, 20, None, C.byref(st)))
    assert rel(big[3:23], Zo[7:27]) < 1e-12
    assert np.all(big[:3] == 7 + 7j) and np.all(big[23:] == 7 + 7j)


def test_column_blocks_and_determinism():
    X = bg.curve_lagrangec0d1(bg.ellipse(300, 1.0, 0.4, jitter=0.3, seed=2))
    op = bg.Helmholtz2D.hypersingular(wavenumber=6.0)
    Z1, st1 = bg.assemble_gpu(op, X, X, return_stats=True)
    Z2 = bg.assemble_gpu(op, X, X)
    assert np.array_equal(Z1, Z2)
    assert st1["out_blocks"] == 1
    # a small HBM budget forces many column blocks: same matrix, bit for bit
    Zb, stb = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(total_GPU_budget=4 << 20), return_stats=True)
    assert stb["out_blocks"] > 4
    assert np.array_equal(Zb, Z1)
    rows = np.random.default_rng(0).choice(X.nfun, 25, replace=False)
    Zo = oracle.assemble_rows_curve(op, X, X, QuadStrat2D(), rows)
    assert rel(Z1[rows], Zo) < 1e-12


def test_local_matrices_match_the_oracle_for_every_class():
    d = dict(np.load(FIX))
    V = d["vertices"]
    T = bg.curve_lagrangec0d1(bg.CurveMesh(V, d["test_segments"]), dirichlet=False)
    B = bg.curve_lagrangec0d1(bg.CurveMesh(V, d["trial_segments"]), dirichlet=False)
    for k in (0.0, 3.0):
        for kind in range(4):
            op = Operator2D(kind, k, 0.7 - 0.2j, 1.3 + 0.4j)
            for qs in (QuadStrat2D(), QuadStrat2D(far_test=7, far_trial=5, near=9, singular=6)):
                L, cls = bg.local_matrices_curve(op, T, B, d["tau"], d["sigma"], quadstrat=qs)
                Lo, clso = oracle.local_matrices_curve(op, T, B, qs, d["tau"], d["sigma"])
                assert np.array_equal(cls, clso) and np.array_equal(cls, d["cls"])
                for p in range(len(cls)):
                    nr = np.abs(Lo[p]).max()
                    assert np.abs(L[p] - Lo[p]).max() <= 1e-12 * max(nr, 1e-300) + (0 if nr else 1e-300), (k, kind, p)
    # forced rules: near on a far pair is fine; a singular rule on a pair of another class is an error
    op = Operator2D(0, 3.0)
    far = np.nonzero(d["cls"] == 0)[0]
    L, _ = bg.local_matrices_curve(op, T, B, d["tau"][far], d["sigma"][far], force_class=4)
    Lo, _ = oracle.local_matrices_curve(op, T, B, QuadStrat2D(), d["tau"][far], d["sigma"][far], force_class=4)
    assert np.abs(L - Lo).max() <= 1e-12 * np.abs(Lo).max()
    with pytest.raises(bg._lib.BGBError):
        bg.local_matrices_curve(op, T, B, d["tau"][far], d["sigma"][far], force_class=1)


def test_identities_at_size():
    """Properties that hold at any size: Gauss's law of the static double layer and W 1 = 0."""
    X = bg.curve_lagrangec0d1(bg.ellipse(2000, 1.0, 0.6, jitter=0.2, seed=9))
    lens = X.mesh.lengths()
    mass = np.zeros(X.nfun)
    np.add.at(mass, X.fn_index[:, 0], lens / 2)
    np.add.at(mass, X.fn_index[:, 1], lens / 2)
    qs = QuadStrat2D(far_test=10, far_trial=10, near=20, singular=14)
    K = bg.assemble_gpu(Operator2D(1, 0.0, 1.0), X, X, quadstrat=qs)
    assert np.abs(K.sum(axis=1) + 0.5 * mass).max() < 1e-13 * mass.max()
    W = bg.assemble_gpu(bg.Helmholtz2D.hypersingular(wavenumber=0.0), X, X)
    assert np.abs(W.sum(axis=1)).max() < 1e-12 * np.abs(W).max()


def test_invalid_inputs_raise():
    X = bg.curve_lagrangec0d1(bg.circle(8))
    with pytest.raises(bg._lib.BGBError):
        bg.assemble_gpu(Operator2D(0, -1.0), X, X)
    with pytest.raises(bg._lib.BGBError):
        bg.assemble_gpu(Operator2D(0, 1.0), X, X, quadstrat=QuadStrat2D(singular=0))
    bad = bg.CurveSpace(bg.CurveMesh(X.mesh.vertices, np.array([[0, 0]] + X.mesh.segments[1:].tolist())),
                        X.refspace, X.fn_index, X.fn_coef, X.nfun)
    with pytest.raises(bg._lib.BGBError):
        bg.assemble_gpu(Operator2D(0, 1.0), bad, bad)
    # mixed precision carries the phase for k times the diameter up to 3e5
    with pytest.raises(bg._lib.BGBError) as e:
        bg.assemble_gpu(Operator2D(0, 2e5), X, X, bg.GPUConfiguration(precision="mixed"))
    assert e.value.code == -7


@pytest.mark.parametrize("curve", list(CURVES))
@pytest.mark.parametrize("k", [0.0, 3.7, 40.0])
def test_mixed_precision_matches_the_oracle(curve, k):
    m = CURVES[curve]()
    cfg = bg.GPUConfiguration(precision="mixed")
    for X in (bg.curve_lagrangec0d1(m), bg.curve_lagrangecxd0(m)):
        for op in _ops(k):
            Z = bg.assemble_gpu(op, X, X, cfg)
            assert Z.dtype == np.complex64
            Zo = oracle.assemble_curve(op, X, X, QuadStrat2D())
            assert rel(Z, Zo) < 1e-5, (curve, X, op, rel(Z, Zo))


def test_mixed_local_matrices():
    d = dict(np.load(FIX))
    V = d["vertices"]
    T = bg.curve_lagrangec0d1(bg.CurveMesh(V, d["test_segments"]), dirichlet=False)
    B = bg.curve_lagrangec0d1(bg.CurveMesh(V, d["trial_segments"]), dirichlet=False)
    for k in (0.0, 3.0, 10.0):
        for kind in range(4):
            op = Operator2D(kind, k, 0.7 - 0.2j, 1.3 + 0.4j)
            Lm, cls = bg.local_matrices_curve(op, T, B, d["tau"], d["sigma"], precision="mixed")
            Ld, _ = bg.local_matrices_curve(op, T, B, d["tau"], d["sigma"], precision="fp64")
            far = cls == 0  # the near pairs of k <= 3 are far at k = 10
            # singular pairs in double-float (single layer, hypersingular) or FP64, near pairs in FP64
            nf = np.abs(Ld[~far]).max(axis=(1, 2))
            err = np.abs(Lm[~far] - Ld[~far]).max(axis=(1, 2))
            assert np.all(err <= 1e-12 * np.where(nf > 0, nf, 1e-300)), (k, kind, err / np.where(nf > 0, nf, 1))
            Lo, _ = oracle.local_matrices_curve(op, T, B, QuadStrat2D(), d["tau"][far], d["sigma"][far])
            assert np.abs(Lm[far] - Lo).max() <= 1e-5 * np.abs(Lo).max(), (k, kind)


def test_mixed_precision_at_high_frequency():
    """k = 2 pi * 100 on 2,000 segments (k R up to 1,300): the phase is carried in FP64 per pair."""
    X = bg.curve_lagrangec0d1(bg.ellipse(2000, 1.0, 0.5, jitter=0.2, seed=11))
    op = bg.Helmholtz2D.hypersingular(wavenumber=2 * np.pi * 100)
    Z = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed"))
    rows = np.random.default_rng(1).choice(X.nfun, 40, replace=False)
    Zo = oracle.assemble_rows_curve(op, X, X, QuadStrat2D(), rows)
    assert rel(Z[rows], Zo) < 1e-5
