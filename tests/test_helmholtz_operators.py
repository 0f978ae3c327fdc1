"""Helmholtz double layer, transposed double layer and hypersingular operators on hats.

Properties of the continuous operators that the discrete ones must reproduce (oracle on CPU,
GPU kernels on the GPU):
* Gauss's law: for k = 0 on a closed surface with outward normals, int dG/dn_y dy = -1/2, so
  K 1 = -1/2 (phi_i, 1) and likewise for the transposed double layer;
* the static hypersingular operator annihilates constants (surface curl of 1 is 0);
* K and K' are transposes of each other with the same rule on both sides (Sauter-Schwab rules
  are not exactly symmetric under the swap: agreement to their error, 1e-5).
"""
import numpy as np
import pytest

import beastgpu_gb300 as bg
import oracle

K1 = 2 * np.pi
SYM = bg.QuadStrat(far_test=4, far_trial=4, near_test=13, near_trial=13)


@pytest.fixture(scope="module")
def sphere():
    m = bg.icosphere(2)
    L = bg.lagrangec0d1(m)
    V, T = m.vertices, m.triangles
    A = 0.5 * np.linalg.norm(np.cross(V[T[:, 1]] - V[T[:, 0]], V[T[:, 2]] - V[T[:, 0]]), axis=1)
    mass1 = np.zeros(L.nfun)  # (phi_i, 1)
    for t in range(m.nt):
        for i in range(3):
            if L.fn_index[t, i] >= 0:
                mass1[L.fn_index[t, i]] += A[t] / 3 * L.fn_coef[t, i]
    return m, L, mass1


@pytest.mark.parametrize("name", ["doublelayer", "doublelayer_transposed"])
def test_oracle_gauss_law(sphere, name):
    m, L, mass1 = sphere
    K = oracle.assemble(getattr(bg.Helmholtz3D, name)(gamma=0.0), L, L, bg.QuadStrat())
    ratio = (K.sum(axis=1) if name == "doublelayer" else K.sum(axis=0)) / mass1
    assert np.abs(ratio + 0.5).max() < 1e-3


def test_oracle_hypersingular_annihilates_constants(sphere):
    m, L, _ = sphere
    W = oracle.assemble(bg.Helmholtz3D.hypersingular(gamma=0.0), L, L, bg.QuadStrat())
    assert np.abs(W.sum(axis=1)).max() < 1e-13 * np.abs(W).max()


def test_oracle_double_layers_are_transposes(sphere):
    m, L, _ = sphere
    K = oracle.assemble(bg.Helmholtz3D.doublelayer(wavenumber=K1), L, L, SYM)
    Kt = oracle.assemble(bg.Helmholtz3D.doublelayer_transposed(wavenumber=K1), L, L, SYM)
    assert np.linalg.norm(K.T - Kt) / np.linalg.norm(K) < 1e-5


def test_hypersingular_defaults():
    op = bg.Helmholtz3D.hypersingular(wavenumber=3.0)
    assert op.alpha == (3j) ** 2 and op.beta == 1.0 and op.kind == 5


OPS = {"dl": bg.Helmholtz3D.doublelayer, "dlt": bg.Helmholtz3D.doublelayer_transposed,
       "hs": bg.Helmholtz3D.hypersingular}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(OPS))
def test_gpu_parity_full_matrices(sphere, name):
    """Full matrices on the level-2 sphere and the jittered plates (near pairs): FP64 to 1e-12 and
    mixed to 1e-5 of the oracle; bit-identical across tile shapes."""
    m, L, _ = sphere
    # two jittered parallel plates 0.01 apart (near pairs; the double layers do not vanish)
    p = bg.plate(12, jitter=0.3, seed=1)
    v2 = p.vertices.copy()
    v2[:, 2] += 0.01
    plates = bg.Mesh(np.concatenate([p.vertices, v2]), np.concatenate([p.triangles, p.triangles + p.nv]))
    for mesh, X, k in ((m, L, K1), (plates, bg.lagrangec0d1(plates), 4 * np.pi)):
        op = OPS[name](wavenumber=k)
        ref = oracle.assemble(op, X, X, bg.QuadStrat())
        z64 = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"))
        zmx = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed"))
        scale = np.linalg.norm(ref)
        assert np.linalg.norm(z64 - ref) / scale < 1e-12
        assert np.linalg.norm(zmx.astype(np.complex128) - ref) / scale < 1e-5
        other = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed", tile_config=6))
        np.testing.assert_array_equal(other, zmx)


@pytest.mark.gpu
def test_gpu_gauss_law_and_constants(sphere):
    m, L, mass1 = sphere
    for prec, tol in (("fp64", 1e-3), ("mixed", 1e-3)):
        K = bg.assemble_gpu(bg.Helmholtz3D.doublelayer(gamma=0.0), L, L, bg.GPUConfiguration(precision=prec))
        assert np.abs(K.sum(axis=1) / mass1 + 0.5).max() < tol
    W = bg.assemble_gpu(bg.Helmholtz3D.hypersingular(gamma=0.0), L, L, bg.GPUConfiguration(precision="fp64"))
    assert np.abs(W.sum(axis=1)).max() < 1e-12 * np.abs(W).max()
