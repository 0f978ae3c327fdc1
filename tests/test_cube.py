"""The reference's own correctness case: Helmholtz3D single layer, k = 1, on lagrangec0d1 over
meshcuboid(1, 1, 1, 0.5) (test/correctness.jl:22-25), checked the way the reference checks it
(max |Z - Z_ref| < 1e-10, test/correctness.jl:39 with test/difference.jl:1-6), for every
configuration its generate_configs() varies that exists here (test/configers.jl:6-53): both
write-back strategies, one or two row chunks ("amount_of_gpus"), output on the host or the device.

The reference compares against a cached BEAST matrix that is absent from its repository; here
the matrix of the FP64 oracle stands in for it.  The mesh-level tests need no GPU.
"""
import numpy as np
import pytest

import beastgpu_gb300 as bg
import oracle

REF_TOL = 1e-10  # test/correctness.jl:39, absolute


def edge_use(m):
    t = m.triangles.astype(np.int64)
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    key = np.minimum(e[:, 0], e[:, 1]) * m.nv + np.maximum(e[:, 0], e[:, 1])
    _, cnt = np.unique(key, return_counts=True)
    return cnt


@pytest.mark.parametrize("d", [1, 2, 3, 40])
def test_meshcuboid_counts_and_closed_surface(d):
    m = bg.meshcuboid(1.0, 1.0, 1.0, 0.5 / d)
    n = 2 * d
    assert m.nt == 12 * n * n and m.nv == 6 * n * n + 2  # data/graph_data.jl:3-4
    assert np.all(edge_use(m) == 2)  # closed two-manifold
    v = m.vertices[m.triangles]
    nrm = np.cross(v[:, 0] - v[:, 2], v[:, 1] - v[:, 2])
    assert np.all(np.einsum("ij,ij->i", nrm, v.mean(axis=1) - 0.5) > 0)  # chart normals outward
    assert np.allclose(m.areas(), 0.5 * (0.5 / d) ** 2)
    assert bg.lagrangec0d1(m).nfun == m.nv  # closed: every vertex carries a hat
    assert m.vertices.min() == 0.0 and m.vertices.max() == 1.0


def test_meshcuboid_boxes_and_bad_steps():
    m = bg.meshcuboid(2.0, 1.0, 0.5, 0.25)
    assert m.nt == 2 * 2 * (8 * 4 + 8 * 2 + 4 * 2)
    assert np.isclose(m.areas().sum(), 2 * (2.0 + 1.0 + 0.5))
    with pytest.raises(ValueError):
        bg.meshcuboid(1.0, 1.0, 1.0, 0.3)


def test_cube_oracle_classes():
    """A structured cube has singular pairs of every class and no near pair (the reference's
    dropped near class is empty on it)."""
    X = bg.lagrangec0d1(bg.meshcuboid(1.0, 1.0, 1.0, 0.25))
    c = oracle.classify_block(X, X, 1.0)
    counts = np.bincount(c.ravel(), minlength=5)
    assert counts[3] == X.mesh.nt and counts[1] > 0 and counts[2] > 0 and counts[4] == 0


@pytest.fixture(scope="module")
def cube1():
    X = bg.lagrangec0d1(bg.meshcuboid(1.0, 1.0, 1.0, 0.5))
    op = bg.Helmholtz3D.singlelayer(wavenumber=1.0)
    return X, op, oracle.assemble(op, X, X, bg.QuadStrat())


@pytest.mark.gpu
@pytest.mark.parametrize("wb", ["true", "false"])
@pytest.mark.parametrize("chunks", [1, 2])
def test_reference_correctness_case_fp64(cube1, wb, chunks):
    X, op, ref = cube1
    strat = bg.GpuWriteBackTrueInstance() if wb == "true" else bg.GpuWriteBackFalseInstance()
    # the reference's configuration fields (test/configers.jl:31-43) and call (test/correctness.jl:36)
    cfg = bg.GPUConfiguration(writeBackStrategy=strat, amount_of_gpus=chunks, total_GPU_budget=3 * 2 ** 30,
                              floatType=np.float64)
    Z = bg.assemble_gpu(op, X, X, cfg, cfg.writeBackStrategy)
    assert Z.shape == (26, 26) and Z.dtype == np.complex128
    assert np.abs(Z - ref).max() < REF_TOL
    assert np.abs(Z - ref).max() < 1e-12 * np.abs(ref).max()


@pytest.mark.gpu
def test_reference_correctness_case_device_output_and_mixed(cube1):
    import torch
    X, op, ref = cube1
    Zd = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"), out="device")
    torch.cuda.synchronize()
    assert np.abs(Zd.cpu().numpy() - ref).max() < REF_TOL
    Zm = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed")).astype(np.complex128)
    # mixed precision at its own bound: FP32 far pairs, 1e-5 of the largest entry
    assert np.abs(Zm - ref).max() < 1e-5 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("d", [2, 4])
def test_cube_denser_meshes(d):
    """meshcuboid(1, 1, 1, 0.5/d) at d = 2 and 4 (the reference's benchmark family, data/graph_data.jl:2):
    full FP64 matrix against the oracle, mixed on seeded rows."""
    X = bg.lagrangec0d1(bg.meshcuboid(1.0, 1.0, 1.0, 0.5 / d))
    op = bg.Helmholtz3D.singlelayer(wavenumber=1.0)
    rows = np.sort(np.random.default_rng(d).choice(X.nfun, min(X.nfun, 64), replace=False)).astype(np.int32)
    ref = oracle.assemble_rows(op, X, X, bg.QuadStrat(), rows)
    Z = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"))
    assert np.abs(Z[rows] - ref).max() < REF_TOL
    Zm = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed"))
    assert np.linalg.norm(Zm[rows] - ref) / np.linalg.norm(ref) < 1e-5
