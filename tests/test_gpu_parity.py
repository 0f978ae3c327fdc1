"""Parity of the CUDA path (through the C ABI) with the FP64 CPU oracle.

Tolerances: classification bit-exact; plain FP64 kernels 1e-12 relative (Frobenius) on full
matrices and singular-pair local matrices; mixed FP32 far pairs 1e-5 relative Frobenius (the
target of the mixed assembler); results bit-identical across tile shapes, runs and output kinds.
"""
import numpy as np
import pytest

import beastgpu_gb300 as bg
import oracle

pytestmark = pytest.mark.gpu

K1 = 2 * np.pi
FP64_TOL = 1e-12
MIXED_TOL = 1e-5


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def c1():
    m = bg.icosphere(2)
    return m, bg.raviartthomas(m), bg.lagrangec0d1(m)


@pytest.fixture(scope="module")
def plates():
    # two coplanar jittered plates: near pairs from the jitter (Lagrange and RWG)
    m = bg.two_plates(12, jitter=0.3, seed=1, gap=0.01)
    return m, bg.raviartthomas(m), bg.lagrangec0d1(m)


OPS = {
    "efie": (lambda k: bg.Maxwell3D.singlelayer(wavenumber=k), 1),
    "mfie": (lambda k: bg.Maxwell3D.doublelayer(wavenumber=k), 1),
    "hh": (lambda k: bg.Helmholtz3D.singlelayer(wavenumber=k), 2),
}


def _space(sp, which):
    return sp[which]


@pytest.mark.parametrize("k", [K1, 30.0, 0.0])
def test_classification_bit_exact_icosphere(c1, k):
    m, X, _ = c1
    np.testing.assert_array_equal(bg.classify(X, X, k * k), oracle.classify_block(X, X, k * k))


def test_classification_bit_exact_plates_with_near_pairs(plates):
    m, X, _ = plates
    k = 4 * np.pi
    got = bg.classify(X, X, k * k)
    np.testing.assert_array_equal(got, oracle.classify_block(X, X, k * k))
    assert (got == 4).sum() > 0, "the jittered plates should produce near pairs"


@pytest.mark.parametrize("n", [7, 13])
def test_classification_and_assembly_ragged_sizes(n):
    """Triangle counts that are not multiples of the 32-triangle chunks of the classifier
    (98 and 338 triangles), shuffled triangle order (loose chunk spheres): classes bit-exact, the
    assembled matrix equal to the oracle's."""
    p = bg.plate(n, jitter=0.3, seed=3)
    perm = np.random.default_rng(n).permutation(p.nt)
    m = bg.Mesh(p.vertices, p.triangles[perm])
    X = bg.raviartthomas(m)
    k = 6 * np.pi
    np.testing.assert_array_equal(bg.classify(X, X, k * k), oracle.classify_block(X, X, k * k))
    op = bg.Maxwell3D.singlelayer(wavenumber=k)
    ref = oracle.assemble(op, X, X, bg.QuadStrat())
    assert rel(bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64")), ref) < FP64_TOL
    assert rel(bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed")).astype(np.complex128), ref) < MIXED_TOL


@pytest.mark.parametrize("name", list(OPS))
@pytest.mark.parametrize("cls", [0, 1, 2, 3])
def test_local_matrices_per_class(c1, qs, name, cls):
    m, X, L = c1
    make, which = OPS[name]
    op = make(K1)
    sp = c1[which]
    c = oracle.classify_block(sp, sp, K1 * K1)
    t, s = np.nonzero(c == cls)
    sel = np.random.default_rng(cls).choice(t.size, min(150, t.size), replace=False)
    t, s = t[sel], s[sel]
    ref, rc = oracle.local_matrices(op, sp, sp, qs, t, s)
    got, gc = bg.local_matrices(op, sp, sp, t, s)
    np.testing.assert_array_equal(gc, rc)
    if name == "mfie" and cls == 3:
        assert np.all(got == 0) and np.all(ref == 0)  # double layer vanishes on a flat common face
        return
    assert rel(got, ref) < FP64_TOL
    # singular entries stay FP64 in the mixed mode; far pairs meet the mixed tolerance
    gm, _ = bg.local_matrices(op, sp, sp, t, s, precision="mixed")
    if cls == 0:
        assert rel(gm, ref) < MIXED_TOL
    else:
        assert rel(gm, ref) < FP64_TOL


@pytest.mark.parametrize("name", list(OPS))
def test_full_assembly_icosphere(c1, qs, name):
    m, X, L = c1
    make, which = OPS[name]
    op = make(K1)
    sp = c1[which]
    ref = oracle.assemble(op, sp, sp, qs)
    z64 = bg.assemble_gpu(op, sp, sp, bg.GPUConfiguration(precision="fp64"))
    assert z64.dtype == np.complex128 and z64.shape == ref.shape
    assert rel(z64, ref) < FP64_TOL
    zmx = bg.assemble_gpu(op, sp, sp, bg.GPUConfiguration(precision="mixed"))
    assert zmx.dtype == np.complex64
    assert rel(zmx.astype(np.complex128), ref) < MIXED_TOL


@pytest.mark.parametrize("name", ["hh", "mfie", "efie"])
def test_full_assembly_plates_near_pairs(plates, qs, name):
    m, X, L = plates
    make, which = OPS[name]
    op = make(4 * np.pi)
    sp = plates[which]
    ref = oracle.assemble(op, sp, sp, qs)
    z64 = bg.assemble_gpu(op, sp, sp, bg.GPUConfiguration(precision="fp64"))
    zmx = bg.assemble_gpu(op, sp, sp, bg.GPUConfiguration(precision="mixed"))
    if name == "mfie":
        # the double layer vanishes on a plane: f(x) . (grad G x g(y)) = 0 for coplanar x, y, f, g
        assert np.all(ref == 0) and np.abs(z64).max() == 0 and np.abs(zmx).max() < 1e-12
        return
    assert rel(z64, ref) < FP64_TOL
    assert rel(zmx.astype(np.complex128), ref) < MIXED_TOL


def test_bit_identical_across_tiles_runs_and_outputs(c1):
    import torch
    m, X, L = c1
    op = bg.Maxwell3D.singlelayer(wavenumber=K1)
    for prec, cfgs in (("fp64", (4, 5, 6, 8)), ("mixed", (0, 1, 2, 3, 5, 8))):
        outs = [bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision=prec, tile_config=c)) for c in cfgs]
        outs.append(bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision=prec)))
        for o in outs[1:]:
            np.testing.assert_array_equal(o, outs[0])
        dev = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision=prec), out="device")
        np.testing.assert_array_equal(dev.cpu().numpy(), outs[0])
        assert isinstance(dev, torch.Tensor)


def test_row_windows_and_writeback_strategies(c1):
    m, X, L = c1
    op = bg.Maxwell3D.singlelayer(wavenumber=K1)
    full = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"))
    part = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"), rows=(100, 77))
    np.testing.assert_array_equal(part, full[100:177])
    cpuwb = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"), bg.GpuWriteBackFalseInstance())
    np.testing.assert_array_equal(cpuwb, full)
    # out-of-core: a tiny HBM budget forces many output blocks; result unchanged
    small = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64", total_GPU_budget=4 * 30 * 480 * 16),
                            return_stats=True)
    np.testing.assert_array_equal(small[0], full)
    assert small[1]["out_blocks"] >= 16  # 30 columns per block (the last one cut shorter)


def test_out_of_core_pipeline_pinned_pageable_and_ring(c1):
    """Output blocks (column ranges) double-buffered on the device, copied while the next block
    is filled: pageable host outputs through a pinned ring (chunks of a few columns, and a ring
    smaller than one column), pinned outputs directly; all bit-identical to the device result."""
    import torch
    m, X, L = c1
    op = bg.Maxwell3D.singlelayer(wavenumber=K1)
    n = X.nfun
    for prec, esz, tdt in (("fp64", 16, torch.complex128), ("mixed", 8, torch.complex64)):
        ref = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision=prec), out="device").cpu().numpy()
        budget = 4 * 37 * n * esz  # 37 columns per block, the last block ragged
        cfg = bg.GPUConfiguration(precision=prec, total_GPU_budget=budget, pinned_ring_bytes=5 * n * esz)
        Z, st = bg.assemble_gpu(op, X, X, cfg, return_stats=True)
        assert st["out_blocks"] >= (n + 36) // 37
        np.testing.assert_array_equal(Z, ref)
        buf = torch.empty((n, n), dtype=tdt, pin_memory=True)  # column-major n x n
        bg.assemble_gpu(op, X, X, cfg, out_buffer=buf)
        np.testing.assert_array_equal(buf.numpy().T, ref)
        tiny_ring = bg.GPUConfiguration(precision=prec, total_GPU_budget=budget, pinned_ring_bytes=1,
                                        pageable_via_ring=True)
        W = bg.assemble_gpu(op, X, X, tiny_ring, rows=(50, 200))
        np.testing.assert_array_equal(W, ref[50:250])
        via_ring = bg.GPUConfiguration(precision=prec, total_GPU_budget=budget, pinned_ring_bytes=5 * n * esz,
                                       pageable_via_ring=True)
        np.testing.assert_array_equal(bg.assemble_gpu(op, X, X, via_ring), ref)


@pytest.mark.parametrize("name", ["efie", "mfie", "hh"])
def test_host_output_blocks_on_plates_with_near_pairs(plates, name):
    """A host output in many column blocks (RWG and Lagrange, the jittered plates' near pairs in
    most blocks), called twice on one handle and on a row window: bit-identical to the one-block
    device output in both precisions."""
    make, which = OPS[name]
    sp = plates[which]
    op = make(K1)
    n = sp.nfun
    for prec, esz in (("fp64", 16), ("mixed", 8)):
        ref = bg.assemble_gpu(op, sp, sp, bg.GPUConfiguration(precision=prec), out="device").cpu().numpy()
        cfg = bg.GPUConfiguration(precision=prec, total_GPU_budget=4 * 23 * n * esz)
        for _ in range(2):  # the second call reuses the handle's staging buffers and events
            Z, st = bg.assemble_gpu(op, sp, sp, cfg, return_stats=True)
            assert st["out_blocks"] >= n // 23
            assert st["ms_singular"] > 0
            np.testing.assert_array_equal(Z, ref)
        part = bg.assemble_gpu(op, sp, sp, cfg, rows=(11, n - 30))
        np.testing.assert_array_equal(part, ref[11:n - 19])


def test_host_output_with_leading_dimension_keeps_other_rows(c1):
    """Host output with ld > nrows (a window into a larger column-major array): the rows
    outside the window are untouched, for pinned, pageable and ring destinations."""
    import ctypes as C
    import torch
    from beastgpu_gb300 import _lib
    from beastgpu_gb300.api import _Keep, c_operator, c_quadstrat, c_space, get_handle
    m, X, L = c1
    op = bg.Maxwell3D.singlelayer(wavenumber=K1)
    n = X.nfun
    ref = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"))
    r0, nr, ld = 37, 101, 160
    keep = _Keep()
    sp = c_space(X, keep)
    cop, cq = c_operator(op), c_quadstrat(bg.QuadStrat())
    for flags, pinned in ((0, False), (0, True), (_lib.CFG_PAGEABLE_VIA_RING, False)):
        h = get_handle(0, 4 * 50 * nr * 16, -1, 3 * nr * 16, flags)
        if pinned:
            t = torch.full((n, ld), 7.0 + 0j, dtype=torch.complex128, pin_memory=True)
            buf, ptr = t.numpy().T, t.data_ptr()  # buf[i, j]: column-major ld x n
        else:
            buf = np.full((ld, n), 7.0 + 0j, dtype=np.complex128, order="F")
            ptr = buf.ctypes.data
        st = _lib.Stats()
        _lib.check(_lib.load().bgb_assemble(h.ptr, C.byref(cop), C.byref(sp), C.byref(sp), C.byref(cq),
                                            _lib.PREC_FP64, C.c_void_p(ptr), _lib.OUT_HOST_C64, ld, r0, nr, None,
                                            C.byref(st)))
        assert st.out_blocks > 1
        np.testing.assert_array_equal(buf[:nr], ref[r0:r0 + nr])
        assert np.all(buf[nr:] == 7.0)


def test_c2_sampled_rows(qs):
    """Level-5 icosphere EFIE (30,720 RWG), k = 8 pi: 24 seeded rows against the oracle."""
    m = bg.icosphere(5)
    X = bg.raviartthomas(m)
    op = bg.Maxwell3D.singlelayer(wavenumber=2 * np.pi * 4)
    rows = np.sort(np.random.default_rng(7).choice(X.nfun, 24, replace=False)).astype(np.int32)
    ref = oracle.assemble_rows(op, X, X, qs, rows)
    for prec, tol in (("mixed", MIXED_TOL), ("fp64", FP64_TOL)):
        Z = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision=prec), out="device")
        import torch
        got = Z[torch.as_tensor(rows.astype(np.int64), device=Z.device)].cpu().numpy().astype(np.complex128)
        assert rel(got, ref) < tol, prec
        del Z


def test_invalid_inputs_fail_cleanly_and_handle_survives(c1):
    m, X, L = c1
    op = bg.Maxwell3D.singlelayer(wavenumber=K1)
    bad = bg.Space(bg.Mesh(m.vertices, m.triangles), X.refspace, X.fn_index.copy(), X.fn_coef, X.nfun)
    bad.fn_index[5, 1] = X.nfun + 3
    with pytest.raises(bg._lib.BGBError) as e:
        bg.assemble_gpu(op, bad, bad)
    assert e.value.code == -1
    v = m.vertices.copy()
    v[3, 1] = np.nan
    nanmesh = bg.Space(bg.Mesh(v, m.triangles), X.refspace, X.fn_index, X.fn_coef, X.nfun)
    with pytest.raises(bg._lib.BGBError):
        bg.assemble_gpu(op, nanmesh, nanmesh)
    with pytest.raises(bg._lib.BGBError) as e:
        bg.assemble_gpu(op, X, X, quadstrat=bg.QuadStrat(far_test=5))
    assert e.value.code == -7
    with pytest.raises(bg._lib.BGBError) as e:
        bg.assemble_gpu(bg.Helmholtz3D.singlelayer(wavenumber=1.0), X, X)  # Helmholtz needs Lagrange
    assert e.value.code == -7
    # mixed precision reduces the phase k R exactly for k times the diameter up to 3e5
    with pytest.raises(bg._lib.BGBError) as e:
        bg.assemble_gpu(bg.Maxwell3D.singlelayer(wavenumber=2e5), X, X, bg.GPUConfiguration(precision="mixed"))
    assert e.value.code == -7
    # the handle still works
    z = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed"))
    assert np.isfinite(z).all()


def test_batch_bit_identical_to_single_assemblies(qs):
    """Uneven batch (ellipsoids of levels 1-2, different k): one persistent far launch over a work
    queue equals assembling each problem alone, for both precisions; the graph replay too."""
    import torch
    probs = []
    for m, k in bg.ellipsoid_batch(6, seed=3, levels=(1, 2)):
        X = bg.raviartthomas(m)
        probs.append((bg.Maxwell3D.singlelayer(wavenumber=k), X, X))
    for prec in ("mixed", "fp64"):
        b = bg.Batch(probs, bg.GPUConfiguration(precision=prec), out="device", autotune=True)
        first = [o.clone() for o in b.outputs]
        b.run()
        for (op, X, Y), o, f in zip(probs, b.outputs, first):
            z = bg.assemble_gpu(op, X, Y, bg.GPUConfiguration(precision=prec), out="device")
            assert torch.equal(z, o) and torch.equal(z, f)
        b.close()
    # host outputs of a one-shot batch, against the oracle
    outs = bg.assemble_batch(probs[:2], bg.GPUConfiguration(precision="fp64"), out="host")
    for (op, X, Y), z in zip(probs[:2], outs):
        assert rel(z, oracle.assemble(op, X, Y, qs)) < FP64_TOL


def test_abort_interrupts_a_running_assembly_and_the_handle_recovers():
    """bgb_abort from another thread makes a running bgb_assemble return BGB_ERR_ABORTED (the
    kernels poll a host-mapped flag between tiles and pairs; nothing traps); the next call on the
    same handle assembles normally."""
    import threading
    import time
    from beastgpu_gb300 import _lib
    from beastgpu_gb300.api import get_handle
    m = bg.icosphere(5)
    X = bg.raviartthomas(m)
    op = bg.Maxwell3D.singlelayer(wavenumber=8 * np.pi)
    cfg = bg.GPUConfiguration(precision="fp64")  # long enough (about a second) to be interrupted
    h = get_handle(0)
    result = {}

    def run():
        try:
            bg.assemble_gpu(op, X, X, cfg, out="device")
            result["rc"] = 0
        except _lib.BGBError as e:
            result["rc"] = e.code

    t = threading.Thread(target=run)
    t.start()
    while t.is_alive():
        _lib.load().bgb_abort(h.ptr)
        time.sleep(0.005)
    t.join()
    assert result["rc"] == -5  # BGB_ERR_ABORTED
    small = bg.icosphere(2)
    Y = bg.raviartthomas(small)
    ref = oracle.assemble(bg.Maxwell3D.singlelayer(wavenumber=K1), Y, Y, bg.QuadStrat())
    z = bg.assemble_gpu(bg.Maxwell3D.singlelayer(wavenumber=K1), Y, Y, bg.GPUConfiguration(precision="fp64"))
    assert rel(z, ref) < FP64_TOL


@pytest.mark.parametrize("name", ["efie", "hh", "hs"])
def test_distinct_test_and_trial_spaces(name):
    """Test and trial spaces on different meshes (a sphere against a nearby plate, in both orders):
    separate geometry, bounds and tile plans per side; rectangular matrices equal to the oracle's."""
    sphere = bg.icosphere(2)
    p = bg.plate(9, jitter=0.2, seed=5)
    v = p.vertices.copy()
    c = v[np.argmin(np.linalg.norm(v[:, :2] - 0.5, axis=1))].copy()
    v[:, :2] -= c[:2]  # a plate vertex 0.01 above the sphere's north pole: near pairs across the meshes
    v[:, 2] += 1.01
    plate = bg.Mesh(v, p.triangles)
    make = {"efie": lambda k: bg.Maxwell3D.singlelayer(wavenumber=k),
            "hh": lambda k: bg.Helmholtz3D.singlelayer(wavenumber=k),
            "hs": lambda k: bg.Helmholtz3D.hypersingular(wavenumber=k)}[name]
    space = bg.raviartthomas if name == "efie" else bg.lagrangec0d1
    op = make(2 * np.pi)
    for X, Y in ((space(sphere), space(plate)), (space(plate), space(sphere))):
        assert (oracle.classify_block(X, Y, op.wavenumber ** 2) == 4).any()
        ref = oracle.assemble(op, X, Y, bg.QuadStrat())
        assert ref.shape == (X.nfun, Y.nfun)
        z64 = bg.assemble_gpu(op, X, Y, bg.GPUConfiguration(precision="fp64"))
        zmx = bg.assemble_gpu(op, X, Y, bg.GPUConfiguration(precision="mixed"))
        assert rel(z64, ref) < FP64_TOL
        assert rel(zmx.astype(np.complex128), ref) < MIXED_TOL
        part = bg.assemble_gpu(op, X, Y, bg.GPUConfiguration(precision="fp64"), rows=(3, X.nfun - 5))
        np.testing.assert_array_equal(part, z64[3:X.nfun - 2])
        # a host output in column blocks of 7: the singular entries in groups by the trial side's blocks
        for prec, esz, want in (("fp64", 16, z64), ("mixed", 8, zmx)):
            Zb, st = bg.assemble_gpu(op, X, Y, bg.GPUConfiguration(precision=prec, total_GPU_budget=4 * 7 * X.nfun * esz),
                                     return_stats=True)
            assert st["out_blocks"] >= Y.nfun // 7
            np.testing.assert_array_equal(Zb, want)


def _nonfar_pairs(X, k2, rows_per_block=2048):
    """(tau, sigma) of every non-far triangle pair, from the GPU classifier in row blocks."""
    nt = X.mesh.nt
    taus, sigmas = [], []
    for t0 in range(0, nt, rows_per_block):
        c = bg.classify(X, X, k2, block=(t0, min(nt, t0 + rows_per_block), 0, nt))
        t, s = np.nonzero(c)
        taus.append(t + t0)
        sigmas.append(s)
    return np.concatenate(taus).astype(np.int32), np.concatenate(sigmas).astype(np.int32)


def _per_pair_rel(a, b):
    """Error of each local matrix relative to its own norm; pairs whose matrix vanishes up to rounding
    (the Maxwell double layer on coplanar pairs) are measured against 1e-6 of the largest pair's norm."""
    num = np.linalg.norm((a - b).reshape(len(a), -1), axis=1)
    den = np.linalg.norm(b.reshape(len(b), -1), axis=1)
    return num / np.maximum(np.maximum(den, 1e-6 * den.max()), 1e-300)


def test_c2_every_singular_entry_of_the_mixed_path_within_1e_12():
    """The EFIE at the benchmark size (icosphere level 5, k = 8 pi): every common-face, -edge and
    -vertex local matrix of the mixed path (double-float Sauter-Schwab) within 1e-12 of the plain
    FP64 kernel, pair by pair (not in aggregate)."""
    m = bg.icosphere(5)
    X = bg.raviartthomas(m)
    k = 2 * np.pi * 4
    op = bg.Maxwell3D.singlelayer(wavenumber=k)
    tau, sigma = _nonfar_pairs(X, k * k)
    L64, c64 = bg.local_matrices(op, X, X, tau, sigma)
    Lmx, cmx = bg.local_matrices(op, X, X, tau, sigma, precision="mixed")
    np.testing.assert_array_equal(c64, cmx)
    assert set(np.unique(c64)) == {1, 2, 3}
    assert tau.size == 20480 * (1 + 3) + int(np.count_nonzero(c64 == 1))  # CF + 3 CE per triangle + CV
    assert _per_pair_rel(Lmx, L64).max() < 1e-12


@pytest.mark.parametrize("name", ["hh", "mfie", "efie"])
def test_near_entries_are_fp64_in_the_mixed_path(name):
    """Near pairs (singularity extraction) run in FP64 in both precisions: identical local matrices;
    the mixed path's singular pairs within 1e-12 of FP64, pair by pair, on jittered and folded plates."""
    make, which = OPS[name]
    k = 4 * np.pi
    op = make(k)
    p = bg.two_plates(16, jitter=0.3, seed=1, gap=0.01)
    v = p.vertices.copy()
    half = v[:, 0] > 1.0  # fold the second plate up by 30 degrees about its edge x = 1.01
    v[half, 2] = (v[half, 0] - 1.01) * np.sin(np.pi / 6)
    v[half, 0] = 1.01 + (v[half, 0] - 1.01) * np.cos(np.pi / 6)
    # the Maxwell double layer vanishes on coplanar pairs: only the tilted plates give it values
    meshes = (p, bg.Mesh(v, p.triangles)) if name != "mfie" else (bg.Mesh(v, p.triangles),)
    for mesh in meshes:
        sp = (mesh, bg.raviartthomas(mesh), bg.lagrangec0d1(mesh))[which]
        tau, sigma = _nonfar_pairs(sp, k * k)
        L64, c = bg.local_matrices(op, sp, sp, tau, sigma)
        Lmx, _ = bg.local_matrices(op, sp, sp, tau, sigma, precision="mixed")
        near = c == 4
        assert near.sum() > 0
        np.testing.assert_array_equal(Lmx[near], L64[near])
        # each singular pair against its own norm; the Maxwell double layer's singular pairs here are all
        # coplanar, i.e. zero up to rounding, so they are measured against the largest local matrix
        num = np.linalg.norm((Lmx - L64)[~near].reshape(-1, 9), axis=1)
        den = np.linalg.norm(L64.reshape(-1, 9), axis=1)
        floor = den.max() if name == "mfie" else 1e-6 * den.max()
        tol = 1e-11 if name == "mfie" else 1e-12  # double-float rounding on entries that vanish analytically
        assert (num / np.maximum(den[~near], floor)).max() < tol


def test_double_float_fallback_for_large_wavenumbers():
    """k (edge_test + edge_trial) 2 >= 350 is beyond the double-float sine table: the mixed path's
    singular pairs fall back to the FP64 kernel (bit-identical local matrices) and the assembly
    still meets the mixed tolerance against the oracle."""
    m = bg.icosphere(1)
    X = bg.raviartthomas(m)
    e = np.linalg.norm(m.vertices[m.triangles[:, 0]] - m.vertices[m.triangles[:, 1]], axis=1).max()
    k = 400.0 / (4 * e)  # k (2 e) 2 = 400 > 350
    op = bg.Maxwell3D.singlelayer(wavenumber=k)
    tau, sigma = _nonfar_pairs(X, k * k)
    L64, _ = bg.local_matrices(op, X, X, tau, sigma)
    Lmx, _ = bg.local_matrices(op, X, X, tau, sigma, precision="mixed")
    np.testing.assert_array_equal(Lmx, L64)
    ref = oracle.assemble(op, X, X, bg.QuadStrat())
    assert rel(bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed")).astype(np.complex128), ref) < MIXED_TOL
    assert rel(bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64")), ref) < FP64_TOL


def test_mixed_far_pairs_hold_the_bound_without_compensated_sums():
    """The mixed far kernel accumulates its moments in plain FP32 (no Kahan compensation): its error
    comes from the phase and from cancellation in the bilinear forms, which the double-float phase
    base and the centroid-relative coordinates remove, not from summation.  Shown where summation
    and phase are hardest: (a) the 13 x 13 far rule, 169 point pairs summed per pair; (b) k times the
    meshes' diameter at 2.9e5, just inside the 3e5 range of the exact phase reduction (two small plates
    29 apart, k h ~ 1); beyond the range the call is refused."""
    m = bg.icosphere(2)
    X = bg.raviartthomas(m)
    op = bg.Maxwell3D.singlelayer(wavenumber=K1)
    c = oracle.classify_block(X, X, K1 * K1)
    t, s = np.nonzero(c == 0)
    sel = np.random.default_rng(5).choice(t.size, 400, replace=False)
    qs = bg.QuadStrat(far_test=13, far_trial=13)
    L64, _ = bg.local_matrices(op, X, X, t[sel], s[sel], quadstrat=qs, force_class=0)
    Lmx, _ = bg.local_matrices(op, X, X, t[sel], s[sel], quadstrat=qs, force_class=0, precision="mixed")
    assert _per_pair_rel(Lmx, L64).max() < 1e-5

    p = bg.plate(4, jitter=0.3, seed=4)
    v = p.vertices * 4e-4  # h = 1e-4
    w = v.copy()
    w[:, 0] += 29.0
    mesh = bg.Mesh(np.concatenate([v, w]), np.concatenate([p.triangles, p.triangles + p.nv]))
    Y = bg.raviartthomas(mesh)
    k = 1.0e4  # k * diameter = 2.9e5, k h = 1
    op = bg.Maxwell3D.singlelayer(wavenumber=k)
    tau = np.repeat(np.arange(p.nt), p.nt).astype(np.int32)
    sig = (p.nt + np.tile(np.arange(p.nt), p.nt)).astype(np.int32)
    L64, c64 = bg.local_matrices(op, Y, Y, tau, sig)
    Lmx, _ = bg.local_matrices(op, Y, Y, tau, sig, precision="mixed")
    assert np.all(c64 == 0)
    assert _per_pair_rel(Lmx, L64).max() < 1e-5
    with pytest.raises(Exception, match="3e5"):
        bg.local_matrices(bg.Maxwell3D.singlelayer(wavenumber=1.1e4), Y, Y, tau, sig, precision="mixed")
