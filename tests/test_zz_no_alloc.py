"""The allocation-free classification entry point, called through the C ABI.

Some callers cannot let a library allocate device memory: a Julia or PyTorch process whose
memory pool already holds the GPU, or an embedding that only allows its own allocator.
bgb_classify_csr_noalloc serves them with scratch in a fixed device array of the library.
This test gives it device inputs and outputs (allocated here, by the caller) and checks its
CSR against the classes of the existing entry point bgb_classify_block, on two calls in a
row (the second call reuses the array the first one left behind).  Collected last, so that a
run stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

import beastgpu_gb300 as bg
from beastgpu_gb300 import _lib


def csr_from_dense(cls):
    offsets = np.zeros(cls.shape[0] + 1, dtype=np.int64)
    tau, sigma = np.nonzero(cls)
    np.add.at(offsets, tau + 1, 1)
    return np.cumsum(offsets), tau.astype(np.int32), sigma.astype(np.int32), cls[tau, sigma].astype(np.int8)


def call_noalloc(test_mesh, trial_mesh, k2, capacity):
    import torch
    dev = torch.device("cuda:0")
    vt = torch.as_tensor(test_mesh.vertices, device=dev)
    tt = torch.as_tensor(test_mesh.triangles, device=dev)
    vb = torch.as_tensor(trial_mesh.vertices, device=dev)
    tb = torch.as_tensor(trial_mesh.triangles, device=dev)
    off = torch.empty(test_mesh.nt + 1, dtype=torch.int64, device=dev)
    tau = torch.empty(max(1, capacity), dtype=torch.int32, device=dev)
    sig = torch.empty(max(1, capacity), dtype=torch.int32, device=dev)
    cls = torch.empty(max(1, capacity), dtype=torch.int8, device=dev)
    total = C.c_int64(-1)
    stream = torch.cuda.current_stream(dev)
    rc = _lib.load().bgb_classify_csr_noalloc(
        C.c_void_p(vt.data_ptr()), C.c_void_p(tt.data_ptr()), test_mesh.nv, test_mesh.nt,
        C.c_void_p(vb.data_ptr()), C.c_void_p(tb.data_ptr()), trial_mesh.nv, trial_mesh.nt, float(k2),
        C.c_void_p(off.data_ptr()), C.c_void_p(tau.data_ptr()), C.c_void_p(sig.data_ptr()),
        C.c_void_p(cls.data_ptr()), capacity, C.byref(total), C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    n = total.value
    return rc, n, off.cpu().numpy(), tau[:n].cpu().numpy(), sig[:n].cpu().numpy(), cls[:n].cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_classify_block_on_two_calls():
    cases = []
    m = bg.icosphere(3)
    cases.append((bg.raviartthomas(m), (2 * np.pi) ** 2))
    p = bg.two_plates(16, jitter=0.3, seed=1, gap=0.01)
    cases.append((bg.raviartthomas(p), (4 * np.pi) ** 2))
    for space, k2 in cases:  # two calls in a row on the shared scratch array
        ref = bg.classify(space, space, k2)  # existing entry point (bgb_classify_block)
        r_off, r_tau, r_sig, r_cls = csr_from_dense(ref)
        rc, n, off, tau, sig, cls = call_noalloc(space.mesh, space.mesh, k2, capacity=r_tau.size + 7)
        assert rc == 0, _lib.load().bgb_last_error()
        assert n == r_tau.size
        np.testing.assert_array_equal(off, r_off)
        np.testing.assert_array_equal(tau, r_tau)
        np.testing.assert_array_equal(sig, r_sig)
        np.testing.assert_array_equal(cls, r_cls)


@pytest.mark.gpu
def test_noalloc_rejects_oversize_and_short_capacity():
    lib = _lib.load()
    total = C.c_int64(0)
    # beyond the fixed scratch: rejected before any device work (pointers are never touched)
    rc = lib.bgb_classify_csr_noalloc(None, None, 3, 200000, None, None, 3, 200000, 1.0, None, None, None, None,
                                      0, C.byref(total), None)
    assert rc == -6
    assert b"scratch" in lib.bgb_last_error()
    m = bg.icosphere(2)
    rc, n, off, *_ = call_noalloc(m, m, 1.0, capacity=10)
    assert rc == -6 and n > 10 and off[-1] == n


@pytest.mark.gpu
def test_noalloc_reports_a_vertex_index_outside_the_mesh():
    """A triangle that names vertex nv is flagged on the device, never read; the call fails
    with BGB_ERR_INVALID and says so, and the next valid call on the same scratch succeeds."""
    m = bg.icosphere(2)
    bad = bg.Mesh(m.vertices.copy(), m.triangles.copy())
    bad.triangles[17, 1] = m.nv  # one past the last vertex
    rc, *_ = call_noalloc(bad, m, 1.0, capacity=16384)
    assert rc == -1
    assert b"vertex index" in _lib.load().bgb_last_error()
    ref = bg.classify(bg.raviartthomas(m), bg.raviartthomas(m), 1.0)
    rc, n, off, tau, sig, cls = call_noalloc(m, m, 1.0, capacity=int(np.count_nonzero(ref)) + 5)
    assert rc == 0 and n == np.count_nonzero(ref)
    np.testing.assert_array_equal(cls, ref[tau, sig])


def test_noalloc_rejects_triangles_without_vertices():
    """nt > 0 with nv == 0 is refused on the host, before any CUDA call (runs without a GPU)."""
    lib = _lib.load()
    total = C.c_int64(-1)
    rc = lib.bgb_classify_csr_noalloc(None, None, 0, 5, None, None, 3, 1, 1.0, None, None, None, None, 0,
                                      C.byref(total), None)
    assert rc == -1 and total.value == 0
    assert b"nv == 0" in lib.bgb_last_error()
    rc = lib.bgb_classify_csr_noalloc(None, None, 3, 1, None, None, 0, 4, 1.0, None, None, None, None, 0,
                                      C.byref(total), None)
    assert rc == -1
