"""Caller-provided output buffers are checked before any device work: the element type must be
the output's, the storage contiguous and large enough, and on the output's side (host memory for
a host output, a CUDA tensor for a device output).  A mismatch raises ValueError instead of
letting the library write past the buffer.  No GPU is needed: the checks run before the handle."""
import numpy as np
import pytest

import beastgpu_gb300 as bg


@pytest.fixture(scope="module")
def small():
    X = bg.raviartthomas(bg.icosphere(1))
    return X, bg.Maxwell3D.singlelayer(wavenumber=2.0)


def test_host_buffer_of_the_wrong_type_or_size_is_refused(small):
    X, op = small
    n = X.nfun
    fp64 = bg.GPUConfiguration(precision="fp64")
    with pytest.raises(ValueError, match="complex128"):
        bg.assemble_gpu(op, X, X, fp64, out_buffer=np.empty((n, n), np.complex64, order="F"))
    with pytest.raises(ValueError, match="elements"):
        bg.assemble_gpu(op, X, X, fp64, out_buffer=np.empty((n, n - 1), np.complex128, order="F"))
    with pytest.raises(ValueError, match="elements"):  # a row window needs nrows x ncols
        bg.assemble_gpu(op, X, X, fp64, rows=(0, 10), out_buffer=np.empty((9, n), np.complex128, order="F"))
    with pytest.raises(ValueError, match="contiguous"):
        bg.assemble_gpu(op, X, X, fp64, out_buffer=np.empty((2 * n, n), np.complex128, order="F")[::2])
    ro = np.empty((n, n), np.complex128, order="F")
    ro.flags.writeable = False
    with pytest.raises(ValueError, match="writeable"):
        bg.assemble_gpu(op, X, X, fp64, out_buffer=ro)
    with pytest.raises(ValueError, match="complex64"):  # mixed: complex64 unless dtype says otherwise
        bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed"), out_buffer=np.empty((n, n), np.complex128))


def test_device_output_needs_a_cuda_tensor_and_torch_types_are_checked(small):
    torch = pytest.importorskip("torch")
    X, op = small
    n = X.nfun
    cfg = bg.GPUConfiguration(precision="fp64")
    with pytest.raises(ValueError, match="torch CUDA tensor"):
        bg.assemble_gpu(op, X, X, cfg, out="device", out_buffer=np.empty((n, n), np.complex128))
    with pytest.raises(ValueError, match="goes to cuda"):
        bg.assemble_gpu(op, X, X, cfg, out="device", out_buffer=torch.empty((n, n), dtype=torch.complex128))
    with pytest.raises(ValueError, match="dtype"):
        bg.assemble_gpu(op, X, X, cfg, out_buffer=torch.empty((n, n), dtype=torch.complex64))
    with pytest.raises(ValueError, match="contiguous"):
        bg.assemble_gpu(op, X, X, cfg, out_buffer=torch.empty((n, 2 * n), dtype=torch.complex128)[:, ::2])
    with pytest.raises(ValueError, match="out must be"):
        bg.assemble_gpu(op, X, X, cfg, out="disk")


def test_curve_path_checks_its_buffers_too():
    X = bg.curve_lagrangec0d1(bg.circle(64))
    op = bg.Helmholtz2D.singlelayer(wavenumber=3.0)
    n = X.nfun
    with pytest.raises(ValueError, match="complex128"):
        bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"), out_buffer=np.empty((n, n), np.complex64))
    with pytest.raises(ValueError, match="elements"):
        bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="fp64"), out_buffer=np.empty(n, np.complex128))
