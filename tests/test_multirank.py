"""The multi-process path with gloo, world size 2.

Each rank takes its row window of one matrix (beastgpu_gb300.row_shard) and the ranks check that
the windows tile the matrix exactly and agree with a single-process assembly.  On the CPU the FP64
oracle stands in for each rank's GPU, and the bench's barrier and max-over-ranks reduction run
under the same process group; with a GPU both ranks drive libbeastgb's row windows (on the one
GPU of this machine: independent launches, no kernel waits on another rank).
"""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    import beastgpu_gb300 as bg
    import oracle
    r, w, local = bench.dist_init(world)
    assert (r, w) == (rank, world) and dist.get_backend() == "gloo"
    m = bg.icosphere(2)
    X = bg.raviartthomas(m)
    op = bg.Maxwell3D.singlelayer(wavenumber=2 * np.pi)
    row0, nrows = bg.row_shard(X.nfun, rank, world)
    Z = oracle.assemble_rows(op, X, X, bg.QuadStrat(), np.arange(row0, row0 + nrows, dtype=np.int32), nthreads=1)
    bench.barrier(world)
    t = torch.from_numpy(np.ascontiguousarray(np.stack([Z.real, Z.imag], -1))).reshape(-1)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([t.numel()], dtype=torch.int64))
    bufs = [torch.zeros(int(s.item()), dtype=t.dtype) for s in sizes]
    dist.all_gather(bufs, t)
    slowest = bench.max_over_ranks(float(rank + 1), world, local)
    if rank == 0:
        parts = [b.reshape(-1, X.nfun, 2).numpy() for b in bufs]
        full = np.concatenate([p[..., 0] + 1j * p[..., 1] for p in parts])
        np.save(os.path.join(out_dir, "gathered.npy"), full)
        np.save(os.path.join(out_dir, "slowest.npy"), np.array(slowest))
    dist.destroy_process_group()


def test_row_windows_tile_the_matrix_on_two_gloo_ranks(tmp_path):
    import beastgpu_gb300 as bg
    import oracle
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    gathered = np.load(tmp_path / "gathered.npy")
    m = bg.icosphere(2)
    X = bg.raviartthomas(m)
    full = oracle.assemble(bg.Maxwell3D.singlelayer(wavenumber=2 * np.pi), X, X, bg.QuadStrat(), nthreads=1)
    np.testing.assert_array_equal(gathered, full)
    assert float(np.load(tmp_path / "slowest.npy")) == 2.0


@pytest.mark.parametrize("n,world", [(480, 2), (7, 3), (1, 4), (30720, 8)])
def test_row_shard_partitions(n, world):
    import beastgpu_gb300 as bg
    spans = [bg.row_shard(n, r, world) for r in range(world)]
    assert spans[0][0] == 0 and sum(s[1] for s in spans) == n
    for (a0, an), (b0, _) in zip(spans, spans[1:]):
        assert a0 + an == b0
    assert max(s[1] for s in spans) - min(s[1] for s in spans) <= 1


def _rank_main_gpu(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import beastgpu_gb300 as bg
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = bg.icosphere(3)
    X = bg.raviartthomas(m)
    op = bg.Maxwell3D.singlelayer(wavenumber=2 * np.pi * 2)
    row0, nrows = bg.row_shard(X.nfun, rank, world)
    out = {}
    for prec in ("fp64", "mixed"):
        Z = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision=prec), rows=(row0, nrows))
        t = torch.from_numpy(np.ascontiguousarray(np.stack([Z.real, Z.imag], -1)).astype(np.float64)).reshape(-1)
        sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(sizes, torch.tensor([t.numel()], dtype=torch.int64))
        bufs = [torch.zeros(int(s.item()), dtype=t.dtype) for s in sizes]
        dist.all_gather(bufs, t)
        out[prec] = bufs
    if rank == 0:
        for prec, bufs in out.items():
            parts = [b.reshape(-1, X.nfun, 2).numpy() for b in bufs]
            np.save(os.path.join(out_dir, f"gathered_{prec}.npy"),
                    np.concatenate([p[..., 0] + 1j * p[..., 1] for p in parts]))
    dist.destroy_process_group()


@pytest.mark.gpu
def test_row_windows_through_the_library_on_two_gloo_ranks(tmp_path):
    """Two ranks assemble their row windows of one EFIE matrix with libbeastgb: the gathered windows
    equal the single-process matrix bit for bit, in both precisions (results do not depend on the
    tiling, which the windows change)."""
    import beastgpu_gb300 as bg
    world = 2
    mp.start_processes(_rank_main_gpu, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    m = bg.icosphere(3)
    X = bg.raviartthomas(m)
    op = bg.Maxwell3D.singlelayer(wavenumber=2 * np.pi * 2)
    for prec in ("fp64", "mixed"):
        full = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision=prec))
        gathered = np.load(tmp_path / f"gathered_{prec}.npy")
        np.testing.assert_array_equal(gathered, full.astype(np.complex128))
