"""Batches of uneven configurations in one evaluation: 256 independent
configurations of 16-432 atoms (bcc/fcc bulk, vacancy cells, (100)/(110)
slabs), the neighbour-count-sorted work queue, and replay of a captured
CUDA graph."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    from magace import structures as S
    confs = S.uneven_batch(64, seed=11)
    parts = [S.neighbor_data(c, 5.0) for c in confs]
    return parts, S.concat_neighbor_data(parts)


@pytest.fixture()
def gpu_lib(seeded_potential):
    from magace import lib
    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    lib.set_work_queue(False)
    yield lib
    lib.set_precision(0)
    lib.set_work_queue(False)


def test_batch_equals_separate_configurations(gpu_lib, batch):
    """Atoms are independent: the batched evaluation reproduces every
    configuration's own evaluation bit for bit (FP64)."""
    parts, nb = batch
    e, f, t, t0 = gpu_lib.acelib(nb)
    a = b = 0
    for p in parts[:12]:
        ep, fp, tp, t0p = gpu_lib.acelib(p)
        assert np.array_equal(e[a:a + p.natom], ep)
        assert np.array_equal(f[3 * b:3 * (b + p.nei)], fp)
        assert np.array_equal(t0[3 * a:3 * (a + p.natom)], t0p)
        a += p.natom
        b += p.nei


def test_batch_matches_oracle(gpu_lib, batch, oracle_seeded):
    parts, nb = batch
    e, f, t, t0 = gpu_lib.acelib(nb)
    eo, fo, to, t0o = oracle_seeded.acelib(nb, nthreads=8)
    assert rel_err(e, eo) < 1e-10 and rel_err(f, fo) < 1e-10
    assert rel_err(t, to) < 1e-10 and rel_err(t0, t0o) < 1e-10


@pytest.mark.parametrize("precision", [0, 1])
def test_work_queue_does_not_change_results(gpu_lib, batch, precision):
    """The sorted work queue changes which CTA evaluates which atom, not the
    result: bitwise in FP64; in split precision up to the order of the
    3-body kernel's shared-memory atomics."""
    _, nb = batch
    gpu_lib.set_precision(precision)
    ref = gpu_lib.acelib(nb)
    gpu_lib.set_work_queue(True)
    got = gpu_lib.acelib(nb)
    for x, y in zip(got, ref):
        if precision == 0:
            assert np.array_equal(x, y)
        else:
            assert rel_err(x, y) < 1e-6


@pytest.mark.parametrize("queue", [False, True])
def test_cuda_graph_replay(gpu_lib, batch, queue):
    """An evaluation captured into a CUDA graph replays on new inputs written
    into the same device arrays and gives the direct call's results."""
    import torch
    from magace import structures as S
    parts, nb = batch
    gpu_lib.set_precision(1)
    gpu_lib.set_work_queue(queue)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    ins = [T(nb.dlist), T(nb.elist), T(nb.dlist_mom), T(nb.elist_mom), T(nb.dlist_momi), T(nb.elist_momi)]
    outs = [torch.empty(nb.natom, dtype=torch.float64, device=dev), torch.empty(3 * nb.nei, dtype=torch.float64, device=dev),
            torch.empty(3 * nb.nei, dtype=torch.float64, device=dev), torch.empty(3 * nb.natom, dtype=torch.float64, device=dev)]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())

    def call():
        gpu_lib.compute_device(nb.natom, nb.nei, off.data_ptr(), *[x.data_ptr() for x in ins],
                               *[y.data_ptr() for y in outs], s.cuda_stream)

    with torch.cuda.stream(s):
        call()  # sizes the library's buffers before the capture
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        call()
    # new moments: magnitudes scaled, the same neighbour list
    nb2 = S.NeighborData(**{**nb.__dict__})
    nb2.dlist_mom = nb.dlist_mom * 0.97
    nb2.dlist_momi = nb.dlist_momi * 0.97
    ins[2].copy_(T(nb2.dlist_mom))
    ins[4].copy_(T(nb2.dlist_momi))
    g.replay()
    torch.cuda.synchronize()
    gpu_lib.device_status()
    ref = gpu_lib.acelib(nb2)
    for y, r in zip(outs, ref):
        assert rel_err(y.cpu().numpy(), r) < 1e-6


def test_side_by_side_density_kernels_match_one_stream(gpu_lib):
    """The split path runs its 2-/4-body and 3-body density kernels side by
    side on two streams; with kernel timing on, every kernel runs on one
    stream. On a 54,000-site system (about 1,700 blocks of 32 atoms, many
    waves of both kernels, so that either may run far ahead of the other)
    both give the same results up to the 3-body kernel's atomic order."""
    import torch
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_vacancies(ncell=30, seed=3), 5.0)
    gpu_lib.set_precision(1)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    ins = [T(nb.dlist), T(nb.elist), T(nb.dlist_mom), T(nb.elist_mom), T(nb.dlist_momi), T(nb.elist_momi)]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())

    def run():
        outs = [torch.empty(n, dtype=torch.float64, device=dev)
                for n in (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)]
        gpu_lib.compute_device(nb.natom, nb.nei, off.data_ptr(), *[x.data_ptr() for x in ins],
                               *[y.data_ptr() for y in outs], s.cuda_stream)
        s.synchronize()
        gpu_lib.device_status()
        return [y.cpu().numpy() for y in outs]

    try:
        gpu_lib.set_kernel_timing(False)
        side = [run() for _ in range(3)]
        gpu_lib.set_kernel_timing(True)
        one = run()
    finally:
        gpu_lib.set_kernel_timing(False)
    for got in side:
        for x, y in zip(got, one):
            assert rel_err(x, y) < 1e-6
