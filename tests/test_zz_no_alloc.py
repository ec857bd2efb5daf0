"""GPU test of ace_compute_device_noalloc, the entry point for callers that
cannot allocate device memory while they evaluate. It is called through the
C ABI twice in a row and must reproduce ace_compute_device (the regular entry
point, which uses library-allocated scratch): in FP64 within the parity
tolerance of the other tests, in split precision within 1e-6. The file sorts last so that a stop-at-first-failure run
has executed every other test before it; it also passes alone in a fresh
process, because it places the potential's tables on the device itself."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_compute_device(seeded_potential, precision):
    """FP64 at the parity tolerance; split precision within 1e-6 (the 3-body
    kernel adds gradients with shared-memory atomics, so two split runs agree
    to FP32 rounding, not bit for bit)."""
    import torch
    from magace import lib, structures as S

    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(precision)
    tol = TOL if precision == 0 else 1e-6
    so = lib.load()
    nb = S.neighbor_data(S.bcc_fe_128(3), 5.0)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    ins = [T(a) for a in (nb.dlist, nb.elist, nb.dlist_mom, nb.elist_mom, nb.dlist_momi, nb.elist_momi)]

    def outputs():
        return [torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
                for n in (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)]

    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    ptr = lambda ts: [t.data_ptr() for t in ts]

    # regular entry point (library-allocated scratch); also places the tables
    ref = outputs()
    st = so.ace_compute_device(nb.natom, nb.nei, off.data_ptr(), *ptr(ins), *ptr(ref), stream.cuda_stream)
    assert st == 0, so.ace_last_error_message()
    stream.synchronize()
    assert so.ace_device_status() == 0
    ref = [t.cpu().numpy() for t in ref]

    for _ in range(2):  # two calls in a row share the same scratch
        got = outputs()
        st = so.ace_compute_device_noalloc(nb.natom, nb.nei, off.data_ptr(), *ptr(ins), *ptr(got),
                                           ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, so.ace_last_error_message()
        got = [t.cpu().numpy() for t in got]
        for g, r in zip(got, ref):
            assert np.all(np.isfinite(g))
            assert _rel(g, r) <= tol
    lib.set_precision(0)


# limits of the 64 MiB scratch for the seeded Fe-layout potential on a
# 152-SM GB300 (FP64, split precision)
DOCUMENTED_LIMIT = {0: 1816, 1: 3305}


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_takes_its_limit_and_refuses_one_more(seeded_potential, precision):
    """The refusal message states the largest atom count the scratch holds;
    a call with exactly that many atoms runs and matches ace_compute_device,
    one more atom is refused with MAGACE_ERR_ARGS."""
    import re

    import torch
    from magace import lib, structures as S

    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(precision)
    so = lib.load()
    # a zero-atom regular call places the tables on the device
    assert so.ace_compute_device(0, 0, *[None] * 12) == 0
    st = so.ace_compute_device_noalloc(100000, 0, *[None] * 12)
    assert st == 7  # MAGACE_ERR_ARGS
    msg = so.ace_last_error_message().decode()
    assert "scratch" in msg
    limit = int(re.search(r"at most (\d+) atoms", msg).group(1))
    if torch.cuda.get_device_properties(0).multi_processor_count == 152:
        assert limit == DOCUMENTED_LIMIT[precision]
    assert so.ace_compute_device_noalloc(limit + 1, 0, *[None] * 12) == 7

    # exactly `limit` atoms: the first atoms of a larger bcc system
    full = S.neighbor_data(S.bcc_fe_vacancies(ncell=12, seed=4), 5.0)
    assert full.natom > limit
    counts = (full.nstop - full.nstart + 1)[:limit]
    nei = int(counts.sum())
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(counts)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    ins = [T(full.dlist[:nei]), T(full.elist[:3 * nei]), T(full.dlist_mom[:nei]), T(full.elist_mom[:3 * nei]),
           T(full.dlist_momi[:limit]), T(full.elist_momi[:3 * limit])]
    outs = lambda: [torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
                    for n in (limit, 3 * nei, 3 * nei, 3 * limit)]
    ptr = lambda ts: [t.data_ptr() for t in ts]
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    ref = outs()
    assert so.ace_compute_device(limit, nei, off.data_ptr(), *ptr(ins), *ptr(ref), stream.cuda_stream) == 0
    stream.synchronize()
    assert so.ace_device_status() == 0
    got = outs()
    st = so.ace_compute_device_noalloc(limit, nei, off.data_ptr(), *ptr(ins), *ptr(got),
                                       ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, so.ace_last_error_message()
    tol = TOL if precision == 0 else 1e-6
    for g, r in zip(got, ref):
        g, r = g.cpu().numpy(), r.cpu().numpy()
        assert np.all(np.isfinite(g))
        assert _rel(g, r) <= tol
    lib.set_precision(0)


def test_noalloc_refuses_a_stream_capture(seeded_potential):
    """The call is synchronous, so on a stream that is being captured into a
    CUDA graph it returns MAGACE_ERR_ARGS before any device work; the
    caller's capture stays valid and the library stays usable."""
    import torch
    from magace import lib, structures as S

    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    so = lib.load()
    nb = S.neighbor_data(S.bcc_fe_54(1), 5.0)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    ins = [T(a) for a in (nb.dlist, nb.elist, nb.dlist_mom, nb.elist_mom, nb.dlist_momi, nb.elist_momi)]
    outs = [torch.zeros(n, dtype=torch.float64, device=dev) for n in (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)]
    ptr = lambda ts: [t.data_ptr() for t in ts]
    # tables on the device first (an uncaptured call)
    assert so.ace_compute_device(0, 0, off.data_ptr(), *ptr(ins), *ptr(outs), None) == 0
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    marker = torch.zeros(1, device=dev)
    with torch.cuda.graph(graph, stream=stream):
        code = so.ace_compute_device_noalloc(nb.natom, nb.nei, off.data_ptr(), *ptr(ins), *ptr(outs),
                                             stream.cuda_stream)
        marker += 1.0
    assert code == 7, so.ace_last_error_message()  # MAGACE_ERR_ARGS
    assert b"stream capture" in so.ace_last_error_message()
    graph.replay()
    torch.cuda.synchronize()
    assert float(marker.item()) == 1.0
    # still usable outside the capture
    assert so.ace_compute_device_noalloc(nb.natom, nb.nei, off.data_ptr(), *ptr(ins), *ptr(outs), None) == 0
