"""GPU parity: the FP64 drop-in path (acelib_ through the C ABI) against the
CPU oracle on identical inputs, at 1e-10 relative (norm-relative for the
per-bond vectors). Edge cases follow the reference's behaviour: neighbours
beyond the cutoff contribute zero (src/radial.F90:77-83), moments inside the
first magnetic bin use the constant branch (src/radial.F90:135-139), and
inputs that stop the reference are reported as errors with NaN outputs.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10


@pytest.fixture()
def gpu_lib(seeded_potential):
    from magace import lib
    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    return lib


def _compare(lib, orc, nb, tol=TOL_FP64):
    e, f, t, t0 = lib.acelib(nb)
    eo, fo, to, t0o = orc.acelib(nb)
    assert rel_err(e, eo) <= tol, ("energy", rel_err(e, eo))
    assert rel_err(f, fo) <= tol, ("flist", rel_err(f, fo))
    assert rel_err(t, to) <= tol, ("tlist", rel_err(t, to))
    assert rel_err(t0, t0o) <= tol, ("tlist0", rel_err(t0, t0o))
    return e, f, t, t0


def test_bcc128_fp64_parity(gpu_lib, oracle_seeded):
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_128(1), 5.0)
    _compare(gpu_lib, oracle_seeded, nb)


def test_notebook_cell_fp64_parity(gpu_lib, oracle_seeded):
    from magace import structures as S
    nb = S.neighbor_data(S.notebook_cell(), 5.0)
    e, *_ = _compare(gpu_lib, oracle_seeded, nb)
    assert abs(e[0] - e[1]) < 1e-12  # the two atoms are equivalent


def test_ragged_slab_with_isolated_atom(gpu_lib, oracle_seeded):
    """(100) slab (non-periodic z), vacancies, and one atom far from all
    others: neighbour counts from 0 to ~58."""
    from magace import structures as S
    rng = np.random.default_rng(7)
    pos, cell = S.bcc_cubic(3, 3, 3, 2.83)
    pos = pos + rng.normal(0, 0.08, pos.shape)
    keep = rng.random(len(pos)) > 0.1
    pos = pos[keep]
    pos = np.vstack([pos, [[4.0, 4.0, 40.0]]])
    n = len(pos)
    st = S.Structure(pos, cell, (True, True, False), rng.uniform(1.5, 2.6, n), S.random_unit(rng, n))
    nb = S.neighbor_data(st, 5.0)
    counts = nb.nstop - nb.nstart + 1
    assert counts.min() == 0 and counts.max() > 30
    _compare(gpu_lib, oracle_seeded, nb)


def test_noncontiguous_ranges(gpu_lib, oracle_seeded):
    """Bond ranges given in a different order than the atoms (the acelib_
    gather path); the outputs stay packed atom by atom."""
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_54(3), 5.0)
    counts = nb.nstop - nb.nstart + 1
    order = np.arange(nb.natom)[::-1]
    # rebuild the bond arrays with atoms' blocks stored in reverse order
    blocks = [np.arange(nb.nstart[i] - 1, nb.nstop[i]) for i in order]
    perm = np.concatenate(blocks)
    new_start = np.zeros(nb.natom, np.int32)
    pos = 1
    for i in order:
        new_start[i] = pos
        pos += counts[i]
    nb2 = S.NeighborData(
        natom=nb.natom, nall=nb.nall, nei=nb.nei, nlist=nb.nlist[perm], occ=nb.occ,
        occlist=nb.occlist[perm], nstart=new_start, nstop=(new_start + counts - 1).astype(np.int32),
        dlist=nb.dlist[perm].copy(), elist=nb.elist.reshape(-1, 3)[perm].reshape(-1).copy(),
        dlist_momi=nb.dlist_momi, elist_momi=nb.elist_momi, dlist_mom=nb.dlist_mom[perm].copy(),
        elist_mom=nb.elist_mom.reshape(-1, 3)[perm].reshape(-1).copy())
    e, f, t, t0 = gpu_lib.acelib(nb)
    e2, f2, t2, t02 = gpu_lib.acelib(nb2)
    # packed outputs follow atom order, so they match the contiguous call
    assert rel_err(e2, e) <= 1e-14
    assert rel_err(f2, f) <= 1e-14 and rel_err(t2, t) <= 1e-14 and rel_err(t02, t0) <= 1e-14
    _compare(gpu_lib, oracle_seeded, nb2)


def test_neighbours_beyond_cutoff_and_small_moments(gpu_lib, oracle_seeded):
    """A LAMMPS-style list with skin (bonds up to 6.5 A) and some moments
    inside the first magnetic LUT bin (|m| < 4e-4 mu_B)."""
    from magace import structures as S
    st = S.bcc_fe_54(11)
    st.mag[:5] = np.array([1e-5, 2e-4, 3.9e-4, 1e-6, 2.5e-4])
    nb = S.neighbor_data(st, 6.5)
    assert nb.dlist.max() > 5.0
    _compare(gpu_lib, oracle_seeded, nb)


def test_repeat_is_bitwise_deterministic(gpu_lib):
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_128(4), 5.0)
    a = gpu_lib.acelib(nb)
    b = gpu_lib.acelib(nb)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_empty_call(gpu_lib):
    from magace import structures as S
    nb = S.NeighborData(natom=0, nall=0, nei=0, nlist=np.zeros(0, np.int32), occ=np.zeros(0, np.int32),
                        occlist=np.zeros(0, np.int32), nstart=np.zeros(0, np.int32),
                        nstop=np.zeros(0, np.int32), dlist=np.zeros(0), elist=np.zeros(0),
                        dlist_momi=np.zeros(0), elist_momi=np.zeros(0), dlist_mom=np.zeros(0),
                        elist_mom=np.zeros(0))
    e, f, t, t0 = gpu_lib.acelib(nb)
    assert e.size == 0 and f.size == 0


def test_small_distance_is_an_error(gpu_lib):
    """r below one LUT bin stops the reference (src/radial.F90:71-75); here
    acelib_ records MAGACE_ERR_SMALL_R and writes NaN."""
    from magace import structures as S
    from magace.lib import MagAceError
    nb = S.neighbor_data(S.bcc_fe_54(5), 5.0)
    nb.dlist = nb.dlist.copy()
    nb.dlist[3] = 1e-4
    with pytest.raises(MagAceError) as ei:
        gpu_lib.acelib(nb)
    assert ei.value.code == 4
    # the library stays usable afterwards
    nb2 = S.neighbor_data(S.bcc_fe_54(5), 5.0)
    e, *_ = gpu_lib.acelib(nb2)
    assert np.all(np.isfinite(e))


@pytest.mark.parametrize("mode", ["direct", "copy"])
def test_neighbour_element_other_than_one_is_an_error(gpu_lib, monkeypatch, mode):
    """The C entry serves one element (src/ace.F90:46-49): a neighbour element
    index other than 1 is refused with MAGACE_ERR_ARGS and NaN outputs in
    every host-access mode (the check runs while the GPU evaluates), and the
    library stays usable."""
    from magace import structures as S
    from magace.lib import MagAceError
    monkeypatch.setenv("MAGACE_HOST_ACCESS", mode)
    nb = S.neighbor_data(S.bcc_fe_54(5), 5.0)
    nb.occlist = nb.occlist.copy()
    nb.occlist[7] = 2
    out = (np.zeros(nb.natom), np.zeros(3 * nb.nei), np.zeros(3 * nb.nei), np.zeros(3 * nb.natom))
    with pytest.raises(MagAceError) as ei:
        gpu_lib.acelib(nb, out)
    assert ei.value.code == 7
    assert all(np.isnan(x).all() for x in out)
    nb.occlist[7] = 1
    e, *_ = gpu_lib.acelib(nb)
    assert np.all(np.isfinite(e))


def test_moment_beyond_cutoff_is_an_error(gpu_lib):
    """|m| >= the magnetic cutoff overruns the reference's table
    (src/radial.F90:126-157 has no upper check); here it is an error."""
    from magace import structures as S
    from magace.lib import MagAceError
    st = S.bcc_fe_54(6)
    st.mag[0] = 4.5
    nb = S.neighbor_data(st, 5.0)
    with pytest.raises(MagAceError) as ei:
        gpu_lib.acelib(nb)
    assert ei.value.code == 5


def test_device_api_matches_acelib(gpu_lib):
    """ace_compute_device on torch-owned device arrays gives the same numbers
    as the host-array drop-in call."""
    import torch
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_128(2), 5.0)
    e, f, t, t0 = gpu_lib.acelib(nb)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    r, ee, mj, mhj, mi, mhi = map(T, (nb.dlist, nb.elist, nb.dlist_mom, nb.elist_mom, nb.dlist_momi,
                                      nb.elist_momi))
    en = torch.empty(nb.natom, dtype=torch.float64, device=dev)
    fij = torch.empty(3 * nb.nei, dtype=torch.float64, device=dev)
    tij = torch.empty_like(fij)
    ti0 = torch.empty(3 * nb.natom, dtype=torch.float64, device=dev)
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    stream = st.cuda_stream
    gpu_lib.compute_device(nb.natom, nb.nei, off.data_ptr(), r.data_ptr(), ee.data_ptr(), mj.data_ptr(),
                           mhj.data_ptr(), mi.data_ptr(), mhi.data_ptr(), en.data_ptr(), fij.data_ptr(),
                           tij.data_ptr(), ti0.data_ptr(), stream)
    st.synchronize()
    gpu_lib.device_status()
    assert np.array_equal(en.cpu().numpy(), e)
    assert np.array_equal(fij.cpu().numpy(), f)
    assert np.array_equal(tij.cpu().numpy(), t)
    assert np.array_equal(ti0.cpu().numpy(), t0)
    # A basis, the 2-/4-body and the dense 3-body density kernels,
    # k_finish_fe and forces (the Fe layout's specialised kernels)
    assert gpu_lib.last_launch_count() == 5


def _ragged_slab():
    from magace import structures as S
    rng = np.random.default_rng(7)
    pos, cell = S.bcc_cubic(3, 3, 3, 2.83)
    pos = pos + rng.normal(0, 0.08, pos.shape)
    pos = pos[rng.random(len(pos)) > 0.1]
    pos = np.vstack([pos, [[4.0, 4.0, 40.0]]])
    n = len(pos)
    return S.Structure(pos, cell, (True, True, False), rng.uniform(1.5, 2.6, n), S.random_unit(rng, n))


@pytest.mark.parametrize("case", ["bcc128", "bcc54", "slab"])
def test_split_precision_accuracy(gpu_lib, oracle_seeded, case):
    """The split path (FP32 features, products and weights; FP64 density,
    energy and embedding) stays within 1 meV/atom and 10 meV/A of the FP64
    oracle; atom counts that are not multiples of the 32-atom tiles of the
    3-body kernel and an atom without neighbours included. The norm-relative
    bounds (1e-5) are far below those limits and catch a wrong sign or a
    missing term in any one part of the basis."""
    from magace import structures as S
    st = {"bcc128": lambda: S.bcc_fe_128(1), "bcc54": lambda: S.bcc_fe_54(2), "slab": _ragged_slab}[case]()
    nb = S.neighbor_data(st, 5.0)
    gpu_lib.set_precision(1)
    try:
        e, f, t, t0 = gpu_lib.acelib(nb)
    finally:
        gpu_lib.set_precision(0)
    eo, fo, to, t0o = oracle_seeded.acelib(nb)
    print(case, "max |dE| meV/atom", np.abs(e - eo).max() * 1e3, "max |dF| meV/A", np.abs(f - fo).max() * 1e3,
          "rel", rel_err(e, eo), rel_err(f, fo), rel_err(t, to), rel_err(t0, t0o))
    assert np.abs(e - eo).max() * 1e3 < 1.0
    assert np.abs(f - fo).max() * 1e3 < 10.0
    assert np.abs(t - to).max() * 1e3 < 10.0 and np.abs(t0 - t0o).max() * 1e3 < 10.0
    for got, ref in ((e, eo), (f, fo), (t, to), (t0, t0o)):
        assert rel_err(got, ref) < 1e-5


@pytest.mark.parametrize("mode", ["copy", "pinned", "direct"])
def test_host_access_modes_agree(gpu_lib, monkeypatch, mode):
    """acelib_ gives bit-identical results whether it copies pageable memory,
    stages through pinned memory, or lets the kernels read and write the
    caller's arrays directly (where the GPU uses the host page tables)."""
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_128(5), 5.0)
    monkeypatch.setenv("MAGACE_HOST_ACCESS", "copy")
    ref = gpu_lib.acelib(nb)
    monkeypatch.setenv("MAGACE_HOST_ACCESS", mode)
    got = gpu_lib.acelib(nb)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", [0, 1])
def test_direct_mode_outputs_at_any_alignment(gpu_lib, monkeypatch, precision):
    """acelib_ writing the caller's arrays directly stores each bond tile's
    outputs as 16-byte lines: output arrays that start 8 bytes past a 16-byte
    boundary, atoms of two 64-bond tiles and an atom without bonds give the
    same results as plain copies, bit for bit."""
    from magace import structures as S
    st = _ragged_slab()
    st = S.Structure(np.vstack([st.positions, [[1.0, 1.0, 90.0]]]), st.cell, st.pbc, np.append(st.mag, 2.0),
                     np.vstack([st.mhat, [[0.0, 0.0, 1.0]]]))
    nb = S.neighbor_data(st, 8.4)
    gpu_lib.set_precision(precision)
    try:
        monkeypatch.setenv("MAGACE_HOST_ACCESS", "copy")
        ref = gpu_lib.acelib(nb)
        monkeypatch.setenv("MAGACE_HOST_ACCESS", "direct")
        for shift in (0, 1):
            bufs = [np.full(n + 1, 7.0) for n in (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)]
            out = tuple(b[shift:shift + n] for b, n in zip(bufs, (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)))
            got = gpu_lib.acelib(nb, out)
            for x, y in zip(got, ref):
                if precision == 0:
                    assert np.array_equal(x, y)
                else:
                    assert rel_err(x, y) < 1e-6
            for b, n in zip(bufs, (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)):
                # nothing outside the caller's arrays is written
                assert b[n if shift == 0 else 0] == 7.0
    finally:
        gpu_lib.set_precision(0)


def test_autotuner_keeps_results(gpu_lib, oracle_seeded):
    """The autotuner times every variant of the split kernels and keeps the
    fastest of each; the split results stay within the split tolerance of
    the oracle."""
    import torch
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_128(3), 5.0)
    gpu_lib.set_precision(1)
    try:
        dev = torch.device("cuda", 0)
        off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
        T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
        arrs = [T(a) for a in (nb.dlist, nb.elist, nb.dlist_mom, nb.elist_mom, nb.dlist_momi, nb.elist_momi)]
        torch.cuda.synchronize()
        rw, bw, fb = gpu_lib.autotune_device(nb.natom, nb.nei, off.data_ptr(), *[a.data_ptr() for a in arrs])
        assert rw in (16, 32) and bw in (8, 12, 16) and fb in (4, 5, 6, 8)
        e, f, t, t0 = gpu_lib.acelib(nb)
    finally:
        gpu_lib.set_precision(0)
    eo, fo, to, t0o = oracle_seeded.acelib(nb)
    for got, ref in ((e, eo), (f, fo), (t, to), (t0, t0o)):
        assert rel_err(got, ref) < 1e-5


# ---------------------------------------------------------------------------
# A second layout: two densities with a non-linear embedding, 4-body clusters
# with l = l' = 1, other radial types; evaluated by the generic kernels.


@pytest.fixture()
def alt_lib(alt_potential):
    from magace import lib
    lib.init(alt_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    yield lib
    lib.set_precision(0)


@pytest.mark.parametrize("case", ["bcc128", "slab"])
def test_second_layout_fp64_parity(alt_lib, oracle_alt, case):
    from magace import structures as S
    st = {"bcc128": lambda: S.bcc_fe_128(4), "slab": _ragged_slab}[case]()
    _compare(alt_lib, oracle_alt, S.neighbor_data(st, 5.0))


def test_second_layout_split_precision(alt_lib, oracle_alt):
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_54(6), 5.0)
    alt_lib.set_precision(1)
    e, f, t, t0 = alt_lib.acelib(nb)
    eo, fo, to, t0o = oracle_alt.acelib(nb)
    assert np.abs(e - eo).max() * 1e3 < 1.0
    assert np.abs(f - fo).max() * 1e3 < 10.0
    assert np.abs(t - to).max() * 1e3 < 10.0 and np.abs(t0 - t0o).max() * 1e3 < 10.0
    for got, ref in ((e, eo), (f, fo), (t, to), (t0, t0o)):
        assert rel_err(got, ref) < 1e-5


def test_second_layout_descriptors_and_density_gradients(alt_lib, oracle_alt):
    """Per-atom basis functions B and dE/drho of both densities through the
    device API, against the oracle's prepB packs."""
    import torch
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_54(8), 5.0)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    arrs = [T(a) for a in (nb.dlist, nb.elist, nb.dlist_mom, nb.elist_mom, nb.dlist_momi, nb.elist_momi)]
    ncoef, nd = alt_lib.num_coefficients()
    assert nd == 2
    B = torch.zeros(nb.natom, ncoef, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    alt_lib.descriptors_device(nb.natom, nb.nei, off.data_ptr(), *[a.data_ptr() for a in arrs], B.data_ptr(), 1)
    outs = [torch.empty(n, dtype=torch.float64, device=dev) for n in (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)]
    alt_lib.compute_device(nb.natom, nb.nei, off.data_ptr(), *[a.data_ptr() for a in arrs],
                           *[o.data_ptr() for o in outs], 1)
    dedrho = torch.empty(nb.natom, 2, dtype=torch.float64, device=dev)
    alt_lib.density_gradient_device(nb.natom, dedrho.data_ptr(), 1)
    torch.cuda.synchronize()
    alt_lib.device_status()
    Bo, dedrho_o = oracle_alt.descriptors(nb)
    assert rel_err(B.cpu().numpy(), Bo) < 1e-10
    assert rel_err(dedrho.cpu().numpy(), dedrho_o) < 1e-10


def _device_eval(lib, nb, shift=0):
    """Split evaluation through ace_compute_device on device arrays; with
    shift = 1 every bond array starts 8 bytes past its allocation's start."""
    import torch
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)

    def T(a):
        buf = torch.zeros(len(a) + shift, dtype=torch.float64, device=dev)
        buf[shift:] = torch.tensor(a, dtype=torch.float64, device=dev)
        return buf[shift:]
    ins = [T(a) for a in (nb.dlist, nb.elist, nb.dlist_mom, nb.elist_mom, nb.dlist_momi, nb.elist_momi)]
    outs = [torch.empty(n, dtype=torch.float64, device=dev) for n in (nb.natom, 3 * nb.nei, 3 * nb.nei, 3 * nb.natom)]
    torch.cuda.synchronize()
    lib.compute_device(nb.natom, nb.nei, off.data_ptr(), *[x.data_ptr() for x in ins], *[o.data_ptr() for o in outs], 1)
    torch.cuda.synchronize()
    lib.device_status()
    return [o.cpu().numpy() for o in outs]


@pytest.mark.parametrize("shift", [0, 1])
def test_abasis_variants_on_device_inputs(gpu_lib, oracle_seeded, shift):
    """Every A-basis variant on device-resident bond arrays, the TMA-staged
    and tensor-core ones included: arrays that start on and 8 bytes past a 16-byte boundary,
    atoms of two 64-bond tiles (neighbours listed out to 8.4 A,
    beyond the cutoff) and an atom without neighbours. Split results stay
    within the split tolerance of the oracle and within 1e-6 of the scalar
    variant (3e-6 where the tensor-core forms' 3xTF32 products enter)."""
    from magace import structures as S
    st = _ragged_slab()
    st = S.Structure(np.vstack([st.positions, [[1.0, 1.0, 90.0]]]), st.cell, st.pbc, np.append(st.mag, 2.0),
                     np.vstack([st.mhat, [[0.0, 0.0, 1.0]]]))
    nb = S.neighbor_data(st, 8.4)
    counts = nb.nstop - nb.nstart + 1
    assert counts.max() > 64 and counts.min() == 0
    gpu_lib.set_precision(1)
    before = gpu_lib.get_tuning_indices()
    try:
        res = []
        for v in range(6):
            gpu_lib.set_tuning([v, 0, 0, 0])
            res.append(_device_eval(gpu_lib, nb, shift))
    finally:
        gpu_lib.set_tuning(before)
        gpu_lib.set_precision(0)
    eo, fo, to, t0o = oracle_seeded.acelib(nb)
    for got in res:
        e, f, t, t0 = got
        assert np.abs(e - eo).max() * 1e3 < 1.0 and np.abs(f - fo).max() * 1e3 < 10.0
        for x, y in zip(got, (eo, fo, to, t0o)):
            assert rel_err(x, y) < 1e-5
        for x, y in zip(got, res[0]):
            # FP32 rounding; the tensor-core forms' 3xTF32 products are within 2^-20
            assert rel_err(x, y) < 3e-6


def test_every_split_variant_matches_oracle(gpu_lib, oracle_seeded):
    """Variant v of the 2-/4-body density, 3-body and force kernels together
    (the A basis and the density kernels at min(v, 5): the force
    kernel has two more forms, on the tensor cores), on device arrays
    and through acelib_ with host arrays (where the GPU writes host memory
    directly, the force kernel's whole-line output form): every combination
    within the split tolerance of the oracle and within 3e-6 of variant 0.
    Neighbours listed out to 8.4 A give atoms of two 64-bond tiles."""
    from magace import structures as S
    nb = S.neighbor_data(_ragged_slab(), 8.4)
    gpu_lib.set_precision(1)
    before = gpu_lib.get_tuning_indices()
    try:
        res = []
        for v in range(8):
            gpu_lib.set_tuning([min(v, 5), min(v, 5), min(v, 5), v])
            res.append(_device_eval(gpu_lib, nb))
            res.append(list(gpu_lib.acelib(nb)))
    finally:
        gpu_lib.set_tuning(before)
        gpu_lib.set_precision(0)
    eo, fo, to, t0o = oracle_seeded.acelib(nb)
    for got in res:
        e, f, t, t0 = got
        assert np.abs(e - eo).max() * 1e3 < 1.0 and np.abs(f - fo).max() * 1e3 < 10.0
        for x, y in zip(got, (eo, fo, to, t0o)):
            assert rel_err(x, y) < 1e-5
        for x, y in zip(got, res[0]):
            # FP32 rounding; the tensor-core forms' 3xTF32 products are within 2^-20
            assert rel_err(x, y) < 3e-6



# ---------------------------------------------------------------------------
# 5- and 6-body clusters (HIGH_LAYOUT, generic kernels with gather entries of
# up to five other factors)

@pytest.fixture()
def high_lib(high_potential):
    from magace import lib
    lib.init(high_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    yield lib
    lib.set_precision(0)


@pytest.mark.parametrize("case", ["bcc54", "slab"])
def test_high_body_fp64_parity(high_lib, oracle_high, case):
    """Energies, forces and magnetic forces with 5- and 6-body clusters
    (src/b_basis.F90:310-532, src/forces.F90:234-331) equal the oracle's at
    1e-10 relative."""
    from magace import structures as S
    assert high_lib.basis_count(5) > 0 and high_lib.basis_count(6) > 0
    st = {"bcc54": lambda: S.bcc_fe_54(9), "slab": _ragged_slab}[case]()
    _compare(high_lib, oracle_high, S.neighbor_data(st, 5.0))
    assert high_lib.last_launch_count() == 3  # the generic kernels


def test_high_body_split_precision(high_lib, oracle_high):
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_54(10), 5.0)
    high_lib.set_precision(1)
    e, f, t, t0 = high_lib.acelib(nb)
    eo, fo, to, t0o = oracle_high.acelib(nb)
    assert np.abs(e - eo).max() * 1e3 < 1.0
    assert np.abs(f - fo).max() * 1e3 < 10.0
    assert np.abs(t - to).max() * 1e3 < 10.0 and np.abs(t0 - t0o).max() * 1e3 < 10.0
    for got, ref in ((e, eo), (f, fo), (t, to), (t0, t0o)):
        assert rel_err(got, ref) < 1e-5


def test_high_body_descriptors(high_lib, oracle_high):
    """The 5- and 6-body basis functions B (six factors per m-term) through
    ace_descriptors_device, against the oracle's prepB packs."""
    import torch
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_54(13), 5.0)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    arrs = [T(a) for a in (nb.dlist, nb.elist, nb.dlist_mom, nb.elist_mom, nb.dlist_momi, nb.elist_momi)]
    ncoef, nd = high_lib.num_coefficients()
    B = torch.zeros(nb.natom, ncoef, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    high_lib.descriptors_device(nb.natom, nb.nei, off.data_ptr(), *[a.data_ptr() for a in arrs], B.data_ptr(), 1)
    torch.cuda.synchronize()
    high_lib.device_status()
    Bo, _ = oracle_high.descriptors(nb)
    n4 = sum(high_lib.basis_count(r) for r in (1, 2, 3, 4))
    assert np.abs(Bo[:, n4:]).max() > 1e-3  # non-trivial 5-/6-body basis functions
    assert rel_err(B.cpu().numpy(), Bo) < 1e-10


def test_padded_high_body_clusters_contribute_nothing(high_lib):
    """A 5-/6-body cluster whose atomic or magnetic half the enumeration pads
    with zeros has no basis function (the reference reads its factors outside
    its A basis): its coefficient leaves every output unchanged."""
    from magace import structures as S
    nb = S.neighbor_data(S.bcc_fe_54(14), 5.0)
    before = high_lib.acelib(nb)
    c = high_lib.get_coefficients()
    n4 = sum(high_lib.basis_count(r) for r in (1, 2, 3, 4))
    r5, r6 = high_lib.basis_rows(5), high_lib.basis_rows(6)
    padded = [n4 + k for k, r in enumerate(r5) if r[0] == 0 or r[4] == 0]
    padded += [n4 + len(r5) + k for k, r in enumerate(r6) if r[0] == 0 or r[5] == 0]
    assert padded
    c2 = c.copy()
    c2[:, padded] += 3.0
    high_lib.set_coefficients(c2)
    after = high_lib.acelib(nb)
    high_lib.set_coefficients(c)
    for a, b in zip(after, before):
        assert np.array_equal(a, b)


# ---------------------------------------------------------------------------
# Radial basis types 6/5 and 4/6 in the Fe layout (the specialised kernels)

@pytest.mark.gpu
@pytest.mark.parametrize("case", ["bcc54", "slab"])
def test_radial_types_parity(radtype_potential, oracle_radtype, case):
    """FP64 equals the oracle at 1e-10 and split stays within the split
    tolerance (1 meV/atom, 10 meV/A, 10 meV/mu_B), with radial types the
    other seeded layouts do not use. The norm-relative bound is 2e-4 here:
    the FP32 copies of these seeded bases' spline coefficients cancel more
    than the Fe layout's (8e-5 measured on the per-bond magnetic forces, whose
    largest value is ~8e-3 eV/mu_B)."""
    from magace import lib, structures as S
    lib.init(radtype_potential, "Fe", 5.0, 4.0, 0.2, 1)
    st = S.bcc_fe_54(4) if case == "bcc54" else _ragged_slab()
    nb = S.neighbor_data(st, 5.0)
    lib.set_precision(0)
    _compare(lib, oracle_radtype, nb)
    lib.set_precision(1)
    try:
        e, f, t, t0 = lib.acelib(nb)
    finally:
        lib.set_precision(0)
    eo, fo, to, t0o = oracle_radtype.acelib(nb)
    assert np.abs(e - eo).max() * 1e3 < 1.0 and np.abs(f - fo).max() * 1e3 < 10.0
    assert np.abs(t - to).max() * 1e3 < 10.0 and np.abs(t0 - t0o).max() * 1e3 < 10.0
    for got, ref in ((e, eo), (f, fo), (t, to), (t0, t0o)):
        assert rel_err(got, ref) < 2e-4
