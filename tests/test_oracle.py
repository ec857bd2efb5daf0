"""CPU tests of the oracle itself: pinned to the reference's only known
answer (example/basic_lammps.ipynb:272) and to centred finite differences,
plus the symmetries the energy must have."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

NOTEBOOK_ETOT = -15.7479878560111  # example/basic_lammps.ipynb:272


def test_basis_sizes_fe(oracle_fe):
    # clusters of example/Fe.pbe.in: 16 'clu 1', 720 'clu 2', 4932 'clu 3', 495 'clu 4', no 5/6-body
    assert oracle_fe.nvar == (16, 720, 4932, 495, 0, 0)
    assert (oracle_fe.nterms2, oracle_fe.nterms3, oracle_fe.nterms4) == (2160, 64008, 495)


def test_notebook_energy(oracle_fe):
    from magace import structures as S
    nb = S.neighbor_data(S.notebook_cell(), 4.5)
    assert np.all(nb.stop_counts == 26) if hasattr(nb, "stop_counts") else True
    e, f, t, t0 = oracle_fe.acelib(nb)
    assert abs(e.sum() - NOTEBOOK_ETOT) < 1e-12 * abs(NOTEBOOK_ETOT) + 1e-13
    F, FM = S.total_forces(nb, f, t, t0)
    assert np.abs(F).max() < 1e-12  # example/basic_lammps.ipynb:292-293


def test_notebook_golden_fixture(oracle_fe):
    """The committed golden vectors (tests/golden/notebook_fe.json, made by
    tests/golden/make_golden.py) match the oracle bit for bit."""
    from magace import structures as S
    with open(os.path.join(GOLDEN, "notebook_fe.json")) as fh:
        g = json.load(fh)
    nb = S.neighbor_data(S.notebook_cell(), 4.5)
    e, f, t, t0 = oracle_fe.acelib(nb)
    assert np.allclose(e, g["eout"], rtol=0, atol=1e-13)
    assert np.allclose(t0, g["tlist0"], rtol=0, atol=1e-13)


def test_reference_cells_golden_fixture(oracle_fe):
    """The oracle on example/Fe.pbe.in for the two non-collinear cells
    reproduces the committed per-atom summaries
    (tests/golden/reference_fe_cells.json)."""
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as mg
    from magace import structures as S
    with open(os.path.join(GOLDEN, "reference_fe_cells.json")) as fh:
        g = json.load(fh)
    for name, st in mg.reference_cells().items():
        nb = S.neighbor_data(st, 4.5)
        got = mg.per_atom_summary(nb, *oracle_fe.acelib(nb))
        for k in ("eout", "tlist0", "fsum", "tsum"):
            assert np.allclose(got[k], g[name][k], rtol=0, atol=1e-12), (name, k)
        for k in ("f_sumsq", "t_sumsq"):
            assert abs(got[k] - g[name][k]) <= 1e-12 * abs(g[name][k]), (name, k)


def _energy(orc, st, rcut):
    from magace import structures as S
    nb = S.neighbor_data(st, rcut)
    e, f, t, t0 = orc.acelib(nb)
    return e.sum(), nb, f, t, t0


def _fd_check(orc, rc, h):
    from magace import structures as S
    rng = np.random.default_rng(3)
    pos, cell = S.bcc_cubic(2, 2, 2, 2.83)
    pos = pos + rng.normal(0, 0.08, pos.shape)
    n = len(pos)
    mvec = rng.uniform(1.8, 2.4, n)[:, None] * S.random_unit(rng, n)

    def st_of(p, mv):
        m = np.linalg.norm(mv, axis=1)
        return S.Structure(p, cell, (True,) * 3, m, mv / m[:, None])

    E, nb, f, t, t0 = _energy(orc, st_of(pos, mvec), rc)
    F, FM = S.total_forces(nb, f, t, t0)
    for k in (0, 5, 11):
        for c in range(3):
            p = pos.copy(); p[k, c] += h
            ep = _energy(orc, st_of(p, mvec), rc)[0]
            p[k, c] -= 2 * h
            em = _energy(orc, st_of(p, mvec), rc)[0]
            assert abs(-(ep - em) / (2 * h) - F[k, c]) < 5e-7 * max(1.0, abs(F[k, c]))
            mv = mvec.copy(); mv[k, c] += h
            ep = _energy(orc, st_of(pos, mv), rc)[0]
            mv[k, c] -= 2 * h
            em = _energy(orc, st_of(pos, mv), rc)[0]
            assert abs(-(ep - em) / (2 * h) - FM[k, c]) < 5e-7 * max(1.0, abs(FM[k, c]))


@pytest.mark.parametrize("which", ["fe", "seeded", "alt", "high"])
def test_finite_differences(which, request):
    """Forces and magnetic forces assembled as in lammps/pair_spin_ace.cpp
    equal -dE/dx and -dE/dm from centred differences (h = 1e-5), for the
    example Fe potential and the seeded layouts (the second one with two
    densities and a non-linear embedding, the third with 5- and 6-body
    clusters; its radial basis has a larger third derivative, so it takes
    h = 2e-6, where the truncation error falls as h^2)."""
    orc = request.getfixturevalue({"fe": "oracle_fe", "seeded": "oracle_seeded", "alt": "oracle_alt",
                                   "high": "oracle_high"}[which])
    _fd_check(orc, 4.5 if which == "fe" else 5.0, 2e-6 if which == "high" else 1e-5)


def test_finite_differences_radial_types(oracle_radtype):
    """The same with radial basis types 6/5 and 4/6 (type 6 is used by no
    other layout)."""
    _fd_check(oracle_radtype, 5.0, 1e-5)


def test_rotation_and_moment_reversal(oracle_seeded):
    """E is invariant under a joint rotation of positions and moments, under
    separate rotations of the moments alone (the magnetic and atomic spaces
    are coupled to invariants separately, src/b_basis.F90:142-212), and under
    m -> -m (even magnetic l sums)."""
    from magace import structures as S
    rng = np.random.default_rng(9)
    pos, cell = S.bcc_cubic(2, 2, 2, 2.83)
    pos = pos + rng.normal(0, 0.05, pos.shape)
    n = len(pos)
    mag = rng.uniform(1.8, 2.4, n)
    mh = S.random_unit(rng, n)
    e0 = oracle_seeded.acelib(S.neighbor_data(S.Structure(pos, cell, (True,) * 3, mag, mh), 5.0))[0]
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    # rotate the moments only
    e1 = oracle_seeded.acelib(S.neighbor_data(S.Structure(pos, cell, (True,) * 3, mag, mh @ q.T), 5.0))[0]
    e2 = oracle_seeded.acelib(S.neighbor_data(S.Structure(pos, cell, (True,) * 3, mag, -mh), 5.0))[0]
    assert np.allclose(e1, e0, rtol=0, atol=1e-10)
    assert np.allclose(e2, e0, rtol=0, atol=1e-10)


def test_high_body_rotation_invariance(oracle_high):
    """With 5- and 6-body clusters the energy stays invariant under a joint
    rotation of positions and moments and under rotating the moments alone:
    the generalized couplings of src/util.F90:4389-4546 form invariants."""
    from magace import structures as S
    assert oracle_high.nvar[4] > 0 and oracle_high.nvar[5] > 0
    rng = np.random.default_rng(12)
    pos, cell = S.bcc_cubic(2, 2, 2, 2.83)
    pos = pos + rng.normal(0, 0.08, pos.shape)
    n = len(pos)
    mag, mh = rng.uniform(1.8, 2.4, n), S.random_unit(rng, n)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    e0 = oracle_high.acelib(S.neighbor_data(S.Structure(pos, cell, (True,) * 3, mag, mh), 5.0))[0]
    e1 = oracle_high.acelib(S.neighbor_data(S.Structure(pos, cell, (True,) * 3, mag, mh @ q.T), 5.0))[0]
    e2 = oracle_high.acelib(S.neighbor_data(S.Structure(pos @ q.T, cell @ q.T, (True,) * 3, mag, mh @ q.T),
                                            5.0))[0]
    assert np.allclose(e1, e0, rtol=0, atol=1e-11)
    assert np.allclose(e2, e0, rtol=0, atol=1e-11)
