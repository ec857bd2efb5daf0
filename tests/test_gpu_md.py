"""Device-resident spin-lattice MD: the GPU cell-list neighbour list against
the host builder, the reverse-bond index, force/field assembly against the
acelib_ outputs assembled as the LAMMPS pair style does, and energy
conservation of the velocity-Verlet + spin-precession steps."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

MUB_OVER_HBAR = 5.78901e-5 / 6.582119569e-4


@pytest.fixture()
def md_lib(seeded_potential):
    from magace import lib
    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    yield lib
    lib.set_precision(0)


def _system(n=6, seed=4):
    from magace import structures as S
    st = S.bcc_fe_vacancies(ncell=n, seed=seed, vacancy_frac=0.02, jitter=0.1)
    return st


def test_neighbor_list_and_reverse_bonds(md_lib):
    from magace import md, structures as S
    st = _system()
    sim = md.SpinLatticeMD(st, skin=0.5)
    b = sim.bonds()
    nb = S.neighbor_data(st, 5.5)
    counts = np.diff(b["off"])
    assert np.array_equal(counts, nb.nstop - nb.nstart + 1)
    x, cell = st.positions, st.cell
    i = np.repeat(np.arange(sim.natom), counts)
    d = x[i] - x[b["j"]] - b["shift"] @ cell
    r = np.linalg.norm(d, axis=1)
    for a in range(0, sim.natom, 37):
        ours = np.sort(r[b["off"][a]:b["off"][a + 1]])
        ref = np.sort(nb.dlist[nb.nstart[a] - 1:nb.nstop[a]])
        assert np.allclose(ours, ref, atol=1e-12)
    rev = b["rev"]
    assert np.all(rev >= 0) and np.array_equal(rev[rev], np.arange(len(rev)))
    assert np.array_equal(b["j"][rev], i) and np.array_equal(b["shift"][rev], -b["shift"])
    sim.close()


def test_assembled_forces_match_acelib(md_lib):
    """Forces -dE/dx and fields -(mub/hbar) dE/dm of the MD state against
    acelib_ on the same configuration (neighbours to 5.0 A), assembled as the
    LAMMPS pair style does."""
    from magace import md, structures as S
    st = _system(seed=5)
    sim = md.SpinLatticeMD(st, skin=0.5)
    sim.run(0)
    s = sim.state()
    nb = S.neighbor_data(st, 5.0)
    e, f, t, t0 = md_lib.acelib(nb)
    F_ref, fm_ref = S.total_forces(nb, f, t, t0)
    assert rel_err(s["F"], F_ref) < 1e-11
    assert rel_err(s["fm"], MUB_OVER_HBAR * fm_ref) < 1e-11
    sim.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_energy_conservation_and_graph_replay(md_lib, precision):
    """100 steps of 1 fs at 300 K: the total energy drifts by far less than
    the kinetic energy's fluctuation; the CUDA-graph replay follows the plain
    launches."""
    from magace import md
    md_lib.set_precision(precision)
    st = _system(seed=6)
    a = md.SpinLatticeMD(st, temperature=300.0, seed=1)
    log_a = a.run(100, dt=0.001, rebuild_every=10, use_graph=True)
    b = md.SpinLatticeMD(st, temperature=300.0, seed=1)
    log_b = b.run(100, dt=0.001, rebuild_every=10, use_graph=False)
    tot = log_a.sum(axis=1)
    n = a.natom
    drift = abs(tot[-1] - tot[0]) / n
    print("precision", precision, "drift eV/atom", drift, "KE range eV/atom", np.ptp(log_a[:, 1]) / n)
    assert drift < 0.05 * np.ptp(log_a[:, 1]) / n
    if precision == 0:
        assert np.array_equal(log_a, log_b)
    else:
        assert np.allclose(log_a, log_b, rtol=1e-6, atol=1e-6 * n)
    a.close()
    b.close()
