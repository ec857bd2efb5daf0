"""The differentiation harness (magace.autograd): forces, magnetic forces,
cell gradient / virial and coefficient gradients of the per-atom energies,
checked by torch.autograd.gradcheck against centred finite differences
(h = 1e-5, FP64) and against the reference algorithm's analytic forces.

CPU tests run the harness over the CPU oracle (an evaluator with the
library's interface), which checks the harness's own algebra: neighbour
list, scatter of per-bond derivatives, cell gradient, coefficient chain
rule. GPU tests run it over the CUDA library."""
from __future__ import annotations

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_err  # noqa: E402

NONLINEAR_PAR = (1.0, 0.5)  # embedding exponent 0.5: F is not linear in rho


class OracleEvaluator:
    """The library's evaluator interface over the CPU oracle (test only)."""

    def __init__(self, potfile: str):
        import oracle as orc
        from magace import lib
        self.orc = orc
        self.src = potfile
        self.path = potfile
        self.o = orc.Oracle(potfile, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)
        lib.init(potfile, "Fe", 5.0, 4.0, 0.2, 1)  # host-only: coefficient order and rows
        self.rows = {r: lib.basis_rows(r) for r in (1, 2, 3, 4, 5, 6)}
        self.coef = lib.get_coefficients()
        self.generation = 0

    def _nb(self, offsets, r, e, magj, mhj, magi, mhi):
        from magace.structures import NeighborData
        off = offsets.cpu().numpy().astype(np.int64)
        natom, nei = len(off) - 1, int(off[-1])
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda t: np.ascontiguousarray(t.detach().cpu().numpy().reshape(-1), dtype=np.float64)
        return NeighborData(natom=natom, nall=natom, nei=nei, nlist=i32(np.ones(nei)), occ=i32(np.ones(natom)),
                            occlist=i32(np.ones(nei)), nstart=i32(off[:-1] + 1), nstop=i32(off[1:]),
                            dlist=f64(r), elist=f64(e), dlist_momi=f64(magi), elist_momi=f64(mhi),
                            dlist_mom=f64(magj), elist_mom=f64(mhj))

    def evaluate(self, *args):
        nb = self._nb(*args)
        E, f, t, t0 = self.o.acelib(nb, nthreads=4)
        _, dedrho = self.o.descriptors(nb)
        T = lambda a, *s: torch.tensor(np.asarray(a).reshape(*s), dtype=torch.float64)
        return T(E, -1), T(f, -1, 3), T(t, -1, 3), T(t0, -1, 3), T(dedrho, -1, 2)

    def descriptors(self, *args):
        B, _ = self.o.descriptors(self._nb(*args))
        return torch.tensor(B, dtype=torch.float64)

    def get_coefficients(self):
        return self.coef.copy()

    def set_coefficients(self, c):
        from magace import potential
        self.generation += 1
        d = os.path.dirname(self.src)
        path = os.path.join(d, f"gen{self.generation}", "Fe.pbe.in")
        os.makedirs(os.path.dirname(path), exist_ok=True)
        potential.write_coefficients(self.src, path, c, self.rows)
        self.o = self.orc.Oracle(path, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)
        self.coef = np.asarray(c, dtype=np.float64).copy()


@pytest.fixture(scope="module")
def nonlinear_potential(tmp_path_factory):
    from magace import potential
    path = str(tmp_path_factory.mktemp("potnl") / "Fe.pbe.in")
    potential.write_seeded_potential(path, seed=77, par=NONLINEAR_PAR)
    return path


def _bcc_batch(ncells, seeds, device="cpu"):
    from magace import structures as S
    pos, mom, cells, pbcs, nat = [], [], [], [], []
    for n, sd in zip(ncells, seeds):
        rng = np.random.default_rng(sd)
        p, cell = S.bcc_cubic(n, n, n, 2.83)
        p = p + rng.normal(0, 0.1, p.shape)
        m = S.random_unit(rng, len(p)) * rng.uniform(1.5, 2.6, len(p))[:, None]
        pos.append(p)
        mom.append(m)
        cells.append(cell)
        pbcs.append((True, True, True))
        nat.append(len(p))
    T = lambda a: torch.tensor(np.concatenate(a) if isinstance(a, list) else a, dtype=torch.float64, device=device)
    return T(pos), T(mom), torch.tensor(np.stack(cells), dtype=torch.float64, device=device), pbcs, nat


def test_neighbor_list_matches_host_builder():
    """The torch neighbour list finds the same bonds as the host builder."""
    from magace import autograd as AG, structures as S
    st = S.bcc_fe_54(4)
    pos = torch.tensor(st.positions)
    cell = torch.tensor(st.cell)
    i, j, sh = AG.neighbor_list(pos, cell, st.pbc, 5.0)
    nb = S.neighbor_data(st, 5.0)
    assert len(i) == nb.nei
    d = (pos[i] - pos[j] - sh.double() @ cell).norm(dim=1).numpy()
    counts = np.bincount(i.numpy(), minlength=nb.natom)
    assert np.array_equal(counts, nb.nstop - nb.nstart + 1)
    for a in range(nb.natom):
        ours = np.sort(d[i.numpy() == a])
        ref = np.sort(nb.dlist[nb.nstart[a] - 1:nb.nstop[a]])
        assert np.allclose(ours, ref, atol=1e-12)


def test_descriptors_reproduce_the_density(oracle_seeded, seeded_potential):
    """rho_i = sum_k c_k B_k(i) with the library's coefficient vector and the
    oracle's descriptors: with the seeded potential's linear embedding and
    no core term, E_i = rho_i."""
    from magace import lib, structures as S
    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    c = lib.get_coefficients()
    nb = S.neighbor_data(S.bcc_fe_54(2), 5.0)
    B, dedrho = oracle_seeded.descriptors(nb)
    E, *_ = oracle_seeded.acelib(nb)
    assert B.shape == (nb.natom, c.shape[1])
    assert rel_err(B @ c[0], E) < 1e-12
    assert np.allclose(dedrho[:, 0], 1.0)


def test_write_coefficients_round_trip(seeded_potential, tmp_path):
    from magace import lib, potential
    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    rows = {r: lib.basis_rows(r) for r in (1, 2, 3, 4)}
    c = lib.get_coefficients()
    c2 = c * 1.5 + 0.01
    out = str(tmp_path / "Fe.pbe.in")
    potential.write_coefficients(seeded_potential, out, c2, rows)
    lib.init(out, "Fe", 5.0, 4.0, 0.2, 1)
    assert np.array_equal(lib.get_coefficients(), c2)
    lib.set_coefficients(c)  # host-side table rebuild
    assert np.array_equal(lib.get_coefficients(), c)


# The magnetic radial basis of the seeded potential is a degree-15 Chebyshev
# expansion in |m|; along some directions the energy's third derivative in m
# reaches ~1e7 eV/mu_B^3, so a centred difference with h = 1e-5 carries up to
# ~1e-4 truncation error there (it falls as h^2: 1.5e-6 at h = 1e-6). The
# moments are therefore checked with h = 1e-6 at tight tolerances and with
# h = 1e-5 at a tolerance above that truncation error.
MOMENT_CHECKS = ((1e-6, 1e-5), (1e-5, 1e-3))  # (h, atol)


def _gradcheck_all(pot, x, m, cells, pbcs, nat, coeffs, **kw):
    f_xh = lambda x_, h_: pot.energies(x_, m.detach(), h_, pbcs, nat, coeffs)
    assert torch.autograd.gradcheck(f_xh, (x, cells), eps=1e-5, atol=1e-6, rtol=1e-5, **kw)
    f_m = lambda m_: pot.energies(x.detach(), m_, cells.detach(), pbcs, nat, coeffs)
    for h, atol in MOMENT_CHECKS:
        assert torch.autograd.gradcheck(f_m, (m,), eps=h, atol=atol, rtol=1e-5, **kw)


def test_gradcheck_positions_moments_cell_on_oracle(nonlinear_potential):
    """Centred finite differences of the per-atom energies of a 16-atom
    periodic cell (neighbours through several images) against the harness's
    backward pass: positions and cell with h = 1e-5, moments as above."""
    from magace import autograd as AG
    pot = AG.MagAcePotential(OracleEvaluator(nonlinear_potential))
    x, m, cells, pbcs, nat = _bcc_batch([2], [5])
    x.requires_grad_(True)
    m.requires_grad_(True)
    cells.requires_grad_(True)
    _gradcheck_all(pot, x, m, cells, pbcs, nat, pot.coefficients())


def test_gradcheck_coefficients_on_oracle(nonlinear_potential):
    """dE/dc = dE/drho * B, checked along random directions (fast mode)."""
    from magace import autograd as AG
    pot = AG.MagAcePotential(OracleEvaluator(nonlinear_potential))
    x, m, cells, pbcs, nat = _bcc_batch([2], [6])
    coeffs = pot.coefficients(requires_grad=True)
    fn = lambda c_: pot.energies(x, m, cells, pbcs, nat, c_)
    assert torch.autograd.gradcheck(fn, (coeffs,), eps=1e-5, atol=1e-6, rtol=1e-5, fast_mode=True)


def test_virial_is_the_strain_derivative(nonlinear_potential):
    """Under a homogeneous strain x -> x (1 + eps), h -> h (1 + eps), the
    energy changes by -sum W_ab eps_ab: W from the per-bond forces."""
    from magace import autograd as AG
    pot = AG.MagAcePotential(OracleEvaluator(nonlinear_potential))
    x, m, cells, pbcs, nat = _bcc_batch([2], [8])
    W = pot.virial(x, m, cells, pbcs, nat)[0]
    h = 1e-5
    for a, b in ((0, 0), (1, 2), (2, 1)):
        eps = torch.zeros(3, 3, dtype=torch.float64)
        eps[a, b] = h
        Ep = pot.config_energies(x @ (torch.eye(3) + eps), m, cells @ (torch.eye(3) + eps), pbcs, nat).sum()
        Em = pot.config_energies(x @ (torch.eye(3) - eps), m, cells @ (torch.eye(3) - eps), pbcs, nat).sum()
        dE = float((Ep - Em) / (2 * h))
        assert abs(dE + float(W[a, b])) < 1e-6 * max(1.0, abs(dE))


# ---------------------------------------------------------------------------
# GPU: the same harness over the CUDA library


@pytest.mark.gpu
def test_gpu_descriptors_match_oracle(seeded_potential, oracle_seeded):
    from magace import autograd as AG, lib, structures as S
    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    st = S.bcc_fe_54(9)
    nb = S.neighbor_data(st, 5.0)
    dev = torch.device("cuda", 0)
    off = torch.tensor(np.concatenate([[0], np.cumsum(nb.nstop - nb.nstart + 1)]).astype(np.int32), device=dev)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    args = (off, T(nb.dlist), T(nb.elist), T(nb.dlist_mom), T(nb.elist_mom), T(nb.dlist_momi), T(nb.elist_momi))
    ev = AG.LibraryEvaluator()
    B = ev.descriptors(*args).cpu().numpy()
    Bo, dedrho_o = oracle_seeded.descriptors(nb)
    assert rel_err(B, Bo) < 1e-10
    E, fij, tij, ti0, dedrho = ev.evaluate(*args)
    assert rel_err(dedrho.cpu().numpy()[:, 0], dedrho_o[:, 0]) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_batch_forces_match_oracle(nonlinear_potential, precision):
    """64 configurations of 54-atom bcc Fe in one evaluation: per-atom forces
    and magnetic forces from the backward pass against the oracle's analytic
    ones (FP64: 1e-10; split: within 10 meV/A)."""
    import oracle as orc
    from magace import autograd as AG, lib, structures as S
    lib.init(nonlinear_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(precision)
    try:
        dev = torch.device("cuda", 0)
        pot = AG.MagAcePotential(AG.LibraryEvaluator())
        x, m, cells, pbcs, nat = _bcc_batch([3] * 64, list(range(100, 164)), device=dev)
        x.requires_grad_(True)
        m.requires_grad_(True)
        E = pot.energies(x, m, cells, pbcs, nat)
        E.sum().backward()
        gx, gm = x.grad.cpu().numpy(), m.grad.cpu().numpy()
    finally:
        lib.set_precision(0)
    o = orc.Oracle(nonlinear_potential, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)
    xs, ms = x.detach().cpu().numpy(), m.detach().cpu().numpy()
    tol = 1e-10 if precision == 0 else None
    for c in (0, 17, 63):
        a = slice(54 * c, 54 * (c + 1))
        st = S.Structure(xs[a], cells[c].cpu().numpy(), (True, True, True), np.linalg.norm(ms[a], axis=1),
                         ms[a] / np.linalg.norm(ms[a], axis=1)[:, None])
        nb = S.neighbor_data(st, 5.0)
        e, f, t, t0 = o.acelib(nb)
        fx, fm = S.total_forces(nb, f, t, t0)  # -dE/dx, -dE/dm of the total energy
        gx_ref, gm_ref = -fx, -fm
        assert rel_err(E[a].detach().cpu().numpy(), e) < (1e-10 if tol else 1e-5)
        if tol:
            assert rel_err(gx[a], gx_ref) < tol and rel_err(gm[a], gm_ref) < tol
        else:
            assert np.abs(gx[a] - gx_ref).max() * 1e3 < 10.0 and np.abs(gm[a] - gm_ref).max() * 1e3 < 10.0


@pytest.mark.gpu
def test_gpu_gradcheck_all_inputs(nonlinear_potential):
    """gradcheck (FP64 path) of positions, moments and cell of a 54-atom
    configuration (steps as in _gradcheck_all), and of the coefficients
    along random directions (h = 1e-5). The backward pass sums per-bond terms
    over segments in a fixed order, so gradcheck's repeated backward passes
    agree bit for bit (nondet_tol 0)."""
    from magace import autograd as AG, lib
    lib.init(nonlinear_potential, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    dev = torch.device("cuda", 0)
    pot = AG.MagAcePotential(AG.LibraryEvaluator())
    x, m, cells, pbcs, nat = _bcc_batch([3], [3], device=dev)
    x.requires_grad_(True)
    m.requires_grad_(True)
    cells.requires_grad_(True)
    _gradcheck_all(pot, x, m, cells, pbcs, nat, pot.coefficients(device=dev), nondet_tol=0.0)
    c = pot.coefficients(device=dev, requires_grad=True)
    x0, m0, h0 = x.detach(), m.detach(), cells.detach()
    fc = lambda c_: pot.energies(x0, m0, h0, pbcs, nat, c_)
    assert torch.autograd.gradcheck(fc, (c,), eps=1e-5, atol=1e-6, rtol=1e-5, fast_mode=True, nondet_tol=0.0)


def test_embedding_derivatives_match_oracle(nonlinear_potential, oracle_seeded):
    """The torch restatement of the embedding (autograd._embed) gives the
    oracle's dE/drho (src/forces.F90:1134-1266) for the non-linear
    embedding, over densities of both signs and near zero."""
    import oracle as orc
    from magace import autograd as AG, structures as S
    o = orc.Oracle(nonlinear_potential, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)
    nb = S.neighbor_data(S.bcc_fe_54(21), 5.0)
    B, dedrho = o.descriptors(nb)
    from magace import lib
    lib.init(nonlinear_potential, "Fe", 5.0, 4.0, 0.2, 1)
    c = lib.get_coefficients()
    emb = lib.embedding()
    assert emb["nfemb"] == 1 and emb["par"][1][0] == 0.5
    rho = torch.tensor(B @ c[0], requires_grad=True)
    F = AG._embed(emb["nfemb"], rho, float(emb["par"][0][0]), float(emb["par"][1][0]))
    (dF,) = torch.autograd.grad(F.sum(), rho)
    assert rel_err(dF.numpy(), dedrho[:, 0]) < 1e-12
    assert (rho.detach().numpy() < 0).any() and (rho.detach().numpy() > 0).any()


def _force_loss_gradcheck(potfile):
    """gradcheck, along random directions, of the coefficients' gradient of
    E, F and FM (MagAceForces) and of a squared force loss."""
    from magace import autograd as AG, lib
    lib.init(potfile, "Fe", 5.0, 4.0, 0.2, 1)
    lib.set_precision(0)
    dev = torch.device("cuda", 0)
    pot = AG.MagAcePotential(AG.LibraryEvaluator())
    x, m, cells, pbcs, nat = _bcc_batch([3], [5], device=dev)
    pot._bonds = pot.build_bonds(x, cells, pbcs, nat)
    c = pot.coefficients(device=dev, requires_grad=True)
    f = lambda c_: pot.forces(x, m, cells, pbcs, nat, c_, rebuild=False)
    assert torch.autograd.gradcheck(f, (c,), eps=1e-5, atol=1e-6, rtol=1e-5, fast_mode=True, nondet_tol=0.0)
    E0, F0, FM0 = (t.detach() for t in f(c.detach()))
    rng = np.random.default_rng(1)
    Fref = F0 + torch.tensor(rng.normal(0, 0.05, F0.shape), device=dev)
    Mref = FM0 + torch.tensor(rng.normal(0, 0.05, FM0.shape), device=dev)

    def loss(c_):
        E, F, FM = pot.forces(x, m, cells, pbcs, nat, c_, rebuild=False)
        return ((F - Fref) ** 2).sum() + 0.3 * ((FM - Mref) ** 2).sum() + 0.1 * E.sum() ** 2

    assert torch.autograd.gradcheck(loss, (c,), eps=1e-5, atol=1e-6, rtol=1e-5, fast_mode=True, nondet_tol=0.0)
    # bitwise-reproducible backward
    g1 = torch.autograd.grad(loss(c), c)[0]
    g2 = torch.autograd.grad(loss(c), c)[0]
    assert torch.equal(g1, g2)
    assert g1.abs().max() > 0


@pytest.mark.gpu
def test_gpu_force_loss_coefficient_gradients(nonlinear_potential):
    """Fitting on forces: d(loss on E, F, FM)/dc through the forward-mode
    tangents of the descriptors, against centred differences (h = 1e-5),
    with a non-linear embedding (exponent 0.5)."""
    _force_loss_gradcheck(nonlinear_potential)


@pytest.mark.gpu
def test_gpu_force_loss_coefficient_gradients_high_body(high_potential):
    """The same with 5- and 6-body clusters (six-factor descriptor tangents)."""
    _force_loss_gradcheck(high_potential)
