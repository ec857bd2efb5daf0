"""Synthetic spin-lattice structures and their flat neighbour lists.

The flat arrays follow the marshalling of the reference's LAMMPS caller
(lammps/pair_spin_ace.cpp:446-543): one full neighbour list, per bond
r_ij = |x_i - x_j| and the unit vector (x_i - x_j)/r_ij, the neighbour's moment
magnitude |m_j| and direction m_hat_j, per atom |m_i| and m_hat_i, and 1-based
CSR ranges nstart/nstop. These are exactly the inputs of acelib_
(src/ace.F90:79-107).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class NeighborData:
    """Inputs of one acelib_ call, as contiguous numpy arrays."""

    natom: int
    nall: int
    nei: int
    nlist: np.ndarray      # int32[nei], 1-based index of j (not used in arithmetic)
    occ: np.ndarray        # int32[natom], element of i (1 = the single element)
    occlist: np.ndarray    # int32[nei], element of j
    nstart: np.ndarray     # int32[natom], 1-based first bond of i
    nstop: np.ndarray      # int32[natom], 1-based last bond of i (inclusive)
    dlist: np.ndarray      # f64[nei], r_ij
    elist: np.ndarray      # f64[3*nei], (x_i - x_j)/r_ij interleaved xyz
    dlist_momi: np.ndarray  # f64[natom], |m_i|
    elist_momi: np.ndarray  # f64[3*natom], m_hat_i
    dlist_mom: np.ndarray  # f64[nei], |m_j|
    elist_mom: np.ndarray  # f64[3*nei], m_hat_j
    # bookkeeping for finite differences and force assembly
    i_of_bond: np.ndarray = field(default=None, repr=False)   # int64[nei], 0-based i
    j_of_bond: np.ndarray = field(default=None, repr=False)   # int64[nei], 0-based owner of j
    shift: np.ndarray = field(default=None, repr=False)       # f64[nei,3], image shift of j

    @property
    def bonds_per_atom(self) -> np.ndarray:
        return (self.nstop - self.nstart + 1).astype(np.int64)


@dataclass
class Structure:
    positions: np.ndarray  # [n,3] Angstrom
    cell: np.ndarray       # [3,3] rows are lattice vectors (orthorhombic here)
    pbc: tuple
    mag: np.ndarray        # [n] |m| in mu_B
    mhat: np.ndarray       # [n,3] unit moment directions


def bcc_cubic(nx: int, ny: int, nz: int, a: float) -> tuple[np.ndarray, np.ndarray]:
    """Positions of an nx*ny*nz supercell of the 2-atom cubic bcc cell."""
    base = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])
    grid = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1)
    grid = grid.reshape(-1, 1, 3)
    pos = ((grid + base[None]) * a).reshape(-1, 3)
    cell = np.diag([nx * a, ny * a, nz * a]).astype(np.float64)
    return pos.astype(np.float64), cell


def fcc_cubic(nx: int, ny: int, nz: int, a: float) -> tuple[np.ndarray, np.ndarray]:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], dtype=np.float64)
    grid = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1)
    grid = grid.reshape(-1, 1, 3)
    pos = ((grid + base[None]) * a).reshape(-1, 3)
    cell = np.diag([nx * a, ny * a, nz * a]).astype(np.float64)
    return pos, cell


def random_unit(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def cone_unit(rng: np.random.Generator, n: int, half_angle_deg: float) -> np.ndarray:
    """Directions uniform on the spherical cap of the given half angle about z."""
    cmin = np.cos(np.deg2rad(half_angle_deg))
    cz = rng.uniform(cmin, 1.0, size=n)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=n)
    s = np.sqrt(np.maximum(0.0, 1.0 - cz * cz))
    return np.stack([s * np.cos(phi), s * np.sin(phi), cz], axis=1)


def neighbor_data(st: Structure, rcut: float) -> NeighborData:
    """Full neighbour list within rcut, including periodic images, in the
    LAMMPS sign convention e_ij = (x_i - x_j)/r_ij
    (lammps/pair_spin_ace.cpp:491-499)."""
    from scipy.spatial import cKDTree

    pos = np.asarray(st.positions, dtype=np.float64)
    n = len(pos)
    cell = np.asarray(st.cell, dtype=np.float64)
    reps = []
    for d in range(3):
        if st.pbc[d]:
            length = np.linalg.norm(cell[d])
            reps.append(int(np.ceil(rcut / length)))
        else:
            reps.append(0)
    shifts = np.array([[i, j, k] for i in range(-reps[0], reps[0] + 1)
                       for j in range(-reps[1], reps[1] + 1)
                       for k in range(-reps[2], reps[2] + 1)], dtype=np.float64)
    svec = shifts @ cell
    # keep only images that can reach the central cell within rcut
    lo = pos.min(0) - rcut
    hi = pos.max(0) + rcut
    img_pos, img_owner, img_shift = [], [], []
    for s in svec:
        p = pos + s
        keep = np.all((p >= lo) & (p <= hi), axis=1)
        img_pos.append(p[keep])
        img_owner.append(np.nonzero(keep)[0])
        img_shift.append(np.broadcast_to(s, (keep.sum(), 3)))
    img_pos = np.concatenate(img_pos)
    img_owner = np.concatenate(img_owner)
    img_shift = np.concatenate(img_shift)
    tree = cKDTree(img_pos)
    lists = tree.query_ball_point(pos, r=rcut)
    ii, jj = [], []
    for i, lst in enumerate(lists):
        lst = np.asarray(sorted(lst), dtype=np.int64)
        d = np.linalg.norm(pos[i] - img_pos[lst], axis=1)
        lst = lst[(d > 1e-8) & (d < rcut)]
        ii.append(np.full(len(lst), i, dtype=np.int64))
        jj.append(lst)
    ii = np.concatenate(ii) if ii else np.zeros(0, np.int64)
    jj = np.concatenate(jj) if jj else np.zeros(0, np.int64)
    counts = np.bincount(ii, minlength=n)
    nstop = np.cumsum(counts)
    nstart = nstop - counts + 1
    delta = pos[ii] - img_pos[jj]
    r = np.linalg.norm(delta, axis=1)
    e = delta / r[:, None]
    owner = img_owner[jj]
    nei = len(ii)
    return NeighborData(
        natom=n, nall=n, nei=nei,
        nlist=(owner + 1).astype(np.int32),
        occ=np.ones(n, np.int32), occlist=np.ones(nei, np.int32),
        nstart=nstart.astype(np.int32), nstop=nstop.astype(np.int32),
        dlist=np.ascontiguousarray(r), elist=np.ascontiguousarray(e.reshape(-1)),
        dlist_momi=np.ascontiguousarray(st.mag.astype(np.float64)),
        elist_momi=np.ascontiguousarray(st.mhat.reshape(-1).astype(np.float64)),
        dlist_mom=np.ascontiguousarray(st.mag[owner].astype(np.float64)),
        elist_mom=np.ascontiguousarray(st.mhat[owner].reshape(-1).astype(np.float64)),
        i_of_bond=ii, j_of_bond=owner, shift=img_shift[jj])


def notebook_cell() -> Structure:
    """2-atom cubic bcc Fe, a = 2.83 A, m = (0, 0, 2.22) mu_B on both atoms
    (example/basic_lammps.ipynb cells 14-17)."""
    pos, cell = bcc_cubic(1, 1, 1, 2.83)
    return Structure(pos, cell, (True, True, True), np.full(2, 2.22),
                     np.tile([0.0, 0.0, 1.0], (2, 1)))


def bcc_fe_128(seed: int = 1) -> Structure:
    """128-atom bcc Fe (4x4x4 cubic cells, a = 2.83 A), jitter N(0, 0.05 A),
    |m| ~ U(2.0, 2.4) mu_B, directions uniform in a 30 degree cone about z."""
    rng = np.random.default_rng(seed)
    pos, cell = bcc_cubic(4, 4, 4, 2.83)
    pos = pos + rng.normal(0.0, 0.05, size=pos.shape)
    n = len(pos)
    return Structure(pos, cell, (True, True, True), rng.uniform(2.0, 2.4, n), cone_unit(rng, n, 30.0))


def bcc_fe_vacancies(ncell: int = 20, seed: int = 2, vacancy_frac: float = 0.01,
                     jitter: float = 0.1) -> Structure:
    """ncell^3 cubic bcc cells (2*ncell^3 sites) with random vacancies, jitter
    N(0, jitter), paramagnetic directions uniform on the sphere,
    |m| ~ U(1.5, 2.6) mu_B. ncell=20 is the 16,000-site workload."""
    rng = np.random.default_rng(seed)
    pos, cell = bcc_cubic(ncell, ncell, ncell, 2.83)
    nsite = len(pos)
    nvac = int(round(vacancy_frac * nsite))
    keep = np.ones(nsite, bool)
    keep[rng.choice(nsite, size=nvac, replace=False)] = False
    pos = pos[keep] + rng.normal(0.0, jitter, size=(keep.sum(), 3))
    n = len(pos)
    return Structure(pos, cell, (True, True, True), rng.uniform(1.5, 2.6, n), random_unit(rng, n))


def bcc_fe_54(seed: int) -> Structure:
    """54-atom bcc Fe (3x3x3), jitter N(0, 0.1 A), random spins."""
    rng = np.random.default_rng(seed)
    pos, cell = bcc_cubic(3, 3, 3, 2.83)
    pos = pos + rng.normal(0.0, 0.1, size=pos.shape)
    n = len(pos)
    return Structure(pos, cell, (True, True, True), rng.uniform(1.5, 2.6, n), random_unit(rng, n))


def total_forces(nb: NeighborData, flist: np.ndarray, tlist: np.ndarray, tlist0: np.ndarray):
    """Per-atom forces and magnetic forces assembled as the LAMMPS caller does
    (lammps/pair_spin_ace.cpp:571-631): f_i -= f_ij, f_j += f_ij,
    fm_j -= t_ij, fm_i -= t0_i."""
    n = nb.natom
    fl = flist.reshape(-1, 3)
    tl = tlist.reshape(-1, 3)
    f = np.zeros((n, 3))
    fm = -tlist0.reshape(-1, 3).copy()
    np.add.at(f, nb.i_of_bond, -fl)
    np.add.at(f, nb.j_of_bond, fl)
    np.add.at(fm, nb.j_of_bond, -tl)
    return f, fm


def bcc_110_slab(nx: int, ny: int, layers: int, a: float, vacuum: float) -> tuple[np.ndarray, np.ndarray]:
    """bcc (110) slab in the orthogonal cell x || [1-10], y || [001],
    z || [110] (lengths a*sqrt2, a, a*sqrt2 per repeat, 4 atoms), `layers`
    repeats along z plus `vacuum` Angstrom of empty space on top."""
    s2 = np.sqrt(2.0)
    # the 4-atom orthogonal cell, fractional coordinates
    base = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
    lx, ly, lz = a * s2, a, a * s2
    grid = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(layers), indexing="ij"), -1).reshape(-1, 1, 3)
    pos = ((grid + base[None]) * np.array([lx, ly, lz])).reshape(-1, 3)
    cell = np.diag([nx * lx, ny * ly, layers * lz + vacuum])
    return pos, cell


def uneven_batch(nconf: int = 256, seed: int = 3) -> list:
    """Independent configurations of 16-432 atoms with 20-70 neighbours per
    atom within 5 A: bcc and fcc Fe bulk and bcc cells with vacancies, each
    under a hydrostatic strain (lattice constant scaled by U(0.88, 1.02), so
    that the compressed cells reach 60-70 neighbours), and (100) / (110) bcc
    slabs of one or more cubic repeats with 10 A of vacuum (20-40 neighbours
    at their surfaces); jitter N(0, 0.1 A), random spins with
    |m| ~ U(1.5, 2.6) mu_B."""
    rng = np.random.default_rng(seed)
    out = []
    kinds = ("bcc", "fcc", "vac", "s100", "s110")
    for c in range(nconf):
        kind = kinds[c % len(kinds)]
        pbc = (True, True, True)
        scale = float(rng.uniform(0.88, 1.02))
        if kind == "bcc":
            n = int(rng.integers(2, 7))                     # 16 .. 432 atoms
            pos, cell = bcc_cubic(n, n, n, 2.83 * scale)
        elif kind == "fcc":
            n = int(rng.integers(2, 5))                     # 32 .. 256 atoms
            pos, cell = fcc_cubic(n, n, n, 3.59 * scale)
        elif kind == "vac":
            n = int(rng.integers(3, 7))
            pos, cell = bcc_cubic(n, n, n, 2.83 * scale)
            keep = rng.random(len(pos)) > 0.05
            keep[0] = True
            pos = pos[keep]
        elif kind == "s100":
            layers = int(rng.integers(1, 6))
            n = int(rng.integers(3 if layers == 1 else 2, 5))  # at least 16 atoms
            pos, cell = bcc_cubic(n, n, layers, 2.83)
            cell[2, 2] += 10.0
            pbc = (True, True, False)
        else:
            n, layers = int(rng.integers(2, 4)), int(rng.integers(1, 5))
            pos, cell = bcc_110_slab(n, 2 * n, layers, 2.83, 10.0)
            pbc = (True, True, False)
        pos = pos + rng.normal(0.0, 0.1, size=pos.shape)
        m = len(pos)
        out.append(Structure(pos, cell, pbc, rng.uniform(1.5, 2.6, m), random_unit(rng, m)))
    return out


def concat_neighbor_data(parts: list) -> NeighborData:
    """One acelib_ input of independent configurations: atoms and bonds of
    part k follow those of part k-1 (bond ranges and j indices shifted)."""
    a_off = np.cumsum([0] + [p.natom for p in parts])
    b_off = np.cumsum([0] + [p.nei for p in parts])
    cat = lambda name: np.ascontiguousarray(np.concatenate([getattr(p, name) for p in parts]))
    return NeighborData(
        natom=int(a_off[-1]), nall=int(a_off[-1]), nei=int(b_off[-1]),
        nlist=np.concatenate([p.nlist + a for p, a in zip(parts, a_off)]).astype(np.int32),
        occ=cat("occ"), occlist=cat("occlist"),
        nstart=np.concatenate([p.nstart + b for p, b in zip(parts, b_off)]).astype(np.int32),
        nstop=np.concatenate([p.nstop + b for p, b in zip(parts, b_off)]).astype(np.int32),
        dlist=cat("dlist"), elist=cat("elist"), dlist_momi=cat("dlist_momi"), elist_momi=cat("elist_momi"),
        dlist_mom=cat("dlist_mom"), elist_mom=cat("elist_mom"),
        i_of_bond=np.concatenate([p.i_of_bond + a for p, a in zip(parts, a_off)]),
        j_of_bond=np.concatenate([p.j_of_bond + a for p, a in zip(parts, a_off)]),
        shift=np.concatenate([p.shift for p in parts]))
