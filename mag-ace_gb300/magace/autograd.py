"""Differentiable mag-ace energies for PyTorch.

`MagAceEnergy` is a torch.autograd.Function over the library's device path.
Its forward pass evaluates the per-atom energies E_i of one or many
configurations; the same kernels return the per-bond derivatives
dE_i/d(x_i - x_j) and dE_i/dm_j and the on-site dE_i/dm_i (the reference's
flist/tlist/tlist0, src/ace.F90:288-318), and dE_i/drho. Its backward pass
contracts them with the incoming per-atom gradient:

  positions  dL/dx_i = sum_{bonds i->j} g_i f_ij - sum_{bonds k->i} g_k f_ki
  moments    dL/dm_j = sum_{bonds i->j} g_i t_ij + g_j t0_j
  cell       dL/dh   = -sum_{bonds} g_i n_ij (x) f_ij   (n_ij the image of j)
  coeffs     dL/dc[d][k] = sum_i g_i dE_i/drho_d B_k(i)

The descriptors B are recomputed in the backward pass (A is not stored
between the passes). The neighbour list is built on the tensors' device by
`neighbor_list`, with the LAMMPS bond convention e_ij = (x_i - x_j)/r_ij
(lammps/pair_spin_ace.cpp:491-499).

The evaluator is pluggable: `LibraryEvaluator` runs the CUDA library on the
GPU; any object with the same four methods can stand in (the tests use the
CPU oracle that way to check this module's own algebra).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import lib


# ---------------------------------------------------------------------------
# neighbour lists

@dataclass
class Bonds:
    """Bonds of one or more configurations, grouped by centre atom (CSR)."""
    i: torch.Tensor        # [nei] centre atom (global index)
    j: torch.Tensor        # [nei] neighbour atom (global index of the original, not the image)
    shift: torch.Tensor    # [nei, 3] integer image of j (x_j + shift @ cell)
    offsets: torch.Tensor  # [natom + 1] int32 CSR offsets
    config: torch.Tensor   # [natom] configuration of each atom
    # for sums in a fixed order (no atomics): bonds per centre atom, the
    # bonds ordered by neighbour atom (a stable sort) with their counts, and
    # bonds per configuration (the bonds of configuration c are contiguous)
    count_i: torch.Tensor = None
    perm_j: torch.Tensor = None
    count_j: torch.Tensor = None
    count_config: torch.Tensor = None

    def sum_by_i(self, x: torch.Tensor) -> torch.Tensor:
        """Per centre atom, the sum of x over its bonds, in bond order."""
        return torch.segment_reduce(x, "sum", lengths=self.count_i, axis=0)

    def sum_by_j(self, x: torch.Tensor) -> torch.Tensor:
        """Per atom, the sum of x over the bonds that have it as neighbour, in
        bond order."""
        return torch.segment_reduce(x[self.perm_j], "sum", lengths=self.count_j, axis=0)

    def sum_by_config(self, x: torch.Tensor) -> torch.Tensor:
        return torch.segment_reduce(x, "sum", lengths=self.count_config, axis=0)


def _image_range(cell: torch.Tensor, pbc, rcut: float) -> list[int]:
    """Images per axis needed to find every neighbour within rcut."""
    h = cell.detach().to(torch.float64).cpu().numpy()
    vol = abs(np.linalg.det(h))
    out = []
    for a in range(3):
        if not pbc[a]:
            out.append(0)
            continue
        b, c = h[(a + 1) % 3], h[(a + 2) % 3]
        width = vol / np.linalg.norm(np.cross(b, c))  # distance between the faces spanned by b, c
        out.append(int(math.ceil(rcut / width)))
    return out


def neighbor_list(positions: torch.Tensor, cell: torch.Tensor, pbc, rcut: float, atom_offset: int = 0):
    """All pairs (i, j, image) with 0 < |x_i - x_j - n h| < rcut of one
    configuration, on the positions' device, sorted by i. Returns
    (i, j, shift) with indices offset by `atom_offset`."""
    n = positions.shape[0]
    dev = positions.device
    k = _image_range(cell, pbc, rcut)
    rng = [torch.arange(-kk, kk + 1, device=dev) for kk in k]
    shifts = torch.stack(torch.meshgrid(*rng, indexing="ij"), dim=-1).reshape(-1, 3).to(torch.float64)
    x = positions.detach().to(torch.float64)
    img = shifts @ cell.detach().to(torch.float64)                    # [S, 3]
    d = x[:, None, None, :] - x[None, :, None, :] - img[None, None]   # [n, n, S, 3]
    r2 = (d * d).sum(-1)
    self_pair = (torch.arange(n, device=dev)[:, None] == torch.arange(n, device=dev)[None, :])[:, :, None] & \
                (shifts.abs().sum(-1) == 0)[None, None, :]
    mask = (r2 < rcut * rcut) & ~self_pair
    ii, jj, ss = torch.nonzero(mask, as_tuple=True)                   # row-major: sorted by i
    return ii + atom_offset, jj + atom_offset, shifts[ss].to(torch.int64)


def batch_bonds(configs, rcut: float) -> Bonds:
    """Neighbour lists of a batch of configurations, concatenated: atoms of
    configuration c follow those of c-1, bonds never cross configurations."""
    parts, natom, cfg = [], 0, []
    for c, (pos, cell, pbc) in enumerate(configs):
        parts.append(neighbor_list(pos, cell, pbc, rcut, natom))
        cfg.append(torch.full((pos.shape[0],), c, dtype=torch.int64, device=pos.device))
        natom += pos.shape[0]
    i = torch.cat([p[0] for p in parts])
    j = torch.cat([p[1] for p in parts])
    shift = torch.cat([p[2] for p in parts])
    counts = torch.bincount(i, minlength=natom)
    offsets = torch.zeros(natom + 1, dtype=torch.int32, device=i.device)
    offsets[1:] = torch.cumsum(counts, 0).to(torch.int32)
    config = torch.cat(cfg)
    return Bonds(i=i, j=j, shift=shift, offsets=offsets, config=config, count_i=counts,
                 perm_j=torch.argsort(j, stable=True), count_j=torch.bincount(j, minlength=natom),
                 count_config=torch.bincount(config[i], minlength=len(configs)))


def bond_vectors(x: torch.Tensor, cells: torch.Tensor, b: Bonds) -> torch.Tensor:
    """d_ij = x_i - x_j - shift_ij @ h_config(i) for every bond."""
    h = cells[b.config[b.i]]                                          # [nei, 3, 3]
    return x[b.i] - x[b.j] - torch.einsum("bk,bkc->bc", b.shift.to(x.dtype), h)


# ---------------------------------------------------------------------------
# evaluators

class LibraryEvaluator:
    """The CUDA library on the current device. Arrays are torch CUDA tensors.
    Each call runs on the caller's current torch stream, so that the library
    reads inputs that torch has finished writing (the library's own stream,
    selected by a NULL stream, does not wait for other streams)."""

    def __init__(self):
        self.ncoef, self.ndensity = lib.num_coefficients()

    @staticmethod
    def _stream(dev):
        """The current torch stream of `dev`, and a handle that is never the
        NULL (library-stream) handle: the legacy default stream when torch is
        on it."""
        st = torch.cuda.current_stream(dev)
        handle = st.cuda_stream
        return st, (handle if handle else 1)  # 1 = cudaStreamLegacy

    def evaluate(self, offsets, r, e, magj, mhj, magi, mhi):
        """(E [N], fij [nei,3], tij [nei,3], ti0 [N,3], dE/drho [N,2])."""
        natom, nei = magi.shape[0], r.shape[0]
        dev = r.device
        out = [torch.empty(natom, dtype=torch.float64, device=dev),
               torch.empty(nei, 3, dtype=torch.float64, device=dev),
               torch.empty(nei, 3, dtype=torch.float64, device=dev),
               torch.empty(natom, 3, dtype=torch.float64, device=dev),
               torch.zeros(natom, 2, dtype=torch.float64, device=dev)]
        st, s = self._stream(dev)
        ptr = lambda t: t.data_ptr() if t.numel() else 0
        lib.compute_device(natom, nei, ptr(offsets), ptr(r), ptr(e), ptr(magj), ptr(mhj), ptr(magi), ptr(mhi),
                           ptr(out[0]), ptr(out[1]), ptr(out[2]), ptr(out[3]), s)
        lib.density_gradient_device(natom, ptr(out[4]), s)
        st.synchronize()
        lib.device_status()
        return tuple(out)

    def descriptors(self, offsets, r, e, magj, mhj, magi, mhi):
        natom = magi.shape[0]
        B = torch.empty(natom, self.ncoef, dtype=torch.float64, device=r.device)
        st, s = self._stream(r.device)
        ptr = lambda t: t.data_ptr() if t.numel() else 0
        lib.descriptors_device(natom, r.shape[0], ptr(offsets), ptr(r), ptr(e), ptr(magj), ptr(mhj), ptr(magi),
                               ptr(mhi), ptr(B), s)
        st.synchronize()
        lib.device_status()
        return B

    def descriptors_tangent(self, offsets, r, e, magj, mhj, magi, mhi, dd, dmj, dmi):
        """(B, dB [N, ncoef], core, dcore [N]) along the tangents dd (bond
        vectors), dmj and dmi (moments)."""
        natom, nei = magi.shape[0], r.shape[0]
        dev = r.device
        B = torch.empty(natom, self.ncoef, dtype=torch.float64, device=dev)
        Bd = torch.empty_like(B)
        core = torch.empty(natom, dtype=torch.float64, device=dev)
        cored = torch.empty_like(core)
        st, s = self._stream(dev)
        ptr = lambda t: t.data_ptr() if t.numel() else 0
        lib.descriptors_tangent_device(natom, nei, ptr(offsets), ptr(r), ptr(e), ptr(magj), ptr(mhj), ptr(magi),
                                       ptr(mhi), ptr(dd), ptr(dmj), ptr(dmi), ptr(B), ptr(Bd), ptr(core),
                                       ptr(cored), s)
        st.synchronize()
        lib.device_status()
        return B, Bd, core, cored

    def embedding(self) -> dict:
        return lib.embedding()

    def get_coefficients(self) -> np.ndarray:
        return lib.get_coefficients()

    def set_coefficients(self, c) -> None:
        lib.set_coefficients(c)


# ---------------------------------------------------------------------------
# the autograd function

def _inputs(x, m, cells, b: Bonds):
    """Library inputs from positions, moments and bonds: r, e, |m_j|, m_j/|m_j|
    per bond and |m_i|, m_i/|m_i| per atom. A zero moment points along z
    (neilist/neilist.F90:764-769)."""
    d = bond_vectors(x, cells, b)
    r = torch.linalg.norm(d, dim=1)
    e = d / r[:, None]
    mag = torch.linalg.norm(m, dim=1)
    zero = mag == 0
    mh = torch.where(zero[:, None], torch.tensor([0.0, 0.0, 1.0], dtype=m.dtype, device=m.device),
                     m / torch.where(zero, torch.ones_like(mag), mag)[:, None])
    return d, r, e.contiguous(), mag[b.j].contiguous(), mh[b.j].contiguous(), mag.contiguous(), mh.contiguous()


class MagAceEnergy(torch.autograd.Function):
    """Per-atom energies E [N] of a batch of configurations.

    Inputs: positions [N,3], moments [N,3] (Cartesian, mu_B), cells [C,3,3]
    (rows are lattice vectors), coefficients [ndensity, ncoef]; `potential`
    is the MagAcePotential that owns the evaluator and the bonds."""

    @staticmethod
    def forward(ctx, positions, moments, cells, coeffs, potential):
        potential._sync_coefficients(coeffs)
        b = potential._bonds
        d, r, e, magj, mhj, magi, mhi = _inputs(positions.detach(), moments.detach(), cells.detach(), b)
        E, fij, tij, ti0, dedrho = potential.evaluator.evaluate(b.offsets, r, e, magj, mhj, magi, mhi)
        ctx.potential = potential
        ctx.bonds = b
        ctx.lib_inputs = (b.offsets, r, e, magj, mhj, magi, mhi)
        ctx.save_for_backward(fij, tij, ti0, dedrho)
        ctx.shapes = (positions.shape, cells.shape)
        return E

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, gE):
        fij, tij, ti0, dedrho = ctx.saved_tensors
        b = ctx.bonds
        gE = gE.to(torch.float64)
        gi = gE[b.i][:, None]
        gpos = gmom = gcell = gcoef = None
        # every sum runs over segments in a fixed order: the backward pass is
        # bitwise reproducible (no floating-point atomics)
        if ctx.needs_input_grad[0]:
            gpos = b.sum_by_i(gi * fij) - b.sum_by_j(gi * fij)
        if ctx.needs_input_grad[1]:
            gmom = gE[:, None] * ti0 + b.sum_by_j(gi * tij)
        if ctx.needs_input_grad[2]:
            # d_ij = x_i - x_j - n_ij h: dd_b/dh_kb = -n_k
            per_bond = -b.shift.to(torch.float64)[:, :, None] * (gi * fij)[:, None, :]
            gcell = b.sum_by_config(per_bond)
        if ctx.needs_input_grad[3]:
            B = ctx.potential.evaluator.descriptors(*ctx.lib_inputs)
            nd = ctx.potential.ndensity
            w = gE[:, None] * dedrho[:, :nd]                                   # [N, nd]
            gcoef = (w.T @ B).reshape(nd, -1)
        return gpos, gmom, gcell, gcoef, None


def _embed(nfemb: int, rho: torch.Tensor, wpre: float, mexp: float) -> torch.Tensor:
    """The embedding F(rho) (src/forces.F90:1134-1266, nfemb 0-2), elementwise
    in torch so that autograd gives F' and F''."""
    if nfemb == 0:
        return rho.clone()
    w, eps = 10.0, 1e-10
    s = 1.0 + rho if nfemb == 2 else rho
    small = s.abs() <= eps
    ss = torch.where(small, torch.ones_like(s), s)
    y1 = w * ss * ss
    g = torch.where(y1 > 30.0, torch.zeros_like(y1), torch.exp(-torch.clamp(y1, max=30.0)))
    a = ss.abs()
    sg = torch.sign(ss)
    big = sg * (torch.pow((1.0 - g) * a, mexp) + mexp * g * a)
    big = wpre * (big - 1.0) if nfemb == 2 else wpre * big
    lin = wpre * mexp * (s - 1.0) if nfemb == 2 else wpre * mexp * rho
    return torch.where(small, lin, big)


def _fcut(e: torch.Tensor, ecut: float, decut: float) -> torch.Tensor:
    """The inner cutoff on the core energy (src/forces.F90:1112-1128)."""
    elow = ecut - decut
    mid = 0.5 * (1.0 + torch.cos(math.pi * (e - elow) / decut))
    return torch.where(e >= ecut, torch.zeros_like(e), torch.where(e <= elow, torch.ones_like(e), mid))


class MagAceForces(torch.autograd.Function):
    """Per-atom energies E [N], forces F [N,3] = -dE_tot/dx and magnetic
    forces FM [N,3] = -dE_tot/dm of a batch of configurations, differentiable
    with respect to the coefficients: the gradient of any loss on E, F and FM
    for fitting (src/modules.F90:57-72 weights energies and forces in the
    reference's fitting loss).

    With u = dL/dF and v = dL/dFM per atom, the force terms of dL/dc are
    -d/de [dE_tot/dc] along the displacement (x + e u, m + e v); with
    E_i = fcut(e_core,i) sum_d F_d(rho_id) + e_core,i and rho_id = c_d . B_i,
      dL/dc_d = sum_i gE_i fcut F_d' B_i
                - sum_i [fcut' de_core,i F_d' B_i + fcut (F_d'' drho_id B_i + F_d' dB_i)],
    where dB_i, drho_id and de_core,i are the directional derivatives that
    ace_descriptors_tangent_device evaluates (forward mode, exact). Gradients
    with respect to positions, moments and cells (second derivatives of the
    energy) are not provided."""

    @staticmethod
    def forward(ctx, positions, moments, cells, coeffs, potential):
        potential._sync_coefficients(coeffs)
        b = potential._bonds
        d, r, e, magj, mhj, magi, mhi = _inputs(positions.detach(), moments.detach(), cells.detach(), b)
        E, fij, tij, ti0, dedrho = potential.evaluator.evaluate(b.offsets, r, e, magj, mhj, magi, mhi)
        F = b.sum_by_j(fij) - b.sum_by_i(fij)      # -dE_tot/dx
        FM = -(ti0 + b.sum_by_j(tij))              # -dE_tot/dm
        ctx.potential = potential
        ctx.bonds = b
        ctx.lib_inputs = (b.offsets, r, e, magj, mhj, magi, mhi)
        ctx.save_for_backward(coeffs.detach().to(torch.float64))
        return E, F, FM

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, gE, gF, gFM):
        if any(ctx.needs_input_grad[:3]):
            raise NotImplementedError("MagAceForces differentiates with respect to the coefficients only")
        gcoef = None
        if ctx.needs_input_grad[3]:
            (c,) = ctx.saved_tensors
            b = ctx.bonds
            pot = ctx.potential
            offsets, r, e, magj, mhj, magi, mhi = ctx.lib_inputs
            dev = r.device
            z3 = lambda n: torch.zeros(n, 3, dtype=torch.float64, device=dev)
            u = gF.to(torch.float64) if gF is not None else z3(magi.shape[0])
            v = gFM.to(torch.float64) if gFM is not None else z3(magi.shape[0])
            gE = gE.to(torch.float64) if gE is not None else torch.zeros(magi.shape[0], dtype=torch.float64,
                                                                        device=dev)
            # tangents: bond vectors d_ij = x_i - x_j - n h move by u_i - u_j
            dd = (u[b.i] - u[b.j]).contiguous()
            dmj = v[b.j].contiguous()
            B, Bd, core, cored = pot.evaluator.descriptors_tangent(offsets, r, e, magj, mhj, magi, mhi, dd, dmj,
                                                                   v.contiguous())
            emb = pot.evaluator.embedding()
            c = c.to(dev)
            rho = B @ c.T                                     # [N, nd]
            rhod = Bd @ c.T
            # F', F'' and fcut' by autograd of the elementwise functions (the
            # backward pass runs with gradients off)
            with torch.enable_grad():
                rr = rho.detach().clone().requires_grad_(True)
                Fsum = sum(_embed(emb["nfemb"], rr[:, k], float(emb["par"][0][k]), float(emb["par"][1][k])).sum()
                           for k in range(rho.shape[1]))
                (dF,) = torch.autograd.grad(Fsum, rr, create_graph=True)            # F_d'(rho_id)
                d2F = torch.stack([torch.autograd.grad(dF[:, k].sum(), rr, retain_graph=True)[0][:, k]
                                   for k in range(rho.shape[1])], dim=1)        # F_d''(rho_id)
                ee = core.detach().clone().requires_grad_(True)
                fc = _fcut(ee, emb["ecut"], emb["decut"])
                (dfc,) = torch.autograd.grad(fc.sum(), ee)
            dF, d2F, fc = dF.detach(), d2F.detach(), fc.detach()
            w_e = (gE * fc)[:, None] * dF                                        # [N, nd]
            w_b = (dfc * cored)[:, None] * dF + fc[:, None] * d2F * rhod
            w_bd = fc[:, None] * dF
            gcoef = (w_e - w_b).T @ B - w_bd.T @ Bd
        return None, None, None, gcoef, None


class MagAcePotential:
    """A mag-ace potential as a differentiable PyTorch function of positions,
    moments, cells and coefficients, for one or many configurations at once."""

    def __init__(self, evaluator=None, rcut: float = 5.0):
        self.evaluator = evaluator if evaluator is not None else LibraryEvaluator()
        self.rcut = rcut
        c = np.asarray(self.evaluator.get_coefficients(), dtype=np.float64)
        self.ndensity, self.ncoef = c.shape
        self._coef = c.copy()
        self._bonds = None

    def coefficients(self, device=None, requires_grad: bool = False) -> torch.Tensor:
        return torch.tensor(self._coef, dtype=torch.float64, device=device, requires_grad=requires_grad)

    def _sync_coefficients(self, coeffs: torch.Tensor) -> None:
        c = coeffs.detach().to(torch.float64).cpu().numpy().reshape(self.ndensity, self.ncoef)
        if not np.array_equal(c, self._coef):
            self.evaluator.set_coefficients(c)
            self._coef = c.copy()

    def build_bonds(self, positions, cells, pbcs, natoms) -> Bonds:
        configs, a = [], 0
        for c, n in enumerate(natoms):
            configs.append((positions[a:a + n].detach(), cells[c].detach(), pbcs[c]))
            a += n
        return batch_bonds(configs, self.rcut)

    def energies(self, positions, moments, cells, pbcs, natoms, coeffs=None, rebuild: bool = True):
        """Per-atom energies of the batch; natoms[c] atoms of configuration c
        follow those of configuration c-1 in positions/moments."""
        if rebuild or self._bonds is None:
            self._bonds = self.build_bonds(positions, cells, pbcs, natoms)
        if coeffs is None:
            coeffs = self.coefficients(device=positions.device)
        return MagAceEnergy.apply(positions, moments, cells, coeffs, self)

    def forces(self, positions, moments, cells, pbcs, natoms, coeffs=None, rebuild: bool = True):
        """(E [N], F [N,3], FM [N,3]): per-atom energies, forces -dE_tot/dx and
        magnetic forces -dE_tot/dm, differentiable with respect to coeffs
        (MagAceForces), for fitting on forces."""
        if rebuild or self._bonds is None:
            self._bonds = self.build_bonds(positions, cells, pbcs, natoms)
        if coeffs is None:
            coeffs = self.coefficients(device=positions.device)
        return MagAceForces.apply(positions, moments, cells, coeffs, self)

    def config_energies(self, positions, moments, cells, pbcs, natoms, coeffs=None) -> torch.Tensor:
        E = self.energies(positions, moments, cells, pbcs, natoms, coeffs)
        return torch.segment_reduce(E, "sum", lengths=torch.tensor(natoms, device=E.device), axis=0)

    def virial(self, positions, moments, cells, pbcs, natoms) -> torch.Tensor:
        """Per-configuration virial W_ab = -sum_bonds d_a dE/dd_b [C,3,3]
        (the pair-style convention, lammps/pair_spin_ace.cpp:571-646, with
        f_ij = -dE_i/dd_ij); -W/V is the stress from the potential."""
        b = self.build_bonds(positions, cells, pbcs, natoms)
        self._bonds = b
        d, r, e, magj, mhj, magi, mhi = _inputs(positions.detach(), moments.detach(), cells.detach(), b)
        _, fij, _, _, _ = self.evaluator.evaluate(b.offsets, r, e, magj, mhj, magi, mhi)
        return b.sum_by_config(-d[:, :, None] * fij[:, None, :])
