"""Writer for "<Elements>.<xc>.in" potential files and the seeded synthetic
potential used by the tests and the benchmark.

The seeded potential keeps the basis layout of the reference's example Fe
potential (example/Fe.pbe.in header, lines 6-13): 16/16 radial base
functions, 5 magnetic radial functions up to l' = 2, 3-body 4/3 radial
functions with l = 1 / l' = 2, 4-body 3/3 with l = l' = 0, one density, a
linear-limit embedding (nfemb 1, par 1.0 1.0), radial types 3 (atomic) and 7
(magnetic), cutoffs 5.0 A / 4.0 mu_B, taper 0.01, no hard core and inner
cutoff 10000/250. Every cluster, rad_atomic and rad_magnetic value is drawn
from N(0, sigma) with a fixed seed. The cluster list is the library's own
enumeration, read through ace_basis_rows.
"""
from __future__ import annotations

import os
import tempfile

import numpy as np

from . import lib

RANKS = (1, 2, 3, 4, 5, 6)  # cluster ranks of the 'clu' records (1 to 6 bodies)

FE_LAYOUT = dict(nradbase_a=16, nradbase_m=16, nradial2_m=5, l2max_m=2,
                 nradial3_a=4, nradial3_m=3, l3max_a=1, l3max_m=2,
                 nradial4_a=3, nradial4_m=3, l4max_a=0, l4max_m=0,
                 ndensity=1, npot=5, nfemb=1, radtype_a=3, radtype_m=7)

# A second, smaller layout that exercises what FE_LAYOUT leaves out: two
# densities with a non-linear embedding (nfemb 2), 4-body clusters with
# l = l' = 1, other radial types, and radial counts that fit none of the
# kernels specialised to FE_LAYOUT (so the generic kernels run).
ALT_LAYOUT = dict(nradbase_a=8, nradbase_m=6, nradial2_m=3, l2max_m=2,
                  nradial3_a=3, nradial3_m=2, l3max_a=2, l3max_m=1,
                  nradial4_a=2, nradial4_m=2, l4max_a=1, l4max_m=1,
                  ndensity=2, npot=5, nfemb=2, radtype_a=5, radtype_m=3)

# A layout with 5- and 6-body clusters (src/b_basis.F90:310-532), small
# enough for the oracle: 5-body with atomic l <= 1 and magnetic l' <= 1,
# 6-body with atomic l = 0 and magnetic l' <= 1, one density, radial types
# 4 (atomic) and 8 (magnetic).
HIGH_LAYOUT = dict(nradbase_a=6, nradbase_m=6, nradial2_m=2, l2max_m=2,
                   nradial3_a=2, nradial3_m=2, l3max_a=1, l3max_m=1,
                   nradial4_a=2, nradial4_m=1, l4max_a=1, l4max_m=1,
                   nradial5_a=1, nradial5_m=1, l5max_a=1, l5max_m=1,
                   nradial6_a=1, nradial6_m=1, l6max_a=0, l6max_m=1,
                   ndensity=1, npot=5, nfemb=1, radtype_a=4, radtype_m=8)


def header_lines(element: str, xc: str, smearing: float, lam=(5.25, 5.25), cut=(5.0, 4.0),
                 dcut=(0.01, 0.01), ecut=10000.0, decut=250.0, layout=FE_LAYOUT) -> list[str]:
    L = layout
    return [
        " Parameters (last)",
        " created        2026           1           1           0           0           0",
        f" Elements {element}",
        f" XC {xc}",
        f" gauss-smearing   {smearing!r}",
        f" lambda    {lam[0]!r}        {lam[1]!r}",
        f" rcut dcut ecut decut    {cut[0]!r}   {cut[1]!r}   {dcut[0]!r}   {dcut[1]!r}   {ecut!r}   {decut!r}",
        f" nradbase l2max   {L['nradbase_a']} {L['nradbase_m']} {L['nradial2_m']} {L['l2max_m']}",
        f" nradial3 l3max   {L['nradial3_a']} {L['nradial3_m']} {L['l3max_a']} {L['l3max_m']}",
        f" nradial4 l4max   {L['nradial4_a']} {L['nradial4_m']} {L['l4max_a']} {L['l4max_m']}",
        f" nradial5 l5max   {L.get('nradial5_a', 0)} {L.get('nradial5_m', 0)} {L.get('l5max_a', 0)} {L.get('l5max_m', 0)}",
        f" nradial6 l6max   {L.get('nradial6_a', 0)} {L.get('nradial6_m', 0)} {L.get('l6max_a', 0)} {L.get('l6max_m', 0)}",
        f" ndensity   {L['ndensity']}",
        f" npot-nfemb-radtype   {L['npot']} {L['nfemb']} {L['radtype_a']} {L['radtype_m']}",
    ]


def library_basis_rows(header: str, element: str, rcut: float, rcut_magnetic: float, smearing: float,
                       xcnumber: int) -> dict:
    """The cluster rows of ranks 1..4 that the library enumerates for the
    potential file `header` (its host-only init; no GPU)."""
    lib.init(header, element, rcut, rcut_magnetic, smearing, xcnumber)
    return {r: lib.basis_rows(r) for r in RANKS}


def write_seeded_potential(path: str, seed: int = 2024, sigma: float = 0.1, element: str = "Fe",
                           xc: str = "pbe", smearing: float = 0.2, layout=FE_LAYOUT,
                           cut=(5.0, 4.0), core=(0.0, 0.0), par=(1.0, 1.0), par2=(1.0, 1.0),
                           enumerate_basis=library_basis_rows) -> str:
    """Writes the seeded potential to `path` and returns the path.
    `enumerate_basis(header, element, rcut, rcut_magnetic, smearing,
    xcnumber)` lists the cluster basis of the header-only file `header`;
    by default the library's host-only init (no GPU). With two densities,
    `par2` holds the second density's embedding parameters and its cluster
    values come from a second generator (seed + 1), so the first density's
    records do not depend on the layout's density count."""
    head = header_lines(element, xc, smearing, cut=cut, layout=layout)
    with tempfile.TemporaryDirectory() as td:
        tmp = os.path.join(td, "header.in")
        with open(tmp, "w") as f:
            f.write("\n".join(head) + "\n")
        rows = enumerate_basis(tmp, element, cut[0], cut[1], smearing, 1 if xc == "pbe" else 2)
    rng = np.random.default_rng(seed)
    L = layout
    out = list(head)
    for k, v in ((1, par[0]), (2, par[1])):
        out += [f" par            {k}           1", f" {element}   {v!r}      F"]
    if L["ndensity"] == 2:
        for k, v in ((1, par2[0]), (2, par2[1])):
            out += [f" par            {k}           2", f" {element}   {v!r}      F"]
    for k, v in ((1, core[0]), (2, core[1])):
        out += [f" core            {k}           0", f" {element} {element}   {v!r}      F"]
    for l in range(L["l3max_a"] + 1):
        for nr in range(1, L["nradial3_a"] + 1):
            for n in range(1, L["nradbase_a"] + 1):
                out += [" rad_atomic            0           0",
                        f" {element} {element}  {n} {nr} {l} {rng.normal(0.0, sigma)!r} T"]
    for l in range(L["l2max_m"] + 1):
        for nr in range(1, L["nradial2_m"] + 1):
            for n in range(1, L["nradbase_m"] + 1):
                out += [" rad_magnetic            0           0",
                        f" {element} {element}  {n} {nr} {l} {rng.normal(0.0, sigma)!r} T"]
    for rank in RANKS:
        els = " ".join([element] * rank)
        for row in rows.get(rank, ()):
            idx = " ".join(str(int(x)) for x in row)
            out += [f" clu            {rank}           1",
                    f" {els}   {idx}   {rng.normal(0.0, sigma)!r}   T"]
    if L["ndensity"] == 2:
        rng2 = np.random.default_rng(seed + 1)
        for rank in RANKS:
            els = " ".join([element] * rank)
            for row in rows.get(rank, ()):
                idx = " ".join(str(int(x)) for x in row)
                out += [f" clu            {rank}           2",
                        f" {els}   {idx}   {rng2.normal(0.0, sigma)!r}   T"]
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return path


_WIDTH = {1: 1, 2: 4, 3: 9, 4: 15, 5: 21, 6: 27}


def write_coefficients(src: str, dst: str, coefs, rows: dict, element: str = "Fe") -> str:
    """Copies the potential file `src` to `dst` with new expansion
    coefficients: coefs[d][k] for the clusters rows[1..4] in coefficient
    order (ace_basis_rows, the library's order; ranks 1..6). The value of
    every 'clu' record (src/util.F90:678-956) is replaced; clusters without a record in
    `src` and with a nonzero coefficient get one appended. Everything else is
    copied unchanged. Returns dst."""
    coefs = np.atleast_2d(np.asarray(coefs, dtype=np.float64))
    index, k = {}, 0
    for rank in RANKS:
        for row in rows.get(rank, ()):
            index[(rank, tuple(int(x) for x in row))] = k
            k += 1
    if coefs.shape[1] != k:
        raise ValueError(f"expected {k} coefficients per density, got {coefs.shape[1]}")
    with open(src) as f:
        lines = f.read().splitlines()
    seen = set()
    out, q = [], 0
    while q < len(lines):
        line = lines[q]
        tok = line.split()
        if len(tok) == 3 and tok[0] == "clu" and q + 1 < len(lines):
            order, dens = int(tok[1]), int(tok[2])
            vals = lines[q + 1].split()
            if order in _WIDTH and 1 <= dens <= coefs.shape[0]:
                key = (order, tuple(int(x) for x in vals[order:order + _WIDTH[order]]))
                if key in index:
                    vals[order + _WIDTH[order]] = repr(float(coefs[dens - 1, index[key]]))
                    seen.add((dens, index[key]))
            out += [line, " " + "   ".join(vals)]
            q += 2
            continue
        out.append(line)
        q += 1
    for (rank, row), kk in index.items():
        for d in range(coefs.shape[0]):
            if (d + 1, kk) not in seen and coefs[d, kk] != 0.0:
                out += [f" clu            {rank}           {d + 1}",
                        f" {' '.join([element] * rank)}   {' '.join(str(x) for x in row)}   {float(coefs[d, kk])!r}   T"]
    with open(dst, "w") as f:
        f.write("\n".join(out) + "\n")
    return dst
