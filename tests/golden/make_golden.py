"""Generates the golden vectors under tests/golden/ with the CPU oracle.

  Fe.pbe.in.gz        the reference's example potential, example/Fe.pbe.in,
                      byte for byte (gzip without a timestamp), the input of
                      every test on the reference's own potential; its sha256
                      is pinned in reference_fe.json. Refreshed only when
                      MAGACE_REFERENCE names a mag-ace checkout.
  notebook_fe.json    the reference's example cell (2-atom cubic bcc Fe,
                      a = 2.83 A, m = (0,0,2.22) mu_B, example/Fe.pbe.in,
                      rcut 4.5 / 4.0, smear 0.2); its total energy is the
                      notebook's -15.7479878560111 eV.
  reference_fe_cells.json  example/Fe.pbe.in (rcut 4.5 / 4.0) on two
                      non-collinear cells: the 128-atom bcc cell with moments
                      in a 30 degree cone (seed 1) and the 54-atom bcc cell
                      with directions uniform on the sphere (seed 3). Per atom:
                      E_i, t0_i, and the per-atom sums of f_ij and t_ij; plus
                      the sums of squares of the per-bond vectors.
  seeded_bcc16.json   the seeded synthetic potential (seed 2024) on a jittered
                      16-atom bcc cell, plus the sha256 of the generated
                      potential file so its generation stays reproducible.

Run from the repository root:
  MAGACE_REFERENCE=<path of a mag-ace checkout> python tests/golden/make_golden.py
(without MAGACE_REFERENCE the committed Fe.pbe.in.gz is used as it is).
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "mag-ace_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from magace import potential, structures as S  # noqa: E402
import oracle as orc  # noqa: E402

FIXTURE = os.path.join(HERE, "Fe.pbe.in.gz")


def seeded_cell16():
    rng = np.random.default_rng(16)
    pos, cell = S.bcc_cubic(2, 2, 2, 2.83)
    pos = pos + rng.normal(0.0, 0.05, pos.shape)
    n = len(pos)
    return S.Structure(pos, cell, (True, True, True), rng.uniform(2.0, 2.4, n), S.cone_unit(rng, n, 30.0))


def reference_cells():
    """The non-collinear cells the reference potential is checked on."""
    return {"bcc128_cone": S.bcc_fe_128(1), "bcc54_random": S.bcc_fe_54(3)}


def per_atom_summary(nb, e, f, t, t0) -> dict:
    """Per-atom energies, on-site magnetic forces and sums of the per-bond
    vectors, plus the sums of squares of the per-bond vectors."""
    ib = np.repeat(np.arange(nb.natom), nb.nstop - nb.nstart + 1)
    fs = np.zeros((nb.natom, 3))
    ts = np.zeros((nb.natom, 3))
    np.add.at(fs, ib, f.reshape(-1, 3))
    np.add.at(ts, ib, t.reshape(-1, 3))
    return {"natom": nb.natom, "nei": nb.nei, "eout": e, "tlist0": t0, "fsum": fs.reshape(-1),
            "tsum": ts.reshape(-1), "f_sumsq": float(np.sum(f * f)), "t_sumsq": float(np.sum(t * t))}


def dump(path, **arrays):
    with open(path, "w") as fh:
        json.dump({k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in arrays.items()}, fh)


def refresh_fixture(checkout: str) -> None:
    src = os.path.join(checkout, "example", "Fe.pbe.in")
    raw = open(src, "rb").read()
    with open(FIXTURE, "wb") as fh:
        with gzip.GzipFile(filename="Fe.pbe.in", mode="wb", fileobj=fh, compresslevel=9, mtime=0) as gz:
            gz.write(raw)
    dump(os.path.join(HERE, "reference_fe.json"), source="example/Fe.pbe.in",
         sha256=hashlib.sha256(raw).hexdigest(), bytes=len(raw))
    print("Fe.pbe.in.gz: sha256", hashlib.sha256(raw).hexdigest()[:16])


def main():
    checkout = os.environ.get("MAGACE_REFERENCE")
    if checkout:
        refresh_fixture(checkout)
    with tempfile.TemporaryDirectory() as td:
        if os.path.exists(FIXTURE):
            fe = os.path.join(td, "Fe.pbe.in")
            with gzip.open(FIXTURE, "rb") as gz, open(fe, "wb") as out:
                out.write(gz.read())
            o = orc.Oracle(fe, "Fe", rcut=4.5, rcut_magnetic=4.0, smear=0.2)
            nb = S.neighbor_data(S.notebook_cell(), 4.5)
            e, f, t, t0 = o.acelib(nb)
            dump(os.path.join(HERE, "notebook_fe.json"), eout=e, flist=f, tlist=t, tlist0=t0,
                 etot=float(e.sum()))
            print("notebook_fe.json: etot =", repr(float(e.sum())))
            cells = {}
            for name, st in reference_cells().items():
                nb = S.neighbor_data(st, 4.5)
                cells[name] = per_atom_summary(nb, *o.acelib(nb))
            with open(os.path.join(HERE, "reference_fe_cells.json"), "w") as fh:
                json.dump({k: {a: (b.tolist() if isinstance(b, np.ndarray) else b) for a, b in v.items()}
                           for k, v in cells.items()}, fh)
            print("reference_fe_cells.json:", {k: v["natom"] for k, v in cells.items()})
        pot = potential.write_seeded_potential(os.path.join(td, "seeded.in"), seed=2024)
        sha = hashlib.sha256(open(pot, "rb").read()).hexdigest()
        o = orc.Oracle(pot, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)
        nb = S.neighbor_data(seeded_cell16(), 5.0)
        e, f, t, t0 = o.acelib(nb)
        dump(os.path.join(HERE, "seeded_bcc16.json"), potential_sha256=sha, eout=e, flist=f, tlist=t,
             tlist0=t0)
        print("seeded_bcc16.json: sha", sha[:16], "E/atom", e.mean())


if __name__ == "__main__":
    main()
