"""Generates the golden vectors under tests/golden/ with the CPU oracle.

  notebook_fe.json   the reference's example cell (2-atom cubic bcc Fe,
                     a = 2.83 A, m = (0,0,2.22) mu_B, example/Fe.pbe.in,
                     rcut 4.5 / 4.0, smear 0.2) -- needs the reference checkout;
                     its total energy is the notebook's -15.7479878560111 eV.
  seeded_bcc16.json  the seeded synthetic potential (seed 2024) on a jittered
                     16-atom bcc cell, plus the sha256 of the generated
                     potential file so its generation stays reproducible.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

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

REFERENCE_FE = "/root/reference/example/Fe.pbe.in"


def seeded_cell16():
    rng = np.random.default_rng(16)
    pos, cell = S.bcc_cubic(2, 2, 2, 2.83)
    pos = pos + rng.normal(0.0, 0.05, pos.shape)
    n = len(pos)
    return S.Structure(pos, cell, (True, True, True), rng.uniform(2.0, 2.4, n), S.cone_unit(rng, n, 30.0))


def dump(path, **arrays):
    with open(path, "w") as fh:
        json.dump({k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in arrays.items()}, fh)


def main():
    if os.path.exists(REFERENCE_FE):
        o = orc.Oracle(REFERENCE_FE, "Fe", rcut=4.5, rcut_magnetic=4.0, smear=0.2)
        nb = S.neighbor_data(S.notebook_cell(), 4.5)
        e, f, t, t0 = o.acelib(nb)
        dump(os.path.join(HERE, "notebook_fe.json"), eout=e, flist=f, tlist=t, tlist0=t0,
             etot=float(e.sum()))
        print("notebook_fe.json: etot =", repr(float(e.sum())))
    with tempfile.TemporaryDirectory() as td:
        pot = potential.write_seeded_potential(os.path.join(td, "Fe.pbe.in"), seed=2024)
        sha = hashlib.sha256(open(pot, "rb").read()).hexdigest()
        o = orc.Oracle(pot, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)
        nb = S.neighbor_data(seeded_cell16(), 5.0)
        e, f, t, t0 = o.acelib(nb)
        dump(os.path.join(HERE, "seeded_bcc16.json"), potential_sha256=sha, eout=e, flist=f, tlist=t,
             tlist0=t0)
        print("seeded_bcc16.json: sha", sha[:16], "E/atom", e.mean())


if __name__ == "__main__":
    main()
