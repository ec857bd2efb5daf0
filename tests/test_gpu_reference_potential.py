"""GPU tests on the reference's own potential, example/Fe.pbe.in (cut 4.5 A,
magnetic cutoff 4.0 mu_B, smear 0.2, pbe), through the drop-in C ABI.

  * The notebook cell (example/basic_lammps.ipynb:272): acelibini_ reads
    ./Fe.pbe.in from the working directory as the LAMMPS pair style makes it
    do, acelib_ evaluates the 2-atom bcc cell, and the total energy is the
    notebook's -15.7479878560111 eV; all four outputs equal the committed
    golden vectors (tests/golden/notebook_fe.json) within 1e-10.
  * Two non-collinear cells (128-atom bcc with moments in a 30 degree cone,
    54-atom bcc with directions uniform on the sphere): FP64 equals the live
    oracle within 1e-10 relative and the committed per-atom summaries
    (tests/golden/reference_fe_cells.json); the split precision stays within
    1 meV/atom, 10 meV/A and 10 meV/mu_B of the oracle.
"""
from __future__ import annotations

import json
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, rel_err

pytestmark = pytest.mark.gpu

NOTEBOOK_ETOT = -15.7479878560111  # example/basic_lammps.ipynb:272
TOL_FP64 = 1e-10
# split precision against the FP64 oracle: eV per atom, eV/A, eV/mu_B
TOL_SPLIT = {"energy": 1e-3, "force": 1e-2, "magforce": 1e-2}


@pytest.fixture()
def fe_lib(reference_fe):
    from magace import lib
    lib.init(reference_fe, "Fe", 4.5, 4.0, 0.2, 1)
    lib.set_precision(0)
    yield lib
    lib.set_precision(0)


# A fresh process, as a LAMMPS run is: acelibini_ exactly as the pair style
# calls it (lammps/pair_spin_ace.cpp:283-288: nele = 1, elenumbers = atomic
# number + 1, ./Fe.pbe.in found in the working directory; later calls are
# no-ops, src/util.F90:29-33), then acelib_ on the notebook cell.
_DROP_IN = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from magace import lib, structures as S
so = lib.load()
nele, xc, el = ctypes.c_int(1), ctypes.c_int(1), (ctypes.c_int * 1)(27)
rc, rcm, sm = ctypes.c_double(4.5), ctypes.c_double(4.0), ctypes.c_double(0.2)
so.acelibini_(ctypes.byref(nele), ctypes.byref(rc), ctypes.byref(rcm), ctypes.byref(sm), ctypes.byref(xc), el)
assert so.ace_last_error() == 0, so.ace_last_error_message()
nb = S.neighbor_data(S.notebook_cell(), 4.5)
e, f, t, t0 = lib.acelib(nb)
np.savez(sys.argv[2], e=e, f=f, t=t, t0=t0, counts=nb.nstop - nb.nstart + 1)
"""


def test_notebook_cell_through_acelibini(reference_fe, tmp_path):
    import subprocess
    import sys

    from conftest import REPO
    from magace import structures as S
    shutil.copy(reference_fe, tmp_path / "Fe.pbe.in")
    out = tmp_path / "out.npz"
    run = subprocess.run([sys.executable, "-c", _DROP_IN, os.path.join(REPO, "mag-ace_gb300"), str(out)],
                         cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    r = np.load(out)
    assert np.all(r["counts"] == 26)  # 8 + 6 + 12 neighbours within 4.5 A
    e, f, t, t0 = r["e"], r["f"], r["t"], r["t0"]
    assert abs(e.sum() - NOTEBOOK_ETOT) <= 1e-12 * abs(NOTEBOOK_ETOT)
    with open(os.path.join(GOLDEN, "notebook_fe.json")) as fh:
        g = json.load(fh)
    # forces vanish by symmetry here (example/basic_lammps.ipynb:292-293), so
    # every output is compared with an absolute floor of 1e-10 of the energy scale
    for got, key in ((e, "eout"), (f, "flist"), (t, "tlist"), (t0, "tlist0")):
        ref = np.asarray(g[key])
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(got - ref).max() <= TOL_FP64 * scale, key
    nb = S.neighbor_data(S.notebook_cell(), 4.5)
    F, FM = S.total_forces(nb, f, t, t0)
    assert np.abs(F).max() < 1e-10


def test_notebook_cell_split_precision(fe_lib):
    from magace import structures as S
    fe_lib.set_precision(1)
    nb = S.neighbor_data(S.notebook_cell(), 4.5)
    e, f, t, t0 = fe_lib.acelib(nb)
    assert abs(e.sum() - NOTEBOOK_ETOT) / 2 <= TOL_SPLIT["energy"]


def _cells():
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as mg
    return mg


@pytest.mark.parametrize("cell", ["bcc128_cone", "bcc54_random"])
def test_noncollinear_cells_fp64(fe_lib, oracle_fe, cell):
    from magace import structures as S
    mg = _cells()
    nb = S.neighbor_data(mg.reference_cells()[cell], 4.5)
    e, f, t, t0 = fe_lib.acelib(nb)
    eo, fo, to, t0o = oracle_fe.acelib(nb)
    for name, a, b in (("energy", e, eo), ("flist", f, fo), ("tlist", t, to), ("tlist0", t0, t0o)):
        assert rel_err(a, b) <= TOL_FP64, (name, rel_err(a, b))
    assert np.abs(f).max() > 1e-3 and np.abs(t).max() > 1e-4  # non-trivial forces and magnetic forces
    with open(os.path.join(GOLDEN, "reference_fe_cells.json")) as fh:
        g = json.load(fh)[cell]
    got = mg.per_atom_summary(nb, e, f, t, t0)
    for k in ("eout", "tlist0", "fsum", "tsum"):
        assert rel_err(got[k], g[k]) <= TOL_FP64, k
    for k in ("f_sumsq", "t_sumsq"):
        assert abs(got[k] - g[k]) <= TOL_FP64 * g[k], k


@pytest.mark.parametrize("cell", ["bcc128_cone", "bcc54_random"])
def test_noncollinear_cells_split(fe_lib, oracle_fe, cell):
    from magace import structures as S
    mg = _cells()
    nb = S.neighbor_data(mg.reference_cells()[cell], 4.5)
    fe_lib.set_precision(1)
    e, f, t, t0 = fe_lib.acelib(nb)
    eo, fo, to, t0o = oracle_fe.acelib(nb)
    assert np.abs(e - eo).max() <= TOL_SPLIT["energy"]
    assert np.abs(f - fo).max() <= TOL_SPLIT["force"]
    assert max(np.abs(t - to).max(), np.abs(t0 - t0o).max()) <= TOL_SPLIT["magforce"]
    assert rel_err(f, fo) <= 1e-4
