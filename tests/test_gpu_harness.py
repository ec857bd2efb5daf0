"""The drop-in ABI driven by a C++ program the way the reference's LAMMPS pair
style drives it (tests/harness/spin_ace_driver.cpp, after
lammps/pair_spin_ace.cpp:340-646): local atoms plus ghost images, a full
neighbour list with a 1 A skin, 1-based flat arrays, acelibini_ reading
./Fe.pbe.in, acelib_ on the GPU, and the pair style's reductions of forces,
magnetic forces, energy and virial with newton_pair on and ghost forces
returned to their owners. The totals are compared with the oracle's
evaluation of the same structure (no skin) assembled in Python."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO

HARNESS = os.path.join(REPO, "tests", "harness", "spin_ace_driver.cpp")
LIBDIR = os.path.join(REPO, "mag-ace_gb300", "lib")


def _build(tmp_path) -> str:
    from magace import build
    build.build()
    exe = str(tmp_path / "spin_ace_driver")
    cc = subprocess.run(["g++", "-O2", "-std=c++17", HARNESS, "-o", exe, "-L" + LIBDIR, "-lmagace",
                         "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    return exe


def test_harness_compiles(tmp_path):
    """The driver builds against libmagace.so with the declarations the pair
    style uses (no GPU needed to link)."""
    _build(tmp_path)


def _run(exe, st, workdir, rcut, skin):
    box = [repr(float(st.cell[a, a])) for a in range(3)]
    lines = [f"{len(st.positions)} {' '.join(box)} {float(rcut)!r} {float(skin)!r} 4.0 0.2"]
    for p, m, u in zip(st.positions, st.mag, st.mhat):
        mv = m * u
        lines.append(" ".join(repr(float(v)) for v in (*p, *mv)))
    run = subprocess.run([exe], input="\n".join(lines) + "\n", cwd=workdir, capture_output=True, text=True,
                         timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    out = run.stdout.splitlines()
    energy = float(out[0].split()[1])
    virial = np.array([float(v) for v in out[1].split()[1:]])
    per = np.array([[float(v) for v in ln.split()[1:]] for ln in out[2:]])
    return energy, virial, per[:, :3], per[:, 3:]


@pytest.mark.gpu
@pytest.mark.parametrize("cell", ["bcc128_cone", "bcc54_random"])
def test_pair_style_driver_matches_oracle(tmp_path, reference_fe, oracle_fe, cell):
    import sys
    from conftest import GOLDEN
    from magace import structures as S
    sys.path.insert(0, GOLDEN)
    import make_golden as mg
    exe = _build(tmp_path)
    shutil.copy(reference_fe, tmp_path / "Fe.pbe.in")
    st = mg.reference_cells()[cell]
    # positions wrapped into the box, as an MD code holds them
    st = S.Structure(np.mod(st.positions, np.diag(st.cell)), st.cell, st.pbc, st.mag, st.mhat)
    energy, virial, F, FM = _run(exe, st, tmp_path, 4.5, 1.0)
    nb = S.neighbor_data(st, 4.5)
    e, f, t, t0 = oracle_fe.acelib(nb)
    Fo, FMo = S.total_forces(nb, f, t, t0)
    d = (nb.elist.reshape(-1, 3) * nb.dlist[:, None])
    fl = f.reshape(-1, 3)
    vo = np.array([(d[:, 0] * fl[:, 0]).sum(), (d[:, 1] * fl[:, 1]).sum(), (d[:, 2] * fl[:, 2]).sum(),
                   (d[:, 0] * fl[:, 1]).sum(), (d[:, 0] * fl[:, 2]).sum(), (d[:, 1] * fl[:, 2]).sum()])
    assert abs(energy - e.sum()) <= 1e-10 * abs(e.sum())
    for got, ref in ((F, Fo), (FM, FMo), (virial, vo)):
        assert np.abs(got - ref).max() <= 1e-10 * max(np.abs(ref).max(), 1.0)
    assert np.abs(F.sum(axis=0)).max() < 1e-9  # momentum conservation
