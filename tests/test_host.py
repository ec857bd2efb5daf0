"""CPU tests of the product library's host side: it loads, exports every
symbol include/magace.h declares, initialises without a GPU, enumerates the
same basis as the oracle and reports the reference's fatal conditions as
status codes. No compute call is made here."""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, REPO


@pytest.fixture(scope="module")
def lib():
    from magace import build, lib as L
    build.build()
    L.load()
    return L


def header_symbols():
    text = open(os.path.join(REPO, "include", "magace.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(\w+)\s*\([^;{]*\)\s*;", text)) - {"defined"})


def test_exports_every_declared_symbol(lib):
    names = header_symbols()
    assert "acelib_" in names and "acelibini_" in names and len(names) >= 15
    so = ctypes.CDLL(lib.LIB_PATH)
    for n in names:
        assert hasattr(so, n), n
    assert set(names) == set(lib.SIGNATURES), "binding table out of sync with the header"


def test_init_and_basis_match_oracle(lib, seeded_potential, oracle_seeded):
    lib.init(seeded_potential, "Fe", 5.0, 4.0, 0.2, 1)
    sz = lib.basis_sizes()
    assert sz["nvar"] == (16, 720, 4932, 495)
    assert (sz["nterms2"], sz["nterms3"], sz["nterms4"]) == (2160, 64008, 495)
    assert sz["unmatched"] == 0
    for r in (1, 2, 3, 4):
        assert np.array_equal(lib.basis_rows(r), oracle_seeded.basis_rows(r))


def test_high_body_enumeration_matches_oracle(lib, high_potential, oracle_high):
    """5- and 6-body clusters: the library's enumeration (model.cpp) and the
    oracle's restatement of src/util.F90:2817-3760, written separately,
    give the same rows in the same order, including the clusters whose
    atomic or magnetic half the reference pads with zeros."""
    lib.init(high_potential, "Fe", 5.0, 4.0, 0.2, 1)
    for r in (1, 2, 3, 4, 5, 6):
        assert np.array_equal(lib.basis_rows(r), oracle_high.basis_rows(r)), r
    r5, r6 = lib.basis_rows(5), lib.basis_rows(6)
    assert len(r5) > 0 and len(r6) > 0
    assert (r5[:, 0] == 0).any() and (r5[:, 4] == 0).any()  # padded halves exist
    assert lib.basis_sizes()["unmatched"] == 0
    assert lib.num_coefficients()[0] == sum(len(lib.basis_rows(r)) for r in range(1, 7))


def test_reference_potential_matches_enumeration(lib, reference_fe):
    lib.init(reference_fe, "Fe", 4.5, 4.0, 0.2, 1)
    sz = lib.basis_sizes()
    # every record of example/Fe.pbe.in is an enumerated cluster
    assert sz["nvar"] == (16, 720, 4932, 495) and sz["unmatched"] == 0


def test_seeded_potential_is_reproducible(tmp_path):
    from magace import potential
    p = potential.write_seeded_potential(str(tmp_path / "Fe.pbe.in"), seed=2024)
    sha = hashlib.sha256(open(p, "rb").read()).hexdigest()
    g = json.load(open(os.path.join(GOLDEN, "seeded_bcc16.json")))
    assert sha == g["potential_sha256"]


def test_error_codes(lib, tmp_path, seeded_potential):
    from magace.lib import MagAceError
    with pytest.raises(MagAceError) as e:
        lib.init(str(tmp_path / "missing.in"))
    assert e.value.code == 1
    with pytest.raises(MagAceError) as e:
        lib.init(seeded_potential, element="Co")
    assert e.value.code == 2
    with pytest.raises(MagAceError) as e:
        lib.init(seeded_potential, smear=0.3)
    assert e.value.code == 2
    with pytest.raises(MagAceError) as e:
        lib.init(seeded_potential, xcnumber=3)
    assert e.value.code == 7
    with pytest.raises(MagAceError) as e:
        lib.init(seeded_potential, rcut=4.0)  # shorter than the file's 5.0 A
    assert e.value.code == 2
    # 5-/6-body dims the A basis does not hold (n' beyond nradial3_magnetic = 3),
    # and 6-body clusters without 5-body ones (the reference skips them), are refused
    text = open(seeded_potential).read()
    for old, new in ((" nradial5 l5max   0 0 0 0", " nradial5 l5max   1 4 0 0"),
                     (" nradial6 l6max   0 0 0 0", " nradial6 l6max   1 1 0 0")):
        p5 = tmp_path / "high.in"
        p5.write_text(text.replace(old, new))
        with pytest.raises(MagAceError) as e:
            lib.init(str(p5))
        assert e.value.code == 3
    assert lib.load().ace_error_string(4).decode().startswith("bond shorter")
    # kernel variants: indices outside a kernel's range are refused, valid ones kept
    before = lib.get_tuning_indices()
    for bad in ([6, 0, 0, 0], [0, 6, 0, 0], [0, 0, -1, 0], [0, 0, 0, 8]):
        with pytest.raises(MagAceError) as e:
            lib.set_tuning(bad)
        assert e.value.code == 7
    assert lib.get_tuning_indices() == before
    lib.set_tuning([3, 5, 5, 7])
    assert lib.get_tuning_indices() == [3, 5, 5, 7]
    assert lib.get_tuning()["abasis"] == "scalar, TMA-staged bond tiles, persistent grid"
    assert lib.get_tuning()["forces"] == "6 CTAs/SM, tensor cores (3xTF32)"
    lib.set_tuning(before)


def test_call_size_limits(lib):
    """The kernels index per-bond vectors as 3 j with 32-bit j: a call with
    more than 715,827,882 bonds or atoms is refused with MAGACE_ERR_ARGS
    before any device work, like negative sizes."""
    so = lib.load()
    for natom, nei in ((0, 715_827_883), (715_827_883, 0), (-1, 0), (0, -5)):
        assert so.ace_compute_device(natom, nei, *[None] * 12) == 7
        assert so.ace_descriptors_device(natom, nei, *[None] * 9) == 7
        assert so.ace_compute_device_noalloc(natom, nei, *[None] * 12) == 7
    n, big = ctypes.c_int(0), ctypes.c_int(715_827_883)
    so.acelib_(ctypes.byref(n), ctypes.byref(n), ctypes.byref(big), *[None] * 15)
    assert so.ace_last_error() == 7


def test_plain_c_caller_links(lib, tmp_path, seeded_potential):
    """A C program that declares the two entry points by their argument lists
    alone, as the pair style does (lammps/pair_spin_ace.cpp:59-62: every
    argument by reference, gfortran naming), links against libmagace.so,
    initialises from the working directory and gets a status code back."""
    import shutil
    import subprocess
    src = tmp_path / "caller.c"
    src.write_text(r"""
extern void acelibini_(int*, double*, double*, double*, int*, int*);
extern void acelib_(int*, int*, int*, int*, int*, int*, int*, int*, double*, double*, double*, double*,
                    double*, double*, double*, double*, double*, double*);
extern int ace_last_error(void);
int main(void) {
  int nele = 1, xc = 1, el[1] = {27}; /* Fe: atomic number + 1 */
  double rcut = 5.0, rcut_mag = 4.0, smear = 0.2;
  acelibini_(&nele, &rcut, &rcut_mag, &smear, &xc, el);
  if (ace_last_error() != 0) return 1;
  int natom = -1, nall = 0, nei = 0; /* refused before any device work */
  acelib_(&natom, &nall, &nei, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0);
  return ace_last_error() == 7 ? 0 : 2;
}
""")
    libdir = os.path.dirname(lib.LIB_PATH)
    exe = tmp_path / "caller"
    cc = subprocess.run(["gcc", str(src), "-o", str(exe), "-L" + libdir, "-lmagace", "-Wl,-rpath," + libdir],
                        capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    shutil.copy(seeded_potential, tmp_path / "Fe.pbe.in")
    run = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr


def test_acelibini_reads_working_directory(lib, tmp_path, seeded_potential, monkeypatch):
    """acelibini_(nele=1, ..., elenumbers=[27]) opens ./Fe.pbe.in
    (src/util.F90:525; 27 = atomic number 26 + 1)."""
    so = lib.load()
    import shutil
    shutil.copy(seeded_potential, tmp_path / "Fe.pbe.in")
    monkeypatch.chdir(tmp_path)
    nele = ctypes.c_int(2)
    rc, rcm, sm, xc = ctypes.c_double(5.0), ctypes.c_double(4.0), ctypes.c_double(0.2), ctypes.c_int(1)
    el = (ctypes.c_int * 1)(27)
    so.acelibini_(ctypes.byref(nele), ctypes.byref(rc), ctypes.byref(rcm), ctypes.byref(sm), ctypes.byref(xc), el)
    assert so.ace_last_error() == 3  # more than one element is refused, as in src/ace.F90:46-49
    nele.value = 1
    so.acelibini_(ctypes.byref(nele), ctypes.byref(rc), ctypes.byref(rcm), ctypes.byref(sm), ctypes.byref(xc), el)
    assert so.ace_last_error() == 0
    assert lib.basis_sizes()["nvar"][2] == 4932


def test_acelib_before_init_reports_error(tmp_path):
    """A fresh process: acelib_ without init records NOT_INIT and fills NaN."""
    import subprocess
    import sys
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r);"
        "from magace import lib, structures as S;"
        "nb = S.neighbor_data(S.notebook_cell(), 5.0);"
        "\ntry:\n    lib.acelib(nb)\nexcept lib.MagAceError as e:\n    print('code', e.code)"
    ) % os.path.join(REPO, "mag-ace_gb300")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert "code 6" in out.stdout, out.stdout + out.stderr
