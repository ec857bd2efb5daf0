"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "mag-ace_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def seeded_potential(tmp_path_factory):
    """The seeded potential in the Fe.pbe.in layout (cut 5.0 A / 4.0 mu_B)."""
    from magace import potential
    path = str(tmp_path_factory.mktemp("pot") / "Fe.pbe.in")
    potential.write_seeded_potential(path, seed=2024)
    return path


@pytest.fixture(scope="session")
def reference_fe(tmp_path_factory):
    """The reference's example potential example/Fe.pbe.in (cut 4.5 A /
    4.0 mu_B), unpacked from the committed fixture tests/golden/Fe.pbe.in.gz
    into a directory of its own and checked against its pinned sha256."""
    import gzip
    import hashlib
    import json
    meta = json.load(open(os.path.join(GOLDEN, "reference_fe.json")))
    with gzip.open(os.path.join(GOLDEN, "Fe.pbe.in.gz"), "rb") as gz:
        raw = gz.read()
    assert hashlib.sha256(raw).hexdigest() == meta["sha256"], "Fe.pbe.in fixture does not match its pinned hash"
    path = tmp_path_factory.mktemp("reference_fe") / "Fe.pbe.in"
    path.write_bytes(raw)
    return str(path)


@pytest.fixture(scope="session")
def oracle_fe(reference_fe):
    import oracle as orc
    return orc.Oracle(reference_fe, "Fe", rcut=4.5, rcut_magnetic=4.0, smear=0.2)


@pytest.fixture(scope="session")
def oracle_seeded(seeded_potential):
    import oracle as orc
    return orc.Oracle(seeded_potential, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)


@pytest.fixture(scope="session")
def alt_potential(tmp_path_factory):
    """A second seeded potential in a smaller layout with two densities, a
    non-linear embedding and 4-body clusters with l = 1 (evaluated by the
    generic kernels)."""
    from magace import potential
    path = str(tmp_path_factory.mktemp("alt") / "Fe.pbe.in")
    potential.write_seeded_potential(path, seed=5, layout=potential.ALT_LAYOUT, par=(1.0, 0.5), par2=(0.7, 0.8))
    return path


@pytest.fixture(scope="session")
def high_potential(tmp_path_factory):
    """A seeded potential with 5- and 6-body clusters (HIGH_LAYOUT: radial
    types 4/8, a non-linear embedding exponent 0.5); it runs on the
    generic kernels."""
    from magace import potential
    path = str(tmp_path_factory.mktemp("high") / "Fe.pbe.in")
    potential.write_seeded_potential(path, seed=7, layout=potential.HIGH_LAYOUT, par=(1.0, 0.5))
    return path


@pytest.fixture(scope="session")
def oracle_high(high_potential):
    import oracle as orc
    return orc.Oracle(high_potential, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)


RADTYPE_PAIRS = ((6, 5), (4, 6))  # (atomic, magnetic) radial basis types beyond the other layouts' 3/7, 5/3, 4/8


@pytest.fixture(scope="session", params=RADTYPE_PAIRS, ids=lambda p: f"radtypes{p[0]}{p[1]}")
def radtype_potential(request, tmp_path_factory):
    """Seeded potentials in the Fe layout (so the specialised kernels run)
    with other radial basis types, type 6 in either role."""
    from magace import potential
    ra, rm = request.param
    path = str(tmp_path_factory.mktemp(f"rt{ra}{rm}") / "Fe.pbe.in")
    potential.write_seeded_potential(path, seed=11 + ra, layout=dict(potential.FE_LAYOUT, radtype_a=ra, radtype_m=rm))
    return path


@pytest.fixture(scope="session")
def oracle_radtype(radtype_potential):
    import oracle as orc
    return orc.Oracle(radtype_potential, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)


@pytest.fixture(scope="session")
def oracle_alt(alt_potential):
    import oracle as orc
    return orc.Oracle(alt_potential, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)


def rel_err(a, b) -> float:
    """max |a-b| / max |b| (norm-relative, robust to components that vanish)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)
