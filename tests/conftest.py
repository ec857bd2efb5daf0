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

REFERENCE_FE = "/root/reference/example/Fe.pbe.in"
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
def oracle_alt(alt_potential):
    import oracle as orc
    return orc.Oracle(alt_potential, "Fe", rcut=5.0, rcut_magnetic=4.0, smear=0.2)


def rel_err(a, b) -> float:
    """max |a-b| / max |b| (norm-relative, robust to components that vanish)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)
