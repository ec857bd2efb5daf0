"""Device-resident spin-lattice MD over the library (ace_md_* C ABI).

The integrator and neighbour list run on the GPU; this class only sets up
the state (Maxwell velocities, moments from |m| and directions) and reads
results back. Units: A, ps, eV, amu, mu_B.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib

KB = 8.617333262e-5             # eV/K
ACCEL = 9648.53321233100        # (eV/A)/amu -> A/ps^2
FE_MASS = 55.845                # amu


def maxwell_velocities(n: int, temperature: float, mass: float, rng: np.random.Generator) -> np.ndarray:
    """Velocities (A/ps) from the Maxwell distribution at `temperature` K,
    without centre-of-mass motion."""
    sigma = np.sqrt(KB * temperature * ACCEL / mass)
    v = rng.normal(0.0, sigma, size=(n, 3))
    return v - v.mean(axis=0)


class SpinLatticeMD:
    def __init__(self, structure, temperature: float = 300.0, seed: int = 0, mass: float = FE_MASS,
                 rcut: float = 5.0, skin: float = 0.5):
        rng = np.random.default_rng(seed)
        self.natom = len(structure.positions)
        x = np.ascontiguousarray(structure.positions, dtype=np.float64)
        v = np.ascontiguousarray(maxwell_velocities(self.natom, temperature, mass, rng))
        m = np.ascontiguousarray(structure.mag[:, None] * structure.mhat, dtype=np.float64)
        cell = np.ascontiguousarray(structure.cell, dtype=np.float64)
        pbc = np.asarray([1 if p else 0 for p in structure.pbc], dtype=np.int32)
        h = ctypes.c_int()
        lib._check(lib.load().ace_md_create(self.natom, lib._dp(x), lib._dp(v), lib._dp(m), lib._dp(cell),
                                            lib._ip(pbc), mass, rcut, skin, ctypes.byref(h)))
        self.handle = h.value

    def run(self, nsteps: int, dt: float = 0.001, rebuild_every: int = 10, use_graph: bool = True) -> np.ndarray:
        """Runs nsteps steps; returns [nsteps + 1, 2] total potential and
        kinetic energies (eV) of the start and after each step."""
        log = np.zeros((nsteps + 1, 2))
        lib._check(lib.load().ace_md_run(self.handle, nsteps, dt, rebuild_every, 1 if use_graph else 0,
                                         lib._dp(log)))
        return log

    def state(self) -> dict:
        a = {k: np.zeros((self.natom, 3)) for k in ("x", "v", "m", "F", "fm")}
        lib._check(lib.load().ace_md_state(self.handle, *[lib._dp(a[k]) for k in ("x", "v", "m", "F", "fm")]))
        return a

    def bonds(self) -> dict:
        nb = ctypes.c_int()
        lib._check(lib.load().ace_md_bonds(self.handle, ctypes.byref(nb), None, None, None, None))
        off = np.zeros(self.natom + 1, np.int32)
        j, shift, rev = (np.zeros(nb.value, np.int32) for _ in range(3))
        lib._check(lib.load().ace_md_bonds(self.handle, ctypes.byref(nb), lib._ip(off), lib._ip(j), lib._ip(shift),
                                           lib._ip(rev)))
        sh = np.stack([(shift & 0xff) - 128, ((shift >> 8) & 0xff) - 128, ((shift >> 16) & 0xff) - 128], axis=1)
        return {"off": off, "j": j, "shift": sh, "rev": rev}

    def close(self) -> None:
        if self.handle:
            lib.load().ace_md_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
