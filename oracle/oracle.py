"""ctypes wrapper around the CPU FP64 oracle (oracle/_build/liboracle*.so).

TEST INFRASTRUCTURE ONLY: this is the parity checker and the CPU baseline.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
it; the product path never does.

The oracle restates the reference Fortran (mttrin93/mag-ace src/*.F90); its
entry points mirror acelibini/acelib (src/ace.F90:10-321).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

_current = [None]  # (library id, init arguments) of the state the library holds

_i = ctypes.c_int
_d = ctypes.c_double
_pi = ctypes.POINTER(ctypes.c_int)
_pd = ctypes.POINTER(ctypes.c_double)


def build(quiet: bool = True) -> None:
    """Compiles the oracle with its Makefile (g++ only, a few seconds)."""
    out = subprocess.run(["make", "-C", HERE, "-j2"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_libs: dict = {}


def _load(fast: bool) -> ctypes.CDLL:
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name in _libs:
        return _libs[name]
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    lib.oracle_init.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _d, _d, _d, _i]
    lib.oracle_init.restype = _i
    lib.oracle_last_error.restype = ctypes.c_char_p
    lib.oracle_basis_sizes.argtypes = [_pi]
    lib.oracle_basis_sizes.restype = _i
    lib.oracle_basis_rows.argtypes = [_i, _pi]
    lib.oracle_basis_rows.restype = _i
    lib.oracle_acelib.argtypes = [_i, _i, _i, _pi, _pi, _pi, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd,
                                  _pd, _pd, _pd, _pd, _i, _i]
    lib.oracle_acelib.restype = _i
    lib.oracle_atom_state.argtypes = [_i, _i, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _i, _pd, _pd,
                                      _pd, _pd, _pd, _pd, _pd, _pd]
    lib.oracle_atom_state.restype = _i
    lib.oracle_descriptors.argtypes = [_i, _i, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd, _pd]
    lib.oracle_descriptors.restype = _i
    _libs[name] = lib
    return lib


def _ip(a):
    return a.ctypes.data_as(_pi)


def _dp(a):
    return a.ctypes.data_as(_pd)


class Oracle:
    """One oracle instance (the library keeps module-global state, like the
    reference; two Oracle objects on the same .so share it)."""

    def __init__(self, potfile: str, element: str = "Fe", rcut: float = 5.0,
                 rcut_magnetic: float = 4.0, smear: float = 0.2, xcnumber: int = 1,
                 fast: bool = False):
        self.lib = _load(fast)
        self._key = (potfile, element, rcut, rcut_magnetic, smear, xcnumber)
        self._activate(force=True)
        sz = np.zeros(9, dtype=np.int32)
        self.lib.oracle_basis_sizes(_ip(sz))
        self.nvar = tuple(int(x) for x in sz[:4]) + (int(sz[7]), int(sz[8]))
        self.nterms3, self.nterms4, self.nterms2 = int(sz[4]), int(sz[5]), int(sz[6])

    def _activate(self, force: bool = False) -> None:
        """The library keeps one global state; re-initialise it when another
        Oracle object used it last."""
        if force or _current[0] != (id(self.lib), self._key):
            st = self.lib.oracle_init(self._key[0].encode(), self._key[1].encode(), *self._key[2:])
            if st != 0:
                raise RuntimeError(f"oracle_init failed ({st}): "
                                   + self.lib.oracle_last_error().decode())
            _current[0] = (id(self.lib), self._key)

    def basis_rows(self, rank: int) -> np.ndarray:
        self._activate()
        width = {1: 1, 2: 4, 3: 9, 4: 15, 5: 21, 6: 27}[rank]
        n = self.nvar[rank - 1]
        out = np.zeros(max(1, n) * width, dtype=np.int32)
        st = self.lib.oracle_basis_rows(rank, _ip(out))
        if st:
            raise RuntimeError("oracle_basis_rows failed")
        return out[: n * width].reshape(n, width)

    def acelib(self, nb, nthreads: int = 1, chunk: int = 64):
        """Runs the restated acelib on a NeighborData-like object `nb`
        (attributes as the C-ABI arrays). Returns (eout, flist, tlist, tlist0)."""
        self._activate()
        natom, nei = nb.natom, nb.nei
        eout = np.zeros(natom)
        flist = np.zeros(3 * nei)
        tlist = np.zeros(3 * nei)
        tlist0 = np.zeros(3 * natom)
        st = self.lib.oracle_acelib(natom, nb.nall, nei, _ip(nb.nlist), _ip(nb.occ), _ip(nb.occlist),
                                    _ip(nb.nstart), _ip(nb.nstop), _dp(eout), _dp(nb.dlist),
                                    _dp(nb.elist), _dp(flist), _dp(nb.dlist_momi), _dp(nb.elist_momi),
                                    _dp(nb.dlist_mom), _dp(nb.elist_mom), _dp(tlist), _dp(tlist0),
                                    nthreads, chunk)
        if st:
            raise RuntimeError(f"oracle_acelib failed ({st}): "
                               + self.lib.oracle_last_error().decode())
        return eout, flist, tlist, tlist0

    def descriptors(self, nb):
        """(B [natom, nvar1+..+nvar6], dE/drho [natom, 2]) of every atom."""
        self._activate()
        nB = sum(self.nvar)
        B = np.zeros((max(1, nb.natom), nB))
        dedrho = np.zeros((max(1, nb.natom), 2))
        st = self.lib.oracle_descriptors(nb.natom, nb.nei, _ip(nb.nstart), _ip(nb.nstop), _dp(nb.dlist),
                                         _dp(nb.elist), _dp(nb.dlist_momi), _dp(nb.elist_momi),
                                         _dp(nb.dlist_mom), _dp(nb.elist_mom), _dp(B), _dp(dedrho))
        if st:
            raise RuntimeError(f"oracle_descriptors failed ({st}): " + self.lib.oracle_last_error().decode())
        return B[: nb.natom], dedrho[: nb.natom]

    def atom_state(self, nb, atom: int, dims: dict) -> dict:
        """Intermediates of one atom (0-based `atom`); `dims` gives the basis
        dims (nradial3_a, lmaxsq_a, ...)."""
        self._activate()
        d = dims
        nA = d["n3a"] * d["lsa"] * d["n3m"] * d["lsm"]
        nA2 = d["nba"] * d["n2m"] * d["lsm"]
        nA0 = d["n2m"] * d["lsm"]
        nwf = (2 * d["l3a"] + 1) * (d["l3a"] + 1) * d["n3a"] * (d["l3m"] + 1) ** 2 * d["n3m"]
        nwf2 = d["nba"] * (d["l2m"] + 1) ** 2 * d["n2m"]
        nwf0 = (d["l2m"] + 1) ** 2 * d["n2m"]
        A = np.zeros(2 * nA)
        A2 = np.zeros(2 * nA2)
        A0 = np.zeros(2 * nA0)
        wf = np.zeros(2 * nwf)
        wf2 = np.zeros(2 * nwf2)
        wf0 = np.zeros(2 * nwf0)
        wf1 = np.zeros(d["nbm"])
        scal = np.zeros(8)
        st = self.lib.oracle_atom_state(nb.natom, nb.nei, _ip(nb.nstart), _ip(nb.nstop),
                                        _dp(nb.dlist), _dp(nb.elist), _dp(nb.dlist_momi),
                                        _dp(nb.elist_momi), _dp(nb.dlist_mom), _dp(nb.elist_mom),
                                        atom + 1, _dp(A), _dp(A2), _dp(A0), _dp(wf), _dp(wf2),
                                        _dp(wf0), _dp(wf1), _dp(scal))
        if st:
            raise RuntimeError(f"oracle_atom_state failed ({st})")
        c = lambda a: a[0::2] + 1j * a[1::2]
        return {"A": c(A), "A2": c(A2), "A0": c(A0), "wf": c(wf), "wf2": c(wf2), "wf0": c(wf0),
                "wf1": wf1, "energy": scal[0], "rho": scal[1:3], "dEdrho": scal[3:5],
                "core": scal[5], "edf": scal[6]}
