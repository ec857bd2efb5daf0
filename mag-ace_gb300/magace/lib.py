"""ctypes binding of libmagace.so, the C ABI declared in include/magace.h.

The product path is this library only: there is no CPU fallback. Loading
fails with an explicit error when the library has not been built, and
evaluation calls fail when no CUDA device is present.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libmagace.so")

MAGACE_OK = 0
ERR_NAMES = {0: "OK", 1: "FILE", 2: "FORMAT", 3: "UNSUPPORTED", 4: "SMALL_R", 5: "MOMENT",
             6: "NOT_INIT", 7: "ARGS", 8: "CUDA", 9: "NAN"}

_i = ctypes.c_int
_d = ctypes.c_double
_pi = ctypes.POINTER(ctypes.c_int)
_pd = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

# every symbol include/magace.h declares, with (restype, argtypes)
SIGNATURES = {
    "acelibini_": (None, [_pi, _pd, _pd, _pd, _pi, _pi]),
    "acelib_": (None, [_pi, _pi, _pi, _pi, _pi, _pi, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd, _pd,
                       _pd, _pd]),
    "ace_last_error": (_i, []),
    "ace_error_string": (ctypes.c_char_p, [_i]),
    "ace_last_error_message": (ctypes.c_char_p, []),
    "ace_clear_error": (None, []),
    "ace_init_file": (_i, [ctypes.c_char_p, ctypes.c_char_p, _d, _d, _d, _i]),
    "ace_set_precision": (_i, [_i]),
    "ace_get_precision": (_i, []),
    "ace_basis_sizes": (_i, [_pi]),
    "ace_basis_rows": (_i, [_i, _pi]),
    "ace_basis_count": (_i, [_i, _pi]),
    "ace_compute_device": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ace_device_status": (_i, []),
    "ace_last_launch_count": (_i, []),
    "ace_release_device": (None, []),
    "ace_set_kernel_timing": (_i, [_i]),
    "ace_kernel_times": (_i, [ctypes.POINTER(ctypes.c_float)]),
    "ace_table_stats": (_i, [ctypes.POINTER(ctypes.c_longlong)]),
    "ace_compute_device_noalloc": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ace_host_access_mode": (_i, []),
    "ace_num_coefficients": (_i, [_pi, _pi]),
    "ace_set_work_queue": (_i, [_i]),
    "ace_get_tuning": (_i, [_pi]),
    "ace_set_tuning": (_i, [_pi]),
    "ace_autotune_device": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _pi, _pi, _pi]),
    "ace_md_create": (_i, [_i, _pd, _pd, _pd, _pd, _pi, _d, _d, _d, _pi]),
    "ace_md_run": (_i, [_i, _i, _d, _i, _i, _pd]),
    "ace_md_state": (_i, [_i, _pd, _pd, _pd, _pd, _pd]),
    "ace_md_bonds": (_i, [_i, _pi, _pi, _pi, _pi, _pi]),
    "ace_md_destroy": (_i, [_i]),
    "ace_get_coefficients": (_i, [_pd]),
    "ace_set_coefficients": (_i, [_pd]),
    "ace_descriptors_device": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ace_density_gradient_device": (_i, [_i, _vp, _vp]),
    "ace_descriptors_tangent_device": (_i, [_i, _i] + [_vp] * 14 + [_vp]),
    "ace_embedding": (_i, [_pi, _pd, _pd]),
}

_lib = None


class MagAceError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"magace error {code} ({ERR_NAMES.get(code, '?')}): {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libmagace.so (once). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libmagace.so not found at {path}; build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(code: int) -> None:
    if code != MAGACE_OK:
        lib = load()
        raise MagAceError(code, lib.ace_last_error_message().decode())


def _ip(a):
    return a.ctypes.data_as(_pi)


def _dp(a):
    return a.ctypes.data_as(_pd)


def init(path: str, element: str = "Fe", rcut: float = 5.0, rcut_magnetic: float = 4.0,
         smear: float = 0.2, xcnumber: int = 1) -> None:
    lib = load()
    _check(lib.ace_init_file(path.encode(), element.encode(), rcut, rcut_magnetic, smear, xcnumber))


def set_precision(mode: int) -> None:
    _check(load().ace_set_precision(mode))


def basis_sizes() -> dict:
    out = np.zeros(8, dtype=np.int32)
    _check(load().ace_basis_sizes(_ip(out)))
    return {"nvar": tuple(int(x) for x in out[:4]), "nterms2": int(out[4]), "nterms3": int(out[5]),
            "nterms4": int(out[6]), "unmatched": int(out[7])}


def basis_count(rank: int) -> int:
    """Number of clusters of rank 1..6 of the loaded potential."""
    n = ctypes.c_int()
    _check(load().ace_basis_count(rank, ctypes.byref(n)))
    return n.value


def basis_rows(rank: int) -> np.ndarray:
    """Cluster index rows of rank 1..6 as in the file's 'clu' records."""
    width = {1: 1, 2: 4, 3: 9, 4: 15, 5: 21, 6: 27}[rank]
    n = basis_count(rank)
    out = np.zeros(max(1, n * width), dtype=np.int32)
    _check(load().ace_basis_rows(rank, _ip(out)))
    return out[: n * width].reshape(n, width)


def acelib(nb, out=None):
    """Calls the drop-in acelib_ exactly as the LAMMPS pair style does, with
    host arrays. Returns (eout, flist, tlist, tlist0); `out` reuses a previous
    call's arrays, as an MD code reuses its own between steps."""
    lib = load()
    natom, nei, nall = ctypes.c_int(nb.natom), ctypes.c_int(nb.nei), ctypes.c_int(nb.nall)
    if out is None:
        eout, flist, tlist, tlist0 = np.zeros(nb.natom), np.zeros(3 * nb.nei), np.zeros(3 * nb.nei), np.zeros(3 * nb.natom)
    else:
        eout, flist, tlist, tlist0 = out
        assert eout.size == nb.natom and flist.size == 3 * nb.nei and tlist0.size == 3 * nb.natom
    lib.acelib_(ctypes.byref(natom), ctypes.byref(nall), ctypes.byref(nei), _ip(nb.nlist), _ip(nb.occ),
                _ip(nb.occlist), _ip(nb.nstart), _ip(nb.nstop), _dp(eout), _dp(nb.dlist), _dp(nb.elist),
                _dp(flist), _dp(nb.dlist_momi), _dp(nb.elist_momi), _dp(nb.dlist_mom), _dp(nb.elist_mom),
                _dp(tlist), _dp(tlist0))
    _check(lib.ace_last_error())
    return eout, flist, tlist, tlist0


def compute_device(natom, nei, off, r, e, magj, mhj, magi, mhi, energy, fij, tij, ti0, stream=0) -> None:
    """Device-pointer evaluation; every array argument is an integer device
    address (e.g. torch.Tensor.data_ptr())."""
    _check(load().ace_compute_device(natom, nei, off, r, e, magj, mhj, magi, mhi, energy, fij, tij, ti0,
                                     stream))


def set_work_queue(on: bool) -> None:
    """Neighbour-count-sorted work queue for the following evaluations."""
    _check(load().ace_set_work_queue(1 if on else 0))


def autotune_device(natom, nei, off, r, e, magj, mhj, magi, mhi, stream=0) -> tuple:
    """Times the split-precision kernel variants on these device arrays and
    keeps each kernel's fastest; returns (warps of the 2-/4-body density
    kernel, warps of the 3-body kernel, CTAs per SM of the force kernel)."""
    rw, bw, fb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(load().ace_autotune_device(natom, nei, off, r, e, magj, mhj, magi, mhi, stream, ctypes.byref(rw),
                                      ctypes.byref(bw), ctypes.byref(fb)))
    return rw.value, bw.value, fb.value


TUNING_NAMES = {
    "abasis": ["scalar", "packed FP32x2", "scalar, TMA-staged bond tiles",
               "scalar, TMA-staged bond tiles, persistent grid",
               "tensor cores (3xTF32), TMA-staged bond tiles, persistent grid", "tensor cores (3xTF32)"],
    "density": ["32 warps", "16 warps", "32 warps, record streams", "16 warps, record streams",
                "32 warps, record streams via shared memory", "16 warps, record streams via shared memory"],
    "b3": ["16 warps", "12 warps", "8 warps", "12 warps, n0' outermost", "16 warps, packed FP32x2",
           "12 warps, packed FP32x2"],
    "forces": ["4 CTAs/SM", "6 CTAs/SM", "8 CTAs/SM", "4 CTAs/SM, packed FP32x2", "6 CTAs/SM, packed FP32x2",
               "8 CTAs/SM, packed FP32x2", "5 CTAs/SM, tensor cores (3xTF32)", "6 CTAs/SM, tensor cores (3xTF32)"],
}


def get_tuning() -> dict:
    """The split-precision kernel variants in use, by kernel."""
    v = np.zeros(4, np.int32)
    _check(load().ace_get_tuning(_ip(v)))
    return {k: TUNING_NAMES[k][int(i)] for k, i in zip(("abasis", "density", "b3", "forces"), v)}


def get_tuning_indices() -> list:
    """The variant indices in use: [A basis, density, 3-body, forces]."""
    v = np.zeros(4, np.int32)
    _check(load().ace_get_tuning(_ip(v)))
    return [int(x) for x in v]


def set_tuning(variants) -> None:
    """Selects the variant indices [A basis, density, 3-body, forces]."""
    v = np.ascontiguousarray(np.asarray(variants, dtype=np.int32).reshape(4))
    _check(load().ace_set_tuning(_ip(v)))


def num_coefficients() -> tuple:
    """(coefficients per density, number of densities)."""
    n, nd = ctypes.c_int(), ctypes.c_int()
    _check(load().ace_num_coefficients(ctypes.byref(n), ctypes.byref(nd)))
    return n.value, nd.value


def get_coefficients() -> np.ndarray:
    """The expansion coefficients [ndensity, ncoef] in the file's record order."""
    n, nd = num_coefficients()
    c = np.zeros((nd, n))
    _check(load().ace_get_coefficients(_dp(c)))
    return c


def set_coefficients(c) -> None:
    n, nd = num_coefficients()
    c = np.ascontiguousarray(np.asarray(c, dtype=np.float64).reshape(nd, n))
    _check(load().ace_set_coefficients(_dp(c)))


def descriptors_device(natom, nei, off, r, e, magj, mhj, magi, mhi, B, stream=0) -> None:
    """B[natom, ncoef] (FP64, device address) for the given device arrays."""
    _check(load().ace_descriptors_device(natom, nei, off, r, e, magj, mhj, magi, mhi, B, stream))


def descriptors_tangent_device(natom, nei, off, r, e, magj, mhj, magi, mhi, dd, dmj, dmi, B, Bdot, core, cored,
                               stream=0) -> None:
    """B and dB along the tangents dd (bond vectors), dmj, dmi (moments), and
    the core energy with its derivative; all device addresses, FP64."""
    _check(load().ace_descriptors_tangent_device(natom, nei, off, r, e, magj, mhj, magi, mhi, dd, dmj, dmi, B, Bdot,
                                                 core, cored, stream))


def embedding() -> dict:
    """nfemb, par[order][density] and the inner cutoff (ecut, decut)."""
    n = ctypes.c_int()
    par = np.zeros(4)
    cut = np.zeros(2)
    _check(load().ace_embedding(ctypes.byref(n), _dp(par), _dp(cut)))
    return {"nfemb": n.value, "par": par.reshape(2, 2), "ecut": float(cut[0]), "decut": float(cut[1])}


def density_gradient_device(natom, dedrho, stream=0) -> None:
    """dE_i/drho_d [natom, 2] of the last evaluation into a device array."""
    _check(load().ace_density_gradient_device(natom, dedrho, stream))


def device_status() -> None:
    _check(load().ace_device_status())


def last_launch_count() -> int:
    return int(load().ace_last_launch_count())


def set_kernel_timing(on: bool) -> None:
    _check(load().ace_set_kernel_timing(1 if on else 0))


def kernel_names(n: int) -> list:
    """Names of the timed kernels of an evaluation that launched n kernels
    (the split path's "k_b3" slot includes its k_finish_fe)."""
    return ["k_abasis", "k_density", "k_b3", "k_forces"] if n >= 4 else ["k_abasis", "k_density", "k_forces"]


def kernel_times() -> list:
    """Per-kernel durations (ms) of the last timed evaluation, in launch
    order (kernel_names(last_launch_count()))."""
    out = (ctypes.c_float * 4)()
    _check(load().ace_kernel_times(out))
    return [float(x) for x in out][:len(kernel_names(last_launch_count()))]


def table_stats() -> dict:
    out = (ctypes.c_longlong * 31)()
    _check(load().ace_table_stats(out))
    keys = ["ne1", "ne2", "ne3", "nseg", "nslot", "nF", "nW", "nWA", "nA2h", "nfa", "nfm",
            "nba", "nbm", "n2m", "l2m", "n3a", "n3m", "l3a", "l3m", "h2", "h3",
            "b3_tasks", "b3_combos", "b3_elements", "rest_segments", "rest_entries",
            "rest_ne1", "rest_ne2", "rest_ne3", "b3_pairs", "rest_factors"]
    return {k: int(v) for k, v in zip(keys, out)}


def host_access() -> str:
    """How acelib_ reaches host arrays under the current MAGACE_HOST_ACCESS."""
    return {0: "copy", 1: "pinned", 2: "direct"}.get(int(load().ace_host_access_mode()), "unavailable")
