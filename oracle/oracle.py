"""ctypes wrapper around the CPU oracle (oracle/_build/libommp_oracle.so).

TEST INFRASTRUCTURE ONLY: the checker for the GPU library.  Only tests/,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module.  The oracle restates OpenMMPol's polarization path; see
``ommp_oracle.h`` for the reference routines (file:line) it follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libommp_oracle.so")
_lib = None

SOLVER_NONE, SOLVER_CG, SOLVER_DIIS, SOLVER_INVERSION = 0, 1, 2, 3
MATV_NONE, MATV_INCORE, MATV_DIRECT = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    srcs = [os.path.join(_HERE, f) for f in ("ommp_oracle.c", "ommp_oracle.h", "Makefile")]
    stale = not os.path.exists(_LIB_PATH) or any(
        os.path.getmtime(f) > os.path.getmtime(_LIB_PATH) for f in srcs if os.path.exists(f))
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        sig = {
            "orc_last_error": (C.c_char_p, []),
            "orc_init_mmp": (vp, [C.c_char_p]),
            "orc_free": (None, [vp]),
            "orc_mm_atoms": (C.c_int32, [vp]),
            "orc_pol_atoms": (C.c_int32, [vp]),
            "orc_n_ipd": (C.c_int32, [vp]),
            "orc_is_amoeba": (C.c_int32, [vp]),
            "orc_ld_cart": (C.c_int32, [vp]),
            "orc_set_tol": (None, [vp, C.c_double]),
            "orc_set_maxiter": (None, [vp, C.c_int32]),
            "orc_set_default_solver": (None, [vp, C.c_int32]),
            "orc_set_default_matv": (None, [vp, C.c_int32]),
            "orc_set_num_threads": (None, [C.c_int32]),
            "orc_get_cmm": (None, [vp, dp]),
            "orc_get_q": (None, [vp, dp]),
            "orc_get_pol": (None, [vp, dp]),
            "orc_get_polar_mm": (None, [vp, ip]),
            "orc_get_thole": (None, [vp, dp]),
            "orc_get_e_m2d": (C.c_int, [vp, dp]),
            "orc_get_ipd": (None, [vp, dp]),
            "orc_screening_nnz": (C.c_int32, [vp, C.c_int32]),
            "orc_get_screening": (None, [vp, C.c_int32, ip, ip, dp]),
            "orc_tmatvec": (C.c_int, [vp, dp, dp, C.c_int32, C.c_int32]),
            "orc_tmatvec_rows": (C.c_int, [vp, dp, ip, C.c_int32, dp]),
            "orc_potential_ext": (C.c_int, [vp, C.c_int32, C.c_int32, dp, dp]),
            "orc_field_ext": (C.c_int, [vp, C.c_int32, C.c_int32, dp, dp]),
            "orc_polelec_geomgrad": (C.c_int, [vp, dp]),
            "orc_polelec_geomgrad_atoms": (C.c_int, [vp, C.c_int32, ip, dp]),
            "orc_set_ipd": (C.c_int, [vp, dp]),
            "orc_get_fixedelec_energy": (C.c_int, [vp, dp]),
            "orc_rotation_geomgrad": (C.c_int, [vp, dp, dp, dp]),
            "orc_fixedelec_geomgrad": (C.c_int, [vp, dp]),
            "orc_nuclei_fields": (C.c_int, [vp, C.c_int32, C.c_int32, dp, dp, dp, dp, dp]),
            "orc_set_external_field": (C.c_int, [vp, dp, C.c_int32, C.c_int32, C.c_int32]),
            "orc_get_polelec_energy": (C.c_double, [vp, ip]),
            "orc_last_iterations": (C.c_int32, [vp, C.c_int32]),
            "orc_matvec_count": (C.c_int64, [vp]),
            "orc_residual_history": (C.c_int32, [vp, C.c_int32, dp, C.c_int32]),
            "orc_update_coordinates": (C.c_int, [vp, dp]),
            "orc_clear_guess": (None, [vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class OracleError(RuntimeError):
    pass


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


class OracleSystem:
    """Mirror of the reference's OMMPSystem for the polarization path."""

    def __init__(self, mmp_path: str):
        L = lib()
        self._h = L.orc_init_mmp(mmp_path.encode())
        if not self._h:
            raise OracleError(L.orc_last_error().decode())
        self.mm_atoms = L.orc_mm_atoms(self._h)
        self.pol_atoms = L.orc_pol_atoms(self._h)
        self.n_ipd = L.orc_n_ipd(self._h)
        self.is_amoeba = bool(L.orc_is_amoeba(self._h))
        self.ld_cart = L.orc_ld_cart(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_free(h)
            self._h = None

    def _check(self, st):
        if st != 0:
            raise OracleError(f"status {st}: {lib().orc_last_error().decode()}")

    def set_tol(self, tol: float):
        lib().orc_set_tol(self._h, float(tol))

    def set_maxiter(self, n: int):
        lib().orc_set_maxiter(self._h, int(n))

    def set_default_solver(self, s: int):
        lib().orc_set_default_solver(self._h, int(s))

    def set_default_matv(self, m: int):
        lib().orc_set_default_matv(self._h, int(m))

    @property
    def cmm(self):
        o = np.zeros((self.mm_atoms, 3))
        lib().orc_get_cmm(self._h, _dp(o))
        return o

    @property
    def q(self):
        o = np.zeros((self.mm_atoms, self.ld_cart))
        lib().orc_get_q(self._h, _dp(o))
        return o

    @property
    def pol(self):
        o = np.zeros(self.pol_atoms)
        lib().orc_get_pol(self._h, _dp(o))
        return o

    @property
    def polar_mm(self):
        o = np.zeros(self.pol_atoms, dtype=np.int32)
        lib().orc_get_polar_mm(self._h, _ip(o))
        return o

    @property
    def thole(self):
        o = np.zeros(self.mm_atoms)
        lib().orc_get_thole(self._h, _dp(o))
        return o

    @property
    def ipd(self):
        o = np.zeros((self.n_ipd, self.pol_atoms, 3))
        lib().orc_get_ipd(self._h, _dp(o))
        return o

    def e_m2d(self):
        o = np.zeros((self.n_ipd, self.pol_atoms, 3))
        self._check(lib().orc_get_e_m2d(self._h, _dp(o)))
        return o

    def screening(self, which: int):
        """which: 0 = S-P (P field), 1 = S-P (D field), 2 = P-P."""
        L = lib()
        nnz = L.orc_screening_nnz(self._h, which)
        nrow = self.pol_atoms if which == 2 else self.mm_atoms
        ri = np.zeros(nrow + 1, dtype=np.int32)
        ci = np.zeros(max(nnz, 1), dtype=np.int32)
        sc = np.zeros(max(nnz, 1))
        if which == 1 and not self.is_amoeba:
            return ri, ci[:0], sc[:0]
        L.orc_get_screening(self._h, which, _ip(ri), _ip(ci), _dp(sc))
        return ri, ci[:nnz], sc[:nnz]

    def tmatvec(self, x, dodiag=True, matv=MATV_DIRECT):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.pol_atoms, 3)
        y = np.zeros_like(x)
        self._check(lib().orc_tmatvec(self._h, _dp(x), _dp(y), int(dodiag), int(matv)))
        return y

    def tmatvec_rows(self, x, rows):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.pol_atoms, 3)
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        y = np.zeros((len(rows), 3))
        self._check(lib().orc_tmatvec_rows(self._h, _dp(x), _ip(rows), len(rows), _dp(y)))
        return y

    def potential_ext(self, which, cext, v=None):
        """Potential at points cext [n][3] added into v (zeros if None);
        which: 0 static + induced, 1 static, 2 induced."""
        cext = np.ascontiguousarray(cext, dtype=np.float64).reshape(-1, 3)
        v = np.zeros(len(cext)) if v is None else np.array(v, dtype=np.float64)
        self._check(lib().orc_potential_ext(self._h, int(which), len(cext), _dp(cext), _dp(v)))
        return v

    def polelec_geomgrad(self):
        """Gradient of the polarization energy w.r.t. the static-site
        coordinates, [mm][3] (a.u.)."""
        g = np.zeros((self.mm_atoms, 3))
        self._check(lib().orc_polelec_geomgrad(self._h, _dp(g)))
        return g

    def polelec_geomgrad_atoms(self, atoms):
        """The gradient on the listed atoms only, [len(atoms)][3]."""
        atoms = np.ascontiguousarray(atoms, dtype=np.int32)
        g = np.zeros((len(atoms), 3))
        self._check(lib().orc_polelec_geomgrad_atoms(self._h, len(atoms), _ip(atoms), _dp(g)))
        return g

    def set_ipd(self, ipd):
        """Install dipoles [n_ipd][npol][3] solved elsewhere as the solved state."""
        ipd = np.ascontiguousarray(ipd, dtype=np.float64).reshape(self.n_ipd, self.pol_atoms, 3)
        self._check(lib().orc_set_ipd(self._h, _dp(ipd)))

    def get_fixedelec_energy(self):
        e = C.c_double(0.0)
        self._check(lib().orc_get_fixedelec_energy(self._h, C.byref(e)))
        return e.value

    def fixedelec_geomgrad(self):
        """Gradient [mm][3] of the static multipole energy."""
        g = np.zeros((self.mm_atoms, 3))
        self._check(lib().orc_fixedelec_geomgrad(self._h, _dp(g)))
        return g

    def rotation_geomgrad(self, E, G):
        """Frame forces [mm][3] of the static multipoles in the field E
        [mm][3] and field gradient G [mm][6] (xx, xy, yy, xz, yz, zz)."""
        E = np.ascontiguousarray(E, dtype=np.float64).reshape(self.mm_atoms, 3)
        G = np.ascontiguousarray(G, dtype=np.float64).reshape(self.mm_atoms, 6)
        g = np.zeros((self.mm_atoms, 3))
        self._check(lib().orc_rotation_geomgrad(self._h, _dp(E), _dp(G), _dp(g)))
        return g

    def nuclei_fields(self, cqm, qqm, grad=False):
        """QM-helper fields of point nuclei at the MM sites: E_n2p [npol][3]
        (grad False) or (E_n2m [mm][3], G_n2m [mm][6], H_n2m [mm][10])."""
        cqm = np.ascontiguousarray(cqm, dtype=np.float64).reshape(-1, 3)
        qqm = np.ascontiguousarray(qqm, dtype=np.float64)
        nt = self.mm_atoms if grad else self.pol_atoms
        E, G, H = np.zeros((nt, 3)), np.zeros((nt, 6)), np.zeros((nt, 10))
        self._check(lib().orc_nuclei_fields(self._h, int(grad), len(cqm), _dp(cqm), _dp(qqm), _dp(E), _dp(G),
                                            _dp(H)))
        return (E, G, H) if grad else E

    def field_ext(self, which, cext, e=None):
        cext = np.ascontiguousarray(cext, dtype=np.float64).reshape(-1, 3)
        e = np.zeros((len(cext), 3)) if e is None else np.array(e, dtype=np.float64).reshape(-1, 3)
        self._check(lib().orc_field_ext(self._h, int(which), len(cext), _dp(cext), _dp(e)))
        return e

    def set_external_field(self, ef, nomm=False, solver=SOLVER_NONE, matv=MATV_NONE):
        ef = np.ascontiguousarray(ef, dtype=np.float64).reshape(self.pol_atoms, 3)
        self._check(lib().orc_set_external_field(self._h, _dp(ef), int(solver), int(matv),
                                                 0 if nomm else 1))

    def get_polelec_energy(self):
        st = C.c_int32(0)
        e = lib().orc_get_polelec_energy(self._h, C.byref(st))
        self._check(st.value)
        return e

    def last_iterations(self, s=0):
        return lib().orc_last_iterations(self._h, s)

    def matvec_count(self):
        return int(lib().orc_matvec_count(self._h))

    def residual_history(self, s=0):
        o = np.zeros(1024)
        n = lib().orc_residual_history(self._h, s, _dp(o), 1024)
        return o[: min(n, 1024)]

    def update_coordinates(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(self.mm_atoms, 3)
        self._check(lib().orc_update_coordinates(self._h, _dp(c)))

    def clear_guess(self):
        lib().orc_clear_guess(self._h)
