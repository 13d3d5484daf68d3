"""GB300-native induced-point-dipole polarization (OpenMMPol's polarization path).

``OMMPSystem`` mirrors the polarization subset of pyopenmmpol's ``OMMPSystem``
(pythonapi/pyopenmmpol/pyommp_interface.cpp:482-505 set_external_field,
:258-266 ipd, get_polelec_energy) on top of the C ABI of libommp_gb300.so;
every computation runs on the GPU through that library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

__all__ = ["OMMPSystem", "OMMPQmHelper", "Server", "OMMPError", "available_solvers", "available_matrix_vector",
           "set_verbose", "PREC_FP64", "PREC_MIXED", "PREC_MIXED_DS", "PRECISIONS"]

# pythonapi/pyopenmmpol/pyommp_interface.cpp:9-23
available_solvers = {"none": 0, "default": 1, "conjugate gradient": 1, "cg": 1,
                     "inversion": 3, "diis": 2}
available_matrix_vector = {"none": 0, "default": 2, "incore": 1, "direct": 2}
verbosity = {"none": 0, "low": 1, "high": 2, "debug": 3}
PREC_FP64, PREC_MIXED, PREC_MIXED_DS = 0, 1, 2
# 'mixed-ds': the refinement residual products in double-single arithmetic
PRECISIONS = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "mixed-ds": PREC_MIXED_DS}
ERR_CANCELLED = 7


class OMMPError(RuntimeError):
    """A library call returned a non-zero status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"[status {status}] {msg}")
        self.status = status


def _check(st: int):
    if st != 0:
        raise OMMPError(st, _lib.load().ommp_gpu_last_error().decode())


def set_verbose(level) -> None:
    lvl = verbosity[level] if isinstance(level, str) else int(level)
    _lib.load().ommp_set_verbose(lvl)


def set_fmm_auto(on: bool) -> None:
    """Process-wide: systems created while on get the FMM when they have more
    than 1,000 MM atoms (the reference's default); off (the default), the
    direct sums stay until set_fmm / ommp_enable_fmm."""
    _lib.load().ommp_gpu_set_fmm_auto(int(bool(on)))


def solve_multi(systems, fields):
    """Solve several systems (mixed or mixed-ds precision), each for its own
    external field [pol_atoms][3], together: their pair products share
    multi-system launches (ommp_gpu_solve_multi).  Returns the energies and a
    dict of engine statistics; the dipoles are on each system as after
    set_external_field."""
    L = _lib.load()
    n = len(systems)
    fs = [np.ascontiguousarray(f, dtype=np.float64).reshape(s.pol_atoms, 3) for s, f in zip(systems, fields)]
    hs = (C.c_void_p * n)(*[s._h for s in systems])
    fp = (_lib._dp * n)(*[f.ctypes.data_as(_lib._dp) for f in fs])
    en = np.zeros(n)
    st = np.zeros(5, dtype=np.int64)
    _check(L.ommp_gpu_solve_multi(n, hs, fp, en.ctypes.data_as(_lib._dp),
                                  st.ctypes.data_as(C.POINTER(C.c_int64))))
    keys = ("rounds", "launches", "shared_launches", "max_systems_per_launch", "spread_products")
    return en, dict(zip(keys, (int(v) for v in st)))


def kernel_launch_count() -> int:
    """Kernels the library has launched in this process (CUDA graph launches
    count their kernels)."""
    return int(_lib.load().ommp_gpu_kernel_launch_count())


def _as_c(a, shape, dtype=np.float64):
    a = np.ascontiguousarray(a, dtype=dtype)
    if a.shape != shape:
        raise ValueError(f"array should be shaped {list(shape)}, got {list(a.shape)}")
    return a


class OMMPSystem:
    """A polarizable system read from a ``.mmp`` file (revision 2 or 3)."""

    def __init__(self, mmp_path: str):
        L = _lib.load()
        h = C.c_void_p()
        _check(L.ommp_gpu_init_mmp(str(mmp_path).encode(), C.byref(h)))
        self._h = h
        self._L = L

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.ommp_terminate(h)
            self._h = None

    def close(self):
        self.__del__()

    # --- sizes ---------------------------------------------------------------
    @property
    def pol_atoms(self) -> int:
        return self._L.ommp_get_pol_atoms(self._h)

    @property
    def mm_atoms(self) -> int:
        return self._L.ommp_get_mm_atoms(self._h)

    @property
    def n_ipd(self) -> int:
        return self._L.ommp_get_n_ipd(self._h)

    @property
    def ld_cart(self) -> int:
        return self._L.ommp_get_ld_cart(self._h)

    @property
    def is_amoeba(self) -> bool:
        return bool(self._L.ommp_ff_is_amoeba(self._h))

    # --- arrays (copies of library memory) -----------------------------------
    def _view(self, ptr, shape, dtype=np.float64):
        n = int(np.prod(shape))
        if n == 0:
            return np.zeros(shape, dtype=dtype)
        return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(shape).copy()

    @property
    def ipd(self) -> np.ndarray:
        """Induced dipoles [n_ipd, pol_atoms, 3] (set 0 = D, 1 = P for AMOEBA)."""
        return self._view(self._L.ommp_get_ipd(self._h), (self.n_ipd, self.pol_atoms, 3))

    @property
    def cpol(self) -> np.ndarray:
        return self._view(self._L.ommp_get_cpol(self._h), (self.pol_atoms, 3))

    @property
    def cmm(self) -> np.ndarray:
        return self._view(self._L.ommp_get_cmm(self._h), (self.mm_atoms, 3))

    @property
    def q(self) -> np.ndarray:
        return self._view(self._L.ommp_get_q(self._h), (self.mm_atoms, self.ld_cart))

    @property
    def polar_mm(self) -> np.ndarray:
        return self._view(self._L.ommp_get_polar_mm(self._h), (self.pol_atoms,), np.int32)

    # --- polarization path ------------------------------------------------------
    def set_external_field(self, ext_field, nomm: bool = False, solver: str = "none",
                           matv: str = "none") -> None:
        if solver not in available_solvers:
            raise ValueError("Selected solver is not available!")
        if matv not in available_matrix_vector:
            raise ValueError("Selected matrix-vector method is not available!")
        ef = _as_c(ext_field, (self.pol_atoms, 3))
        _check(self._L.ommp_gpu_set_external_field(
            self._h, ef.ctypes.data_as(_lib._dp), available_solvers[solver],
            available_matrix_vector[matv], 0 if nomm else 1))

    def set_external_fields_batch(self, fields):
        """Solve several external fields together (cold start each); returns
        (ipd [nfields, n_ipd, pol_atoms, 3], energies [nfields])."""
        f = np.ascontiguousarray(fields, dtype=np.float64)
        if f.ndim != 3 or f.shape[1:] != (self.pol_atoms, 3):
            raise ValueError("fields should be shaped [nfields, pol_atoms, 3]")
        nf = f.shape[0]
        out = np.zeros((nf, self.n_ipd, self.pol_atoms, 3))
        e = np.zeros(nf)
        _check(self._L.ommp_gpu_set_external_fields_batch(self._h, nf, f.ctypes.data_as(_lib._dp),
                                                          out.ctypes.data_as(_lib._dp),
                                                          e.ctypes.data_as(_lib._dp)))
        return out, e

    def set_use_graphs(self, on: bool = True) -> None:
        self._L.ommp_gpu_set_use_graphs(self._h, int(on))

    def set_block_cg(self, on: bool = True) -> None:
        """Batches of at least 4 columns in the mixed modes: block CG for the
        FP32 inner solve (default) or the scalar PCG per column."""
        self._L.ommp_gpu_set_block_cg(self._h, int(on))

    def set_residual_update(self, mode) -> None:
        """Refinement residuals of the mixed modes after the first recomputed
        one: 'recompute' (the mode's residual product every step), 'update'
        (r -= T d by the FP32 product of the correction when its error bound
        is below a tenth of the tolerance) or 'auto' (update in mixed-ds,
        recompute in the strict mixed mode; the default)."""
        m = {"auto": -1, "recompute": 0, "update": 1}.get(mode, mode)
        _check(self._L.ommp_gpu_set_residual_update(self._h, int(m)))

    def get_polelec_energy(self) -> float:
        e = C.c_double(0.0)
        _check(self._L.ommp_gpu_get_polelec_energy(self._h, C.byref(e)))
        return e.value

    def get_fixedelec_energy(self) -> float:
        """Interaction energy of the static multipoles (EM)."""
        e = C.c_double(0.0)
        _check(self._L.ommp_gpu_get_fixedelec_energy(self._h, C.byref(e)))
        return e.value

    def get_full_ele_energy(self) -> float:
        """Static multipole plus polarization energy (the reference's
        ommp_get_full_ele_energy, src/mod_interface.F90:388-398)."""
        return self.get_fixedelec_energy() + self.get_polelec_energy()

    def _numerical_grad(self, energy) -> np.ndarray:
        """Central differences of energy() with a 1e-5 bohr step, as the
        reference's numerical_grad (pythonapi/pyopenmmpol/pyommp_interface.cpp:518-543)."""
        g = np.zeros((self.mm_atoms, 3))
        c0 = np.array(self.cmm, copy=True)
        c = c0.copy()
        dd = 1e-5
        for k in range(c.size):
            c.flat[k] = c0.flat[k] + dd
            self.update_coordinates(c)
            ep = energy()
            c.flat[k] = c0.flat[k] - dd
            self.update_coordinates(c)
            g.flat[k] = (ep - energy()) / (2 * dd)
            c.flat[k] = c0.flat[k]
        self.update_coordinates(c0)
        return g

    def polelec_geomgrad(self, numerical: bool = False) -> np.ndarray:
        """Geometric gradient of the polarization energy, [mm_atoms, 3].

        Mirrors the reference's OMMPSystem.polelec_geomgrad
        (pythonapi/pyopenmmpol/pyommp_interface.cpp:592-606): analytic on the
        GPU, or with numerical=True central differences of
        get_polelec_energy."""
        if numerical:
            return self._numerical_grad(self.get_polelec_energy)
        g = np.zeros((self.mm_atoms, 3))
        _check(self._L.ommp_gpu_polelec_geomgrad(self._h, g.ctypes.data_as(_lib._dp)))
        return g

    def fixedelec_geomgrad(self, numerical: bool = False) -> np.ndarray:
        """Geometric gradient of the static multipole energy, [mm_atoms, 3]
        (pythonapi/pyopenmmpol/pyommp_interface.cpp:574-590): analytic on the
        GPU, or with numerical=True central differences of
        get_fixedelec_energy."""
        if numerical:
            return self._numerical_grad(self.get_fixedelec_energy)
        g = np.zeros((self.mm_atoms, 3))
        _check(self._L.ommp_gpu_fixedelec_geomgrad(self._h, g.ctypes.data_as(_lib._dp)))
        return g

    def rotation_geomgrad(self, E, Egrd) -> np.ndarray:
        """Forces [mm_atoms, 3] from the rotation of the static multipoles
        in the field E [mm_atoms, 3] and field gradient Egrd [mm_atoms, 6]
        (xx, xy, yy, xz, yz, zz); mirrors the reference's
        OMMPSystem.rotation_geomgrad (pythonapi/pyopenmmpol/pyommp_interface.cpp:559-566)."""
        E = _as_c(E, (self.mm_atoms, 3))
        Egrd = _as_c(Egrd, (self.mm_atoms, 6))
        g = np.zeros((self.mm_atoms, 3))
        _check(
            self._L.ommp_gpu_rotation_geomgrad(
                self._h, E.ctypes.data_as(_lib._dp), Egrd.ctypes.data_as(_lib._dp), g.ctypes.data_as(_lib._dp)
            )
        )
        return g

    def update_coordinates(self, c) -> None:
        c = _as_c(c, (self.mm_atoms, 3))
        _check(self._L.ommp_gpu_update_coordinates(self._h, c.ctypes.data_as(_lib._dp)))

    def set_default_solver(self, solver: str) -> None:
        _check(self._L.ommp_gpu_set_default_solver(self._h, available_solvers[solver]))

    def set_default_matv(self, matv: str) -> None:
        _check(self._L.ommp_gpu_set_default_matv(self._h, available_matrix_vector[matv]))

    def use_fmm(self) -> bool:
        return bool(self._L.ommp_use_fmm(self._h))

    def set_fmm(self, on: bool = True, order: int = 10) -> None:
        """Fast multipole method for the FP64 T.mu products and the permanent
        field (expansion order 2..12, default 10)."""
        _check(self._L.ommp_gpu_set_fmm(self._h, int(bool(on)), int(order)))

    # the reference's FMM settings (pyopenmmpol names)
    def set_fmm_lmax_pol(self, lmax: int) -> None:
        _check(self._L.ommp_gpu_set_fmm_lmax_pol(self._h, int(lmax)))

    def set_fmm_lmax(self, lmax: int) -> None:
        _check(self._L.ommp_gpu_set_fmm_lmax(self._h, int(lmax)))

    def set_fmm_distance(self, d: float) -> None:
        """near-field distance, bohr"""
        _check(self._L.ommp_gpu_set_fmm_distance(self._h, float(d)))

    def set_fmm_min_cell_size(self, d: float) -> None:
        """minimum cell size (half diagonal), bohr"""
        _check(self._L.ommp_gpu_set_fmm_min_cell_size(self._h, float(d)))

    def fmm_settings(self):
        """(lmax_pol, lmax, leaf-side lower bound in bohr)"""
        a, b, c = C.c_int32(), C.c_int32(), C.c_double()
        self._L.ommp_gpu_get_fmm_settings(self._h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    # --- potential and field at external points (pyopenmmpol names) -------------
    def _ext(self, field: bool, which: int, cext) -> np.ndarray:
        c = np.ascontiguousarray(cext, dtype=np.float64)
        if c.ndim != 2 or c.shape[1] != 3:
            raise ValueError("cext should be shaped [:, 3]")
        out = np.zeros((len(c), 3) if field else len(c))
        fn = self._L.ommp_gpu_field_ext if field else self._L.ommp_gpu_potential_ext
        _check(fn(self._h, which, len(c), c.ctypes.data_as(_lib._dp), out.ctypes.data_as(_lib._dp)))
        return out

    def potential_mmpol2ext(self, cext) -> np.ndarray:
        return self._ext(False, 0, cext)

    def potential_mm2ext(self, cext) -> np.ndarray:
        return self._ext(False, 1, cext)

    def potential_pol2ext(self, cext) -> np.ndarray:
        return self._ext(False, 2, cext)

    def field_mmpol2ext(self, cext) -> np.ndarray:
        return self._ext(True, 0, cext)

    def field_mm2ext(self, cext) -> np.ndarray:
        return self._ext(True, 1, cext)

    def field_pol2ext(self, cext) -> np.ndarray:
        return self._ext(True, 2, cext)

    # --- extensions ---------------------------------------------------------------
    def set_solver_tol(self, tol: float) -> None:
        self._L.ommp_gpu_set_solver_tol(self._h, float(tol))

    def set_solver_maxiter(self, n: int) -> None:
        self._L.ommp_gpu_set_solver_maxiter(self._h, int(n))

    def set_precision(self, mode) -> None:
        m = PRECISIONS.get(mode, mode)
        self._L.ommp_gpu_set_precision(self._h, int(m))

    def set_fp64_kernel(self, mode) -> None:
        """'auto' | 'ordered' (all ordered pairs) | 'symmetric' (unordered pairs)."""
        m = {"auto": 0, "ordered": 1, "symmetric": 2}.get(mode, mode)
        _check(self._L.ommp_gpu_set_fp64_kernel(self._h, int(m)))

    def set_inner_preconditioner(self, mode) -> None:
        """'diagonal' (the reference's alpha) | 'block' (block Jacobi) |
        'near' (block Jacobi with a Neumann step over the near-field
        couplings between the blocks; the default) for the FP32 inner solver
        of the mixed modes."""
        m = {"diagonal": 0, "block": 1, "near": 2}.get(mode, mode)
        _check(self._L.ommp_gpu_set_inner_preconditioner(self._h, int(m)))

    def set_inner_blocks(self, max_sites: int, link_bohr: float) -> None:
        """Runs of the block-Jacobi inner preconditioner: at most max_sites
        consecutive polarizable sites, each within link_bohr of an earlier one."""
        _check(self._L.ommp_gpu_set_inner_blocks(self._h, int(max_sites), float(link_bohr)))

    def set_fp32_kernel(self, mode) -> None:
        """'auto' (autotuned) | 'pairwise' (kernel 1) | 'tiled' (kernel 2) |
        'symmetric' (kernel 3: each unordered pair once)."""
        m = {"auto": 0, "pairwise": 1, "tiled": 2, "symmetric": 3}.get(mode, mode)
        _check(self._L.ommp_gpu_set_fp32_kernel(self._h, int(m)))

    def fp32_shape(self, ncol: int = 1):
        """The autotuned FP32 launch shape for ncol columns: (kernel, columns
        per launch, source splits) with kernel 'pairwise' | 'tiled' |
        'symmetric', or None before the first mixed solve with ncol columns."""
        out = (C.c_int32 * 3)()
        _check(self._L.ommp_gpu_get_fp32_shape(self._h, int(ncol), out))
        if out[0] == 0:
            return None
        return ({1: "pairwise", 2: "tiled", 3: "symmetric"}[out[0]], int(out[1]), int(out[2]))

    def clear_guess(self) -> None:
        self._L.ommp_gpu_clear_guess(self._h)

    def iterations(self, s: int = 0) -> int:
        return self._L.ommp_gpu_get_iterations(self._h, s)

    def residual_history(self, s: int = 0) -> np.ndarray:
        out = np.zeros(4096)
        n = self._L.ommp_gpu_get_residual_history(self._h, s, out.ctypes.data_as(_lib._dp), 4096)
        return out[: min(n, 4096)].copy()

    def counter(self, which: int) -> int:
        return int(self._L.ommp_gpu_get_counter(self._h, which))

    def last_solve_ms(self) -> float:
        return float(self._L.ommp_gpu_last_solve_ms(self._h))

    def e_m2d(self) -> np.ndarray:
        out = np.zeros((self.n_ipd, self.pol_atoms, 3))
        _check(self._L.ommp_gpu_get_e_m2d(self._h, out.ctypes.data_as(_lib._dp)))
        return out

    def tmatvec(self, x, dodiag: bool = True, matv: str = "direct") -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        nrhs = 1 if x.ndim == 2 else x.shape[0]
        x = x.reshape(nrhs, self.pol_atoms, 3)
        y = np.zeros_like(x)
        _check(self._L.ommp_gpu_tmatvec(self._h, x.ctypes.data_as(_lib._dp), y.ctypes.data_as(_lib._dp),
                                        nrhs, int(dodiag), available_matrix_vector[matv]))
        return y[0] if nrhs == 1 else y

    def tmatvec_fp32(self, x) -> np.ndarray:
        return self._tmatvec_alt(self._L.ommp_gpu_tmatvec_fp32, x)

    def tmatvec_ds(self, x) -> np.ndarray:
        """y = T x with the double-single kernel of the 'mixed-ds' mode."""
        return self._tmatvec_alt(self._L.ommp_gpu_tmatvec_ds, x)

    def _tmatvec_alt(self, fn, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        nrhs = 1 if x.ndim == 2 else x.shape[0]
        x = x.reshape(nrhs, self.pol_atoms, 3)
        y = np.zeros_like(x)
        _check(fn(self._h, x.ctypes.data_as(_lib._dp), y.ctypes.data_as(_lib._dp), nrhs))
        return y[0] if nrhs == 1 else y

    def enable_kernel_timing(self, on: bool = True) -> None:
        self._L.ommp_gpu_enable_kernel_timing(self._h, int(on))

    def kernel_stats(self, which: int):
        """(launches, total ms, right-hand-side columns) of the timed pair
        kernel: which 0 = FP64 T.mu, 1 = FP32 T.mu, 2 = double-single T.mu."""
        n = C.c_int64(0)
        ms = C.c_double(0.0)
        cols = C.c_int64(0)
        self._L.ommp_gpu_kernel_stats(self._h, which, C.byref(n), C.byref(ms), C.byref(cols))
        return n.value, ms.value, cols.value

    def synchronize(self) -> None:
        _check(self._L.ommp_gpu_synchronize(self._h))


class OMMPQmHelper:
    """QM nuclei and their electrostatics with one system, as pyopenmmpol's
    OMMPQmHelper (pythonapi/pyopenmmpol/pyommp_interface.cpp:946-1285):
    ``OMMPQmHelper(cqm [n, 3], qqm [n], zqm [n])``, ``prepare_qm_ele_ene(s)``,
    ``prepare_qm_ele_grd(s)``, ``update_coord(cqm)`` and the read-only arrays
    ``E_n2p``, ``G_n2p``, ``E_n2m``, ``G_n2m``, ``H_n2m``, ``V_m2n``,
    ``V_p2n``, ``E_m2n``, ``E_p2n`` (AttributeError before they are
    computed, like the reference's)."""

    _SHAPES = {"E_n2p": ("npol", 3), "G_n2p": ("npol", 6), "E_n2m": ("nmm", 3), "G_n2m": ("nmm", 6),
               "H_n2m": ("nmm", 10), "V_m2n": ("qm", None), "V_p2n": ("qm", None), "E_m2n": ("qm", 3),
               "E_p2n": ("qm", 3)}
    _WHEN = {"E_n2p": "prepare_qm_ele_ene", "V_m2n": "prepare_qm_ele_ene", "V_p2n": "prepare_qm_ele_ene"}

    def __init__(self, cqm, qqm, zqm):
        self._L = _lib.load()
        cqm = np.ascontiguousarray(cqm, dtype=np.float64).reshape(-1, 3)
        n = cqm.shape[0]
        qqm = _as_c(qqm, (n,))
        zqm = _as_c(zqm, (n,), np.int32)
        h = C.c_void_p()
        _check(self._L.ommp_gpu_init_qm_helper(n, cqm.ctypes.data_as(_lib._dp), qqm.ctypes.data_as(_lib._dp),
                                               zqm.ctypes.data_as(_lib._ip), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.ommp_terminate_qm_helper(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def qm_atoms(self) -> int:
        return self._L.ommp_qm_helper_get_qm_atoms(self._h)

    @property
    def npol(self) -> int:
        return self._L.ommp_qm_helper_get_npol(self._h)

    @property
    def nmm(self) -> int:
        return self._L.ommp_qm_helper_get_nmm(self._h)

    @property
    def cqm(self) -> np.ndarray:
        p = self._L.ommp_qm_helper_get_cqm(self._h)
        return np.ctypeslib.as_array(p, shape=(self.qm_atoms, 3)).copy()

    def update_coord(self, cqm) -> None:
        c = _as_c(cqm, (self.qm_atoms, 3))
        self._L.ommp_qm_helper_update_coord(self._h, c.ctypes.data_as(_lib._dp))

    def prepare_qm_ele_ene(self, system: "OMMPSystem") -> None:
        _check(self._L.ommp_gpu_prepare_qm_ele_ene(system._h, self._h))

    def prepare_qm_ele_grd(self, system: "OMMPSystem") -> None:
        _check(self._L.ommp_gpu_prepare_qm_ele_grd(system._h, self._h))

    def __getattr__(self, name):
        shape = OMMPQmHelper._SHAPES.get(name)
        if shape is None:
            raise AttributeError(name)
        p = getattr(self._L, "ommp_qm_helper_get_" + name)(self._h)
        if not p:
            when = OMMPQmHelper._WHEN.get(name, "prepare_qm_ele_grd")
            raise AttributeError(f"{name} is not available. OMMPQmHelper.{when}() should be called before!")
        rows = {"npol": self.npol, "nmm": self.nmm, "qm": self.qm_atoms}[shape[0]]
        full = (rows,) if shape[1] is None else (rows, shape[1])
        return np.ctypeslib.as_array(p, shape=full).copy()


class Server:
    """Request server over ommp_gpu_server_* (continuous admission of solves).

    ``submit(path, field)`` starts a new system; ``submit_followup(instance,
    field)`` reuses a resident one with a warm start; ``wait(rid)`` returns a
    dict with ``ipd``, ``energy``, ``instance`` and ``latency_ms``.
    """

    def __init__(self, hbm_budget_bytes: int, slots: int = 4, precision="mixed", tol: float = 1e-10):
        self._L = _lib.load()
        p = PRECISIONS.get(precision, precision)
        h = C.c_void_p()
        _check(self._L.ommp_gpu_server_create(int(hbm_budget_bytes), int(slots), int(p), float(tol), C.byref(h)))
        self._h = h
        self._meta = {}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.ommp_gpu_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def submit(self, mmp_path: str, field, n_ipd: int) -> int:
        f = np.ascontiguousarray(field, dtype=np.float64)
        rid = C.c_int64(0)
        _check(self._L.ommp_gpu_server_submit(self._h, str(mmp_path).encode(), f.ctypes.data_as(_lib._dp),
                                              f.shape[0], C.byref(rid)))
        self._meta[rid.value] = (f.shape[0], n_ipd)
        return rid.value

    def submit_followup(self, instance: int, field, n_ipd: int) -> int:
        f = np.ascontiguousarray(field, dtype=np.float64)
        rid = C.c_int64(0)
        _check(self._L.ommp_gpu_server_submit_followup(self._h, int(instance), f.ctypes.data_as(_lib._dp),
                                                       f.shape[0], C.byref(rid)))
        self._meta[rid.value] = (f.shape[0], n_ipd)
        return rid.value

    def wait(self, rid: int) -> dict:
        npol, nipd = self._meta.pop(rid)
        out = np.zeros((nipd, npol, 3))
        e = C.c_double(0)
        inst = C.c_int64(-1)
        lat = C.c_double(0)
        _check(self._L.ommp_gpu_server_wait(self._h, int(rid), out.ctypes.data_as(_lib._dp), C.byref(e),
                                            C.byref(inst), C.byref(lat)))
        return {"ipd": out, "energy": e.value, "instance": inst.value, "latency_ms": lat.value}

    def release(self, instance: int) -> None:
        self._L.ommp_gpu_server_release(self._h, int(instance))

    def cancel(self, rid: int) -> bool:
        """True when the request was still queued and is now cancelled."""
        return self._L.ommp_gpu_server_cancel(self._h, int(rid)) == 0

    def set_round_ms(self, ms: float) -> None:
        """Work per product kind in one round of the mixed modes' engine (ms)."""
        _check(self._L.ommp_gpu_server_set_round_ms(self._h, float(ms)))

    def engine_stats(self) -> dict:
        """The multi-system engine of the mixed modes (zeros in FP64)."""
        o = np.zeros(5, dtype=np.int64)
        self._L.ommp_gpu_server_engine_stats(self._h, o.ctypes.data_as(C.POINTER(C.c_int64)))
        keys = ("rounds", "launches", "shared_launches", "max_systems_per_launch", "spread_products")
        out = dict(zip(keys, (int(v) for v in o)))
        t = np.zeros(3)
        self._L.ommp_gpu_server_engine_times(self._h, t.ctypes.data_as(_lib._dp))
        out.update({"product_gpu_ms": float(t[0]), "bookkeeping_gpu_ms": float(t[1]), "round_wall_ms": float(t[2])})
        return out

    def phase_stats(self) -> dict:
        """Mean milliseconds per phase of the new systems that completed:
        waiting for a worker, host setup, waiting for device memory, upload,
        permanent field (mixed modes), solve; and their count."""
        o = np.zeros(7)
        self._L.ommp_gpu_server_phase_stats(self._h, o.ctypes.data_as(_lib._dp))
        n = int(o[0])
        keys = ("queue_ms", "host_setup_ms", "admission_ms", "upload_ms", "field_ms", "solve_ms")
        out = {k: (float(v) / n if n else 0.0) for k, v in zip(keys, o[1:])}
        out["new_systems"] = n
        return out

    def stats(self) -> dict:
        o = np.zeros(7)
        self._L.ommp_gpu_server_stats(self._h, o.ctypes.data_as(_lib._dp))
        keys = ["bytes_in_use", "peak_bytes", "resident", "evictions", "peak_concurrent", "completed", "budget"]
        return dict(zip(keys, o.tolist()))
