"""The oracle's polarization-energy gradient (polelec_geomgrad restated,
src/mod_geomgrad.F90:113-277 with rotation_geomgrad) pinned by central finite
differences of the oracle's own energy.

The reference ships no gradient golden file, so the analytic restatement is
checked against the derivative of the energy it already reproduces to the
reference's goldens: dipoles solved exactly (inversion) at each displaced
geometry, permanent field only, h = 1e-5 bohr.  AMOEBA exercises the
field-gradient/Hessian terms and the multipole-rotation (frame) terms; Wang-AL
the charge-only path.
"""
import numpy as np
import pytest

from openmmpol_gb300 import synth
from oracle.oracle import SOLVER_DIIS, SOLVER_INVERSION, OracleSystem


def fd_check(path, atoms=None, h=1e-5, exact=True):
    o = OracleSystem(path)
    if exact:
        o.set_default_solver(SOLVER_INVERSION)
    else:  # converged far below the finite-difference error
        o.set_default_solver(SOLVER_DIIS)
        o.set_tol(1e-13)
    c0 = o.cmm.copy()

    def energy(c):
        o.update_coordinates(c)
        o.set_external_field(np.zeros((o.pol_atoms, 3)))
        return o.get_polelec_energy()

    energy(c0)
    g = o.polelec_geomgrad()
    if atoms is None:
        atoms = range(o.mm_atoms)
    fd = np.zeros((len(atoms), 3))
    for r, a in enumerate(atoms):
        for k in range(3):
            cp, cm = c0.copy(), c0.copy()
            cp[a, k] += h
            cm[a, k] -= h
            fd[r, k] = (energy(cp) - energy(cm)) / (2 * h)
    return np.abs(fd - g[list(atoms)]).max() / np.abs(g).max()


@pytest.mark.parametrize("case,tol", [("nma_amoeba", 1e-8), ("nma_wang", 1e-8), ("1crn_amoeba", 1e-7),
                                      ("1ao6cut_wang", 1e-5)])
def test_gradient_matches_finite_differences(case, tol, golden_mmp):
    # nma: every atom; 1ao6 (18,331 static sites, 37 polarizable): the
    # polarizable sites and a few static ones; 1crn: a sample
    atoms = {"1ao6cut_wang": [13442, 13450, 13460, 13478, 0, 9000, 18330],
             "1crn_amoeba": [0, 101, 250, 377, 640]}.get(case)
    assert fd_check(golden_mmp[case], atoms, exact=not case.startswith("1crn")) < tol


def test_water_gradient_matches_finite_differences(tmp_path):
    w = synth.water_cluster(12, seed=3)
    p = synth.write_mmp(str(tmp_path / "w.mmp"), w)
    assert fd_check(p) < 1e-8


@pytest.mark.parametrize("case,tol", [("nma_amoeba", 1e-12), ("1crn_wang", 1e-12), ("1crn_amoeba", 1e-6)])
def test_gradient_is_translation_invariant(case, tol, golden_mmp):
    # no external field: the forces of the polarization energy sum to zero.
    # 1crn AMOEBA: its two hydroxyl oxygens (atoms 73 and 153) carry a
    # quadrupole trace of 3.3e-6 from the input's rounding; the reference's
    # field formulas drop the trace while its Hessian contraction keeps it,
    # so in damped pairs the analytic forces there differ from the energy's
    # derivative at the 1e-7 level (the sampled atoms of the finite-difference
    # test avoid them)
    o = OracleSystem(golden_mmp[case])
    o.set_default_solver(SOLVER_DIIS)
    o.set_tol(1e-13)
    o.set_external_field(np.zeros((o.pol_atoms, 3)))
    g = o.polelec_geomgrad()
    assert np.abs(g.sum(0)).max() < tol * np.abs(g).max()


@pytest.mark.parametrize("case", ["nma_amoeba", "1crn_amoeba", "1crn_wang"])
def test_gradient_rows_and_installed_dipoles(case, golden_mmp):
    # the per-atom restriction (used on the full-size water box) and dipoles
    # installed from elsewhere reproduce the full gradient exactly
    o = OracleSystem(golden_mmp[case])
    o.set_tol(1e-12)
    o.set_external_field(np.zeros((o.pol_atoms, 3)))
    g = o.polelec_geomgrad()
    atoms = np.array([0, 3, 5, 7, 11]) if case.startswith("nma") else np.array([0, 73, 101, 153, 250, 377, 640])
    assert np.array_equal(o.polelec_geomgrad_atoms(atoms), g[atoms])
    o2 = OracleSystem(golden_mmp[case])
    o2.set_ipd(o.ipd)
    assert np.array_equal(o2.polelec_geomgrad(), g)


def rotation_energy(o, c, E, G):
    """-mu.E + Q:G of the rotated static multipoles at geometry c (E, G held
    fixed; off-diagonal quadrupole components counted twice)."""
    o.update_coordinates(c)
    q = o.q
    w = np.array([1.0, 2.0, 1.0, 2.0, 2.0, 1.0])
    return -np.sum(q[:, 1:4] * E) + np.sum(q[:, 4:10] * G * w)


@pytest.mark.parametrize("case", ["nma_amoeba", "1crn_amoeba"])
def test_rotation_gradient_matches_finite_differences(case, golden_mmp):
    # ommp_rotation_geomgrad (src/rotate_multipoles.F90:3-230) is the
    # derivative of -mu.E + Q:G through the frame rotation alone
    o = OracleSystem(golden_mmp[case])
    rng = np.random.default_rng(5)
    E = rng.standard_normal((o.mm_atoms, 3)) * 1e-2
    G = rng.standard_normal((o.mm_atoms, 6)) * 1e-2
    c0 = o.cmm.copy()
    g = o.rotation_geomgrad(E, G)
    atoms = range(o.mm_atoms) if o.mm_atoms < 40 else [0, 1, 2, 57, 101, 250, 377, 640]
    h = 1e-5
    fd = np.zeros((len(atoms), 3))
    for r, a in enumerate(atoms):
        for k in range(3):
            cp, cm = c0.copy(), c0.copy()
            cp[a, k] += h
            cm[a, k] -= h
            fd[r, k] = (rotation_energy(o, cp, E, G) - rotation_energy(o, cm, E, G)) / (2 * h)
    o.update_coordinates(c0)
    assert np.abs(g).max() > 0
    assert np.abs(fd - g[list(atoms)]).max() / np.abs(g).max() < 1e-8
    # the rotation forces of a rigid frame sum to zero (no net force)
    assert np.abs(g.sum(axis=0)).max() < 1e-12 * np.abs(g).max() * o.mm_atoms


def test_rotation_gradient_of_point_charges_is_zero(golden_mmp):
    o = OracleSystem(golden_mmp["nma_wang"])
    g = o.rotation_geomgrad(np.ones((o.mm_atoms, 3)), np.ones((o.mm_atoms, 6)))
    assert g.shape == (o.mm_atoms, 3) and not g.any()


@pytest.mark.parametrize("case,tol", [("nma_amoeba", 1e-8), ("nma_wang", 1e-8), ("1crn_amoeba", 5e-8)])
def test_static_gradient_matches_finite_differences(case, tol, golden_mmp):
    # fixedelec_geomgrad (src/mod_geomgrad.F90:17-111) against central
    # differences of the static multipole energy, which holds the
    # reference's EM goldens (tests/test_oracle_golden.py); 1crn's larger
    # total energy leaves ~5e-10 of rounding in each difference quotient
    o = OracleSystem(golden_mmp[case])
    g = o.fixedelec_geomgrad()
    c0 = o.cmm.copy()
    atoms = range(o.mm_atoms) if o.mm_atoms < 40 else [0, 1, 57, 250, 377, 640]
    h = 1e-5
    fd = np.zeros((len(atoms), 3))
    for r, a in enumerate(atoms):
        for k in range(3):
            cp, cm = c0.copy(), c0.copy()
            cp[a, k] += h
            cm[a, k] -= h
            o.update_coordinates(cp)
            ep = o.get_fixedelec_energy()
            o.update_coordinates(cm)
            fd[r, k] = (ep - o.get_fixedelec_energy()) / (2 * h)
    o.update_coordinates(c0)
    assert np.abs(fd - g[list(atoms)]).max() / np.abs(g).max() < tol
    # no net force, up to the 1crn input's quadrupole trace (3.3e-6 on two
    # oxygens): the reference's fields drop the trace, its Hessian
    # contraction keeps it, so the pair terms are not exactly antisymmetric
    net = 1e-6 if case.startswith("1crn") else 1e-12 * o.mm_atoms
    assert np.abs(g.sum(axis=0)).max() < net * np.abs(g).max()
