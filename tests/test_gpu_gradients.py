"""Polarization-energy gradient on the GPU (ommp_polelec_geomgrad) against
the oracle's restatement of polelec_geomgrad (src/mod_geomgrad.F90:113-277).

The oracle evaluates the gradient on the GPU's own dipoles (installed with
set_ipd), so the comparison isolates the gradient arithmetic: FP64 pair sums
in a different order (fp64 mode) or double-single pair sums (mixed modes),
tolerance 1e-11 relative (max over atoms and
components, normalised by the largest component).  Against an independent
oracle solve (both converged to 1e-12) the tolerance is 1e-9.  The water box
at benchmark size (90,000 sites) is checked on sampled atoms through the
oracle's per-atom restriction, plus translation invariance (forces of the
polarization energy sum to zero without an external field).
"""
import numpy as np
import pytest

from openmmpol_gb300 import OMMPError, OMMPSystem, set_verbose, synth
from oracle.oracle import OracleSystem

pytestmark = pytest.mark.gpu

CASES = ["nma_amoeba", "nma_wang", "nma_amoeba_cut", "nma_wang_cut", "1crn_amoeba", "1crn_wang",
         "1ubq_amoeba", "1ubq_wang", "1ao6cut_wang"]


def maxrel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


def solved(path, tol=1e-12, precision="fp64"):
    g = OMMPSystem(path)
    g.set_precision(precision)
    g.set_solver_tol(tol)
    g.set_external_field(np.zeros((g.pol_atoms, 3)))
    return g


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES)
def test_gradient_matches_oracle_on_same_dipoles(case, precision, golden_mmp):
    # fp64: the FP64 pair pass; mixed modes: the double-single pair passes
    g = solved(golden_mmp[case], precision=precision)
    gg = g.polelec_geomgrad()
    o = OracleSystem(golden_mmp[case])
    o.set_ipd(g.ipd)
    assert maxrel(gg, o.polelec_geomgrad()) < 1e-11


@pytest.mark.parametrize("case", ["nma_amoeba", "1crn_amoeba", "1crn_wang"])
def test_gradient_matches_independent_oracle_solve(case, golden_mmp):
    g = solved(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    o.set_tol(1e-12)
    o.set_external_field(np.zeros((o.pol_atoms, 3)))
    assert maxrel(g.polelec_geomgrad(), o.polelec_geomgrad()) < 1e-9


def test_gradient_solves_first_when_no_dipoles(golden_mmp):
    # like the reference, the gradient solves with the permanent field alone
    # (default solver) when the system holds no dipoles
    p = golden_mmp["1crn_amoeba"]
    g = OMMPSystem(p)
    g.set_solver_tol(1e-12)
    first = g.polelec_geomgrad()
    ref = solved(p).polelec_geomgrad()
    assert maxrel(first, ref) < 1e-9


def test_gradient_is_deterministic(golden_mmp):
    g = solved(golden_mmp["1ubq_amoeba"])
    a, b = g.polelec_geomgrad(), g.polelec_geomgrad()
    assert np.array_equal(a, b)


def test_gradient_matches_finite_differences(golden_mmp):
    # the reference's numerical option: central differences of the energy,
    # dipoles solved exactly (inversion) at every displaced geometry
    g = OMMPSystem(golden_mmp["nma_amoeba"])
    g.set_default_solver("inversion")
    ana = g.polelec_geomgrad()
    num = g.polelec_geomgrad(numerical=True)
    assert maxrel(num, ana) < 1e-8


@pytest.mark.parametrize("precision", ["mixed", "mixed-ds"])
def test_gradient_after_mixed_precision_solve(precision, golden_mmp):
    # the gradient is FP64 whatever the mode; the mixed solvers deliver
    # dipoles at the FP64 residual tolerance
    p = golden_mmp["1ubq_amoeba"]
    ref = solved(p).polelec_geomgrad()
    g = solved(p, tol=1e-10, precision=precision)
    assert maxrel(g.polelec_geomgrad(), ref) < 1e-7


def test_gradient_after_coordinate_update(golden_mmp):
    p = golden_mmp["1crn_amoeba"]
    g = solved(p)
    g.polelec_geomgrad()
    c = g.cmm.copy()
    c += np.random.default_rng(5).normal(scale=0.02, size=c.shape)
    g.update_coordinates(c)
    g.set_external_field(np.zeros((g.pol_atoms, 3)))
    gg = g.polelec_geomgrad()
    o = OracleSystem(p)
    o.update_coordinates(c)
    o.set_ipd(g.ipd)
    assert maxrel(gg, o.polelec_geomgrad()) < 1e-11


def test_coincident_sites_are_reported(golden_mmp):
    p = golden_mmp["nma_wang"]
    g = solved(p)
    c = g.cmm.copy()
    c[1] = c[0]
    g.update_coordinates(c)
    with pytest.raises(OMMPError):
        g.polelec_geomgrad()


@pytest.mark.parametrize("precision", ["fp64", "mixed-ds"])
def test_water_box_gradient_sampled(precision, tmp_path):
    # benchmark geometry: 30,000 AMOEBA waters (90,000 sites)
    w = synth.water_cluster(30000, seed=1)
    p = synth.write_mmp(str(tmp_path / "w30k.mmp"), w)
    g = OMMPSystem(p)
    g.set_precision(precision)
    g.set_solver_tol(1e-10)
    g.set_external_field(np.zeros((g.pol_atoms, 3)))
    gg = g.polelec_geomgrad()
    assert np.isfinite(gg).all()
    assert np.abs(gg.sum(0)).max() < 1e-8 * np.abs(gg).max()
    o = OracleSystem(p)
    o.set_ipd(g.ipd)
    atoms = np.sort(np.random.default_rng(7).choice(g.mm_atoms, 48, replace=False)).astype(np.int32)
    ref = o.polelec_geomgrad_atoms(atoms)
    assert np.abs(gg[atoms] - ref).max() / np.abs(ref).max() < 1e-11


@pytest.mark.parametrize("case", ["nma_amoeba", "1crn_amoeba", "1ubq_amoeba", "nma_wang", "1ubq_wang"])
def test_rotation_gradient_matches_oracle(case, golden_mmp):
    # ommp_rotation_geomgrad (src/rotate_multipoles.F90:3-230) in a random
    # field and field gradient: FP64 frame pullback on the GPU against the
    # oracle's rotation-matrix derivatives; zeros for point charges
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    rng = np.random.default_rng(11)
    E = rng.standard_normal((g.mm_atoms, 3)) * 1e-2
    G = rng.standard_normal((g.mm_atoms, 6)) * 1e-2
    gg = g.rotation_geomgrad(E, G)
    go = o.rotation_geomgrad(E, G)
    if case.endswith("wang"):
        assert not gg.any() and not go.any()
        return
    assert maxrel(gg, go) < 1e-12
    # again after a coordinate update (frames follow the new geometry)
    c = g.cmm + rng.standard_normal((g.mm_atoms, 3)) * 1e-2
    g.update_coordinates(c)
    o.update_coordinates(c)
    assert maxrel(g.rotation_geomgrad(E, G), o.rotation_geomgrad(E, G)) < 1e-12


def test_rotation_gradient_rejects_bad_shapes(golden_mmp):
    g = OMMPSystem(golden_mmp["nma_amoeba"])
    with pytest.raises(ValueError):
        g.rotation_geomgrad(np.zeros((g.mm_atoms, 6)), np.zeros((g.mm_atoms, 6)))


def test_rotation_gradient_on_water_box(tmp_path):
    # the water box's bisector frames (6,000 sites)
    p = synth.write_mmp(str(tmp_path / "w.mmp"), synth.water_cluster(2000, seed=4))
    g = OMMPSystem(p)
    o = OracleSystem(p)
    rng = np.random.default_rng(2)
    E = rng.standard_normal((g.mm_atoms, 3))
    G = rng.standard_normal((g.mm_atoms, 6))
    gg = g.rotation_geomgrad(E, G)
    assert maxrel(gg, o.rotation_geomgrad(E, G)) < 1e-12
    assert np.abs(gg.sum(axis=0)).max() < 1e-10 * np.abs(gg).max()
