"""Fast multipole method for the FP64 T.mu products (ommp_enable_fmm;
csrc/fmm.cu) against the direct sums.

The expansions are Cartesian Taylor series truncated at total order p
(|g| + |h| <= p in the M2L) with the one-neighbour separation of a uniform
octree.  On water the far field carries ~7e-4 relative error at order 8,
~2.5e-4 at 10 (the default) and ~9e-5 at 12.  Order 10 holds the reference's
own FMM-produced 1ubq goldens (its order-8 spherical expansions) at their
tolerance, atol 1e-3; order 8 does not.  Tolerances: the product against the
direct one 3e-3 at order 8, shrinking with the order; solves at the default
order against the direct solve 3e-4 in the dipoles, 1e-5 in the energy.
"""
import numpy as np
import pytest

from openmmpol_gb300 import OMMPSystem, set_verbose, synth

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


@pytest.fixture(scope="module")
def water(tmp_path_factory):
    w = synth.water_cluster(4000, seed=2)
    return synth.write_mmp(str(tmp_path_factory.mktemp("fmm") / "w4k.mmp"), w)


def test_fmm_product_converges_with_order(water):
    g = OMMPSystem(water)
    x = np.random.default_rng(0).standard_normal((2, g.pol_atoms, 3)) * 0.01
    ref = g.tmatvec(x, dodiag=False)
    errs = {}
    for order in (4, 8, 12):
        g.set_fmm(True, order)
        assert g.use_fmm()
        errs[order] = rel(g.tmatvec(x, dodiag=False), ref)
    assert errs[8] < 3e-3
    assert errs[12] < 0.5 * errs[8] < 0.5 * errs[4]
    # the diagonal term is exact
    g.set_fmm(True, 8)
    d = g.tmatvec(x, dodiag=True) - g.tmatvec(x, dodiag=False)
    g.set_fmm(False)
    d0 = g.tmatvec(x, dodiag=True) - g.tmatvec(x, dodiag=False)
    np.testing.assert_allclose(d, d0, rtol=1e-12, atol=1e-16)


def test_fmm_product_is_deterministic(water):
    g = OMMPSystem(water)
    g.set_fmm(True, 8)
    x = np.random.default_rng(1).standard_normal((g.pol_atoms, 3))
    assert np.array_equal(g.tmatvec(x), g.tmatvec(x))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fmm_solve_against_direct(water, precision):
    g = OMMPSystem(water)
    g.set_precision(precision)
    g.set_solver_tol(1e-9)
    ef = synth.point_charge_field(g.cpol, g.cmm.mean(0) / 1.8897261245650, seed=5, all_sites_bohr=g.cmm)[0]
    g.set_external_field(ef)
    ref, e_ref = g.ipd.copy(), g.get_polelec_energy()
    g.set_fmm(True)  # default order 10
    g.clear_guess()
    g.set_external_field(ef)
    assert rel(g.ipd, ref) < 3e-4
    assert abs(g.get_polelec_energy() - e_ref) < 1e-5 * abs(e_ref)


def test_fmm_follows_coordinate_updates(water):
    g = OMMPSystem(water)
    g.set_fmm(True, 8)
    x = np.random.default_rng(2).standard_normal((g.pol_atoms, 3)) * 0.01
    c = g.cmm + np.random.default_rng(3).normal(scale=0.05, size=(g.mm_atoms, 3))
    g.tmatvec(x)
    g.update_coordinates(c)
    y = g.tmatvec(x, dodiag=False)
    g.set_fmm(False)
    assert rel(y, g.tmatvec(x, dodiag=False)) < 3e-3


@pytest.mark.parametrize("case", ["1ubq_amoeba", "1ubq_wang"])
def test_fmm_matches_reference_fmm_goldens(case, golden, golden_mmp):
    g = OMMPSystem(golden_mmp[case])
    g.set_fmm(True)  # default order 10
    for with_field in (0, 1):
        ef = golden[case + "_ef1"] if with_field else np.zeros((g.pol_atoms, 3))
        g.clear_guess()
        g.set_external_field(ef)
        ref = golden[f"{case}_ipd{with_field}"]
        np.testing.assert_allclose(g.ipd.reshape(-1, 3), ref, rtol=1e-6, atol=float(golden[case + "_atol"]))
        np.testing.assert_allclose(g.get_polelec_energy(), float(golden[f"{case}_ep{with_field}"]), rtol=1e-6,
                                   atol=1e-3)


def test_fmm_small_system_uses_direct_sums(golden_mmp):
    g = OMMPSystem(golden_mmp["nma_amoeba"])
    x = np.random.default_rng(4).standard_normal((g.pol_atoms, 3))
    ref = g.tmatvec(x)
    g.set_fmm(True, 8)
    np.testing.assert_array_equal(g.tmatvec(x), ref)


@pytest.mark.parametrize("case", ["1ubq_amoeba", "1ubq_wang"])
def test_fmm_permanent_field_against_direct(case, golden_mmp):
    # E_M2D from the static multipoles through the FMM in the FP64 modes; a
    # field of the direct sums stays valid for every mode, the double-single
    # mode computes its own
    ref = OMMPSystem(golden_mmp[case]).e_m2d()
    errs = {}
    for order in (8, 12):
        g = OMMPSystem(golden_mmp[case])
        g.set_fmm(True, order)
        errs[order] = rel(g.e_m2d(), ref)
    assert errs[8] < 3e-3 and errs[12] < 0.5 * errs[8]
    g.set_precision("mixed-ds")
    assert rel(g.e_m2d(), ref) < 1e-11
    g.set_precision("fp64")
    g.set_fmm(False)
    assert rel(g.e_m2d(), ref) < 1e-13


def test_fmm_permanent_field_water(water):
    ref = OMMPSystem(water).e_m2d()
    g = OMMPSystem(water)
    g.set_fmm(True, 8)
    assert rel(g.e_m2d(), ref) < 3e-3
    c = g.cmm + np.random.default_rng(6).normal(scale=0.05, size=(g.mm_atoms, 3))
    g.update_coordinates(c)
    f_new = g.e_m2d()
    g.set_fmm(False)
    assert rel(f_new, g.e_m2d()) < 3e-3


def test_fmm_reference_settings(water, golden_mmp):
    """ommp_set_fmm_lmax_pol / _lmax / _distance / _min_cell_size: the two
    orders set the induced-dipole and permanent-field expansions separately;
    the distance and the minimum cell size bound the leaf side from below."""
    from openmmpol_gb300 import OMMPError
    g = OMMPSystem(water)
    x = np.random.default_rng(3).standard_normal((g.pol_atoms, 3)) * 0.01
    g.set_fmm(True, 10)
    g.set_fmm_lmax_pol(8)
    assert g.fmm_settings()[:2] == (8, 10)
    ref8 = OMMPSystem(water)
    ref8.set_fmm(True, 8)
    assert np.array_equal(g.tmatvec(x, dodiag=False), ref8.tmatvec(x, dodiag=False))
    ref10 = OMMPSystem(water)
    ref10.set_fmm(True, 10)
    e10 = ref10.e_m2d()
    assert np.array_equal(g.e_m2d(), e10)  # the static order is still 10
    g.set_fmm_lmax(8)
    assert g.fmm_settings()[:2] == (8, 8)
    assert np.array_equal(g.e_m2d(), ref8.e_m2d())
    # leaf lower bound: distance, and the minimum cell size as a half diagonal
    g.set_fmm_min_cell_size(15.0)
    assert abs(g.fmm_settings()[2] - 30.0 / np.sqrt(3.0)) < 1e-12
    g.set_fmm_distance(20.0)
    assert g.fmm_settings()[2] == 20.0
    # larger leaves: more of the sum in the exact near field
    direct = OMMPSystem(water)
    yd = direct.tmatvec(x, dodiag=False)
    err_big = rel(g.tmatvec(x, dodiag=False), yd)
    err_def = rel(ref8.tmatvec(x, dodiag=False), yd)
    assert err_big < err_def
    # leaves wider than a quarter of the box: no tree, the direct sums serve
    g.set_fmm_distance(1e4)  # far beyond the ~93 bohr box
    np.testing.assert_allclose(g.tmatvec(x, dodiag=False), yd, rtol=1e-13, atol=0)
    np.testing.assert_allclose(g.e_m2d(), direct.e_m2d(), rtol=1e-13, atol=0)
    for bad in (lambda: g.set_fmm_distance(-1.0), lambda: g.set_fmm_lmax(1), lambda: g.set_fmm_lmax_pol(13)):
        with pytest.raises(OMMPError):
            bad()


def test_fmm_default_off_and_reference_auto_switch(water, golden_mmp):
    """The direct sums are the default for every size; the process-wide
    switch mirrors the reference's FMM above 1,000 MM atoms."""
    from openmmpol_gb300 import set_fmm_auto
    assert not OMMPSystem(water).use_fmm()  # 12,000 MM atoms
    set_fmm_auto(True)
    try:
        big = OMMPSystem(water)
        small = OMMPSystem(golden_mmp["1crn_amoeba"])  # 648 MM atoms
        assert big.use_fmm() and not small.use_fmm()
    finally:
        set_fmm_auto(False)
    assert not OMMPSystem(water).use_fmm()
