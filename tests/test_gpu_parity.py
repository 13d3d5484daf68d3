"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
files and against the CPU oracle on the same inputs.

Tolerances:
* reference goldens: the reference's own (ipd rtol 1e-6 / atol 1e-5, or 1e-3
  for the FMM-produced 1ubq files; EP rtol 1e-6 / atol 1e-6);
* E_M2D and T.mu against the oracle: relative 1e-12 (same FP64 formulas,
  different summation order);
* FP64 solves against the oracle at the same tolerance: relative 1e-9 in
  dipoles and energy (the plain-method contract);
* mixed precision (FP32 inner CG + FP64 refinement) against the FP64 oracle:
  relative 1e-7 in dipoles and energy.
Relative error of an array = ||a - b||_2 / ||b||_2.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES
from openmmpol_gb300 import OMMPSystem, synth
from oracle.oracle import (MATV_DIRECT, MATV_INCORE, SOLVER_CG, SOLVER_DIIS, SOLVER_INVERSION,
                           OracleSystem)

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def converged_reference(path, ef):
    """Oracle solution converged far below the comparison threshold: Jacobi/DIIS
    to a 1e-12 max increment.  The reference CG leaves its loop as converged
    once |p.Tp| < 100*eps (mod_solvers.F90:177-181), which for small systems is
    long before a 1e-10 residual, so it is not an accuracy reference."""
    o = OracleSystem(path)
    o.set_tol(1e-12)
    o.set_default_solver(SOLVER_DIIS)
    o.set_external_field(ef)
    return o


@pytest.fixture(scope="module", autouse=True)
def quiet():
    from openmmpol_gb300 import set_verbose
    set_verbose(0)


@pytest.fixture(scope="module")
def w1k(tmp_path_factory):
    w = synth.water_cluster(1000, seed=1)
    p = synth.write_mmp(str(tmp_path_factory.mktemp("w1k") / "w1k.mmp"), w)
    o = OracleSystem(p)
    cmm = o.cmm
    ef, _, _ = synth.point_charge_field(cmm[o.polar_mm], w.box_center(), seed=1, all_sites_bohr=cmm)
    return p, ef


@pytest.fixture(scope="module")
def chains(tmp_path_factory):
    c = synth.chain_system(n_chains=10, chain_len=40, n_waters=600, seed=2)
    p = synth.write_mmp(str(tmp_path_factory.mktemp("chains") / "c.mmp"), c)
    o = OracleSystem(p)
    cmm = o.cmm
    ef, _, _ = synth.point_charge_field(cmm[o.polar_mm], c.box_center(), seed=3, all_sites_bohr=cmm)
    return p, ef


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("with_field", [0, 1])
def test_gpu_matches_reference_golden(case, with_field, golden, golden_mmp):
    s = OMMPSystem(golden_mmp[case])
    ef = golden[case + "_ef1"] if with_field else np.zeros((s.pol_atoms, 3))
    s.set_external_field(ef)
    ep = s.get_polelec_energy()
    atol = float(golden[case + "_atol"])
    np.testing.assert_allclose(s.ipd.reshape(-1, 3), golden[f"{case}_ipd{with_field}"], rtol=1e-6, atol=atol)
    key = f"{case}_ep{with_field}"
    if key in golden.files:
        np.testing.assert_allclose(ep, float(golden[key]), rtol=1e-6, atol=1e-6 if atol <= 1e-5 else 1e-3)


@pytest.mark.parametrize("case", ["nma_amoeba", "nma_amoeba_cut", "nma_wang", "1crn_amoeba", "1crn_wang",
                                  "1ao6cut_wang", "1ubq_amoeba"])
def test_gpu_m2d_field_and_tmatvec_match_oracle(case, golden_mmp):
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    assert g.pol_atoms == o.pol_atoms and g.mm_atoms == o.mm_atoms
    np.testing.assert_array_equal(g.polar_mm, o.polar_mm)
    np.testing.assert_allclose(g.q, o.q, rtol=0, atol=1e-14)
    assert rel(g.e_m2d(), o.e_m2d()) < 1e-12
    x = np.random.default_rng(7).standard_normal((o.pol_atoms, 3))
    assert rel(g.tmatvec(x), o.tmatvec(x)) < 1e-12
    assert rel(g.tmatvec(x, dodiag=False), o.tmatvec(x, dodiag=False)) < 1e-12
    x2 = np.random.default_rng(8).standard_normal((2, o.pol_atoms, 3))
    y2 = g.tmatvec(x2)
    assert rel(y2[1], o.tmatvec(x2[1])) < 1e-12


@pytest.mark.parametrize("case", ["nma_amoeba", "1crn_amoeba", "1crn_wang", "1ao6cut_wang", "1ubq_amoeba",
                                  "1ubq_wang"])
@pytest.mark.parametrize("kernel", ["ordered", "symmetric"])
def test_fp64_kernel_variants_match_oracle(case, kernel, golden, golden_mmp):
    """Both FP64 T.mu kernels (all ordered pairs; each unordered pair once in
    the half-shell schedule) on 1, 6 (even) and 11 (odd) tiles of 128 sites,
    partial last tiles, and Wang exclusions."""
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    g.set_fp64_kernel(kernel)
    x = np.random.default_rng(5).standard_normal((2, o.pol_atoms, 3))
    y = g.tmatvec(x)
    for r in range(2):
        assert rel(y[r], o.tmatvec(x[r])) < 1e-12
    assert rel(g.tmatvec(x[0], dodiag=False), o.tmatvec(x[0], dodiag=False)) < 1e-12
    g.set_solver_tol(1e-10)
    o.set_tol(1e-10)
    ef = golden[case + "_ef1"]
    g.set_external_field(ef)
    o.set_external_field(ef)
    assert rel(g.ipd, o.ipd) < 1e-9


def test_symmetric_kernel_is_deterministic(w1k):
    p, _ = w1k
    g = OMMPSystem(p)
    g.set_fp64_kernel("symmetric")
    x = np.random.default_rng(9).standard_normal((g.pol_atoms, 3))
    a, b = g.tmatvec(x), g.tmatvec(x)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("case", ["nma_amoeba", "nma_wang_cut", "1crn_amoeba", "1crn_wang"])
@pytest.mark.parametrize("solver", ["cg", "diis", "inversion"])
def test_gpu_solvers_match_oracle(case, solver, golden, golden_mmp):
    code = {"cg": SOLVER_CG, "diis": SOLVER_DIIS, "inversion": SOLVER_INVERSION}[solver]
    ef = golden[case + "_ef1"]
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    # tight tolerance: DIIS stops on its increment, so runs that differ by
    # rounding stop a tolerance apart
    g.set_solver_tol(1e-12)
    o.set_tol(1e-12)
    g.set_default_solver(solver)
    o.set_default_solver(code)
    g.set_external_field(ef)
    o.set_external_field(ef)
    assert rel(g.ipd, o.ipd) < 1e-9
    assert abs(g.get_polelec_energy() - o.get_polelec_energy()) <= 1e-9 * abs(o.get_polelec_energy())


@pytest.mark.parametrize("case", ["nma_amoeba", "1crn_wang"])
def test_gpu_incore_matvec_matches_oracle(case, golden, golden_mmp):
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    x = np.random.default_rng(3).standard_normal((o.pol_atoms, 3))
    assert rel(g.tmatvec(x, matv="incore"), o.tmatvec(x, matv=MATV_INCORE)) < 1e-12
    # nomm path forwards matv (mod_interface.F90:223-230)
    ef = golden[case + "_ef1"]
    g.set_external_field(ef, nomm=True, matv="incore")
    o.set_external_field(ef, nomm=True, matv=MATV_INCORE)
    assert rel(g.ipd, o.ipd) < 1e-9


@pytest.mark.parametrize("case", ["nma_amoeba", "1crn_wang"])
def test_gpu_nomm_solves_set_one_only(case, golden, golden_mmp):
    ef = golden[case + "_ef1"]
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    g.set_external_field(ef, nomm=True)
    o.set_external_field(ef, nomm=True)
    assert rel(g.ipd, o.ipd) < 1e-9
    if g.n_ipd == 2:
        assert np.all(g.ipd[1] == 0)


def test_gpu_warm_start_and_update_coordinates(golden, golden_mmp):
    case = "1crn_amoeba"
    ef = golden[case + "_ef1"]
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    g.set_external_field(ef)
    o.set_external_field(ef)
    # second solve starts from the previous dipoles (ipd_use_guess)
    ef2 = ef * 1.01
    g.set_external_field(ef2)
    o.set_external_field(ef2)
    assert rel(g.ipd, o.ipd) < 1e-9
    assert abs(g.iterations(0) - o.last_iterations(0)) <= 1
    # new geometry: M2D and the guess are recomputed / dropped
    c = o.cmm + np.random.default_rng(1).normal(0, 0.02, o.cmm.shape)
    g.update_coordinates(c)
    o.update_coordinates(c)
    np.testing.assert_allclose(g.q, o.q, rtol=0, atol=1e-13)
    g.set_external_field(ef)
    o.set_external_field(ef)
    assert rel(g.ipd, o.ipd) < 1e-9
    assert abs(g.get_polelec_energy() - o.get_polelec_energy()) <= 1e-9 * abs(o.get_polelec_energy())


@pytest.mark.parametrize("precision", ["mixed", "mixed-ds"])
def test_mixed_solves_across_coordinate_updates(precision, golden, golden_mmp):
    # the captured inner iteration (CUDA graph) and the block preconditioner
    # rebuilt for each geometry: solves on successive geometries match the
    # oracle at each one
    case = "1ubq_amoeba"
    ef = golden[case + "_ef1"]
    g = OMMPSystem(golden_mmp[case])
    o = OracleSystem(golden_mmp[case])
    g.set_precision(precision)
    g.set_solver_tol(1e-10)
    o.set_tol(1e-12)
    o.set_default_solver(SOLVER_DIIS)
    rng = np.random.default_rng(4)
    c0 = o.cmm.copy()
    for step in range(3):
        if step:
            c = c0 + rng.normal(0, 0.02, c0.shape)
            g.update_coordinates(c)
            o.update_coordinates(c)
        g.set_external_field(ef)
        o.set_external_field(ef)
        assert rel(g.ipd, o.ipd) < 1e-7


def test_w1k_fp64_parity_and_energy(w1k):
    p, ef = w1k
    g = OMMPSystem(p)
    o = OracleSystem(p)
    g.set_solver_tol(1e-10)
    o.set_tol(1e-10)
    g.set_external_field(ef)
    o.set_external_field(ef)
    assert rel(g.ipd, o.ipd) < 1e-9
    eg, eo = g.get_polelec_energy(), o.get_polelec_energy()
    assert abs(eg - eo) <= 1e-9 * abs(eo)
    assert abs(g.iterations(0) - o.last_iterations(0)) <= 1
    hg, ho = g.residual_history(0), o.residual_history(0)
    m = min(len(hg), len(ho))
    np.testing.assert_allclose(hg[:m], ho[:m], rtol=1e-6)
    # the GPU skips only the product with the all-zero first guess
    assert abs(g.counter(0) + 1 - o.matvec_count()) <= 2


def test_w1k_mixed_precision_within_1e7(w1k):
    p, ef = w1k
    g = OMMPSystem(p)
    o = converged_reference(p, ef)
    g.set_solver_tol(1e-10)
    g.set_precision("mixed")
    g.set_external_field(ef)
    assert rel(g.ipd, o.ipd) < 1e-7
    eg, eo = g.get_polelec_energy(), o.get_polelec_energy()
    assert abs(eg - eo) <= 1e-7 * abs(eo)
    assert g.counter(2) >= 1 and g.counter(1) > 0  # refinement steps, FP32 products
    hist = g.residual_history(0)
    assert hist[-1] < 1e-10


@pytest.mark.parametrize("kernel", ["pairwise", "tiled", "symmetric"])
@pytest.mark.parametrize("case", ["w1k", "chains", "1crn_amoeba", "1crn_wang", "nma_amoeba"])
def test_fp32_operator_accuracy(case, kernel, w1k, chains, golden_mmp):
    """The FP32 kernels against the FP64 operator: relative 1e-5 overall and
    at every site (damped near pairs and scaled pairs included)."""
    p = {"w1k": w1k[0], "chains": chains[0]}.get(case) or golden_mmp[case]
    g = OMMPSystem(p)
    g.set_fp32_kernel(kernel)
    x = np.random.default_rng(2).standard_normal((g.pol_atoms, 3)) * 0.05
    y64 = g.tmatvec(x)
    y32 = g.tmatvec_fp32(x)
    assert rel(y32, y64) < 1e-5
    site = np.linalg.norm(y32 - y64, axis=1) / np.maximum(np.linalg.norm(y64, axis=1), 1e-3 * np.abs(y64).max())
    assert site.max() < 1e-4


@pytest.mark.parametrize("case", ["w1k", "chains", "1crn_amoeba", "1crn_wang", "nma_amoeba", "nma_wang"])
def test_double_single_operator_accuracy(case, w1k, chains, golden_mmp):
    """The double-single product against the FP64 one: 1e-11 relative overall
    and 1e-9 at every site (the refinement residual needs ~1e-10)."""
    p = {"w1k": w1k[0], "chains": chains[0]}.get(case) or golden_mmp[case]
    g = OMMPSystem(p)
    rng = np.random.default_rng(5)
    x = rng.standard_normal((2, g.pol_atoms, 3)) * 0.05
    y64 = g.tmatvec(x)
    yds = g.tmatvec_ds(x)
    assert rel(yds, y64) < 1e-11
    site = np.linalg.norm(yds - y64, axis=2) / np.maximum(np.linalg.norm(y64, axis=2), 1e-3 * np.abs(y64).max())
    assert site.max() < 1e-9


def test_double_single_symmetric_kernel(tmp_path):
    """From 2048 sites the double-single product evaluates each unordered pair
    once (2,100 sites: 17 tiles of 128, odd, the last one partial): the same
    bar against FP64, one and two columns, and bit-identical repeats (the
    fixed-point sums do not depend on the order of the work items)."""
    p = synth.write_mmp(str(tmp_path / "w700.mmp"), synth.water_cluster(700, seed=6))
    g = OMMPSystem(p)
    assert g.pol_atoms == 2100
    x = np.random.default_rng(6).standard_normal((2, g.pol_atoms, 3)) * 0.05
    y64 = g.tmatvec(x)
    yds = g.tmatvec_ds(x)
    assert rel(yds, y64) < 1e-11
    site = np.linalg.norm(yds - y64, axis=2) / np.maximum(np.linalg.norm(y64, axis=2), 1e-3 * np.abs(y64).max())
    assert site.max() < 1e-9
    y1 = g.tmatvec_ds(x[0])
    assert rel(y1, y64[0]) < 1e-11
    assert np.array_equal(y1, g.tmatvec_ds(x[0]))


@pytest.mark.parametrize("case", ["w1k", "chains", "1crn_amoeba", "1crn_wang", "nma_amoeba", "nma_wang_cut",
                                  "1ubq_amoeba"])
def test_double_single_m2d_accuracy(case, w1k, chains, golden_mmp):
    """E_M2D of the mixed-ds mode (all pairs in double-single, scaled pairs
    in FP64) against the FP64 field: 1e-11 relative, 1e-9 per site; back in
    FP64 mode the field is recomputed in FP64."""
    p = {"w1k": w1k[0], "chains": chains[0]}.get(case) or golden_mmp[case]
    e64 = OMMPSystem(p).e_m2d()
    g = OMMPSystem(p)
    g.set_precision("mixed-ds")
    eds = g.e_m2d()
    assert rel(eds, e64) < 1e-11
    site = np.linalg.norm(eds - e64, axis=2) / np.maximum(np.linalg.norm(e64, axis=2), 1e-3 * np.abs(e64).max())
    assert site.max() < 1e-9
    g.set_precision("fp64")
    assert rel(g.e_m2d(), e64) < 1e-13


@pytest.mark.parametrize("case", ["w1k", "chains"])
def test_mixed_ds_solve(case, w1k, chains):
    p, ef = {"w1k": w1k, "chains": chains}[case]
    ref = converged_reference(p, ef)
    g = OMMPSystem(p)
    g.set_solver_tol(1e-10)
    g.set_precision("mixed-ds")
    g.set_external_field(ef)
    assert rel(g.ipd, ref.ipd) < 1e-7
    assert abs(g.get_polelec_energy() - ref.get_polelec_energy()) <= 1e-7 * abs(ref.get_polelec_energy())
    assert g.counter(4) >= 1 and g.counter(0) == 0  # residual products in double-single, none in FP64
    assert g.residual_history(0)[-1] < 1e-10


@pytest.mark.parametrize("case", ["w1k", "chains", "1crn_amoeba"])
def test_refinement_residual_update_and_recompute(case, w1k, chains, golden, golden_mmp):
    """mixed-ds updates the refinement residual after the first recomputed
    one by the FP32 product of the step's correction (fewer double-single
    products); the strict mode recomputes every residual in FP64 unless told
    to update.  Every variant reaches the converged reference within 1e-7 and
    its certified residual below the tolerance.  The protein's D and P
    right-hand sides differ, so its products and updates take two columns."""
    if case in ("w1k", "chains"):
        p, ef = {"w1k": w1k, "chains": chains}[case]
    else:
        p, ef = golden_mmp[case], golden[case + "_ef1"]
    ref = converged_reference(p, ef)
    res = {}
    for prec, mode in (("mixed-ds", "auto"), ("mixed-ds", "recompute"), ("mixed", "auto"), ("mixed", "update")):
        g = OMMPSystem(p)
        g.set_solver_tol(1e-10)
        g.set_precision(prec)
        g.set_residual_update(mode)
        g.set_external_field(ef)
        assert rel(g.ipd, ref.ipd) < 1e-7, (prec, mode)
        assert abs(g.get_polelec_energy() - ref.get_polelec_energy()) <= 1e-7 * abs(ref.get_polelec_energy())
        assert g.residual_history(0)[-1] < 1e-10
        expect_update = mode == "update" or (mode == "auto" and prec == "mixed-ds")
        assert (g.counter(5) >= 1) == expect_update, (prec, mode, g.counter(5))
        res[(prec, mode)] = g
    assert res[("mixed-ds", "auto")].counter(4) < res[("mixed-ds", "recompute")].counter(4)
    assert res[("mixed", "update")].counter(0) < res[("mixed", "auto")].counter(0)
    with pytest.raises(Exception):
        res[("mixed", "auto")].set_residual_update(2)


@pytest.mark.parametrize("precond", ["diagonal", "block", "near"])
@pytest.mark.parametrize("case", ["w1k", "chains", "1crn_amoeba", "1crn_wang", "nma_amoeba"])
def test_mixed_solve_with_each_inner_preconditioner(case, precond, w1k, chains, golden, golden_mmp):
    """The inner preconditioner changes only the FP32 inner iterations: both
    reach the converged reference within the mixed-precision tolerance."""
    if case in ("w1k", "chains"):
        p, ef = {"w1k": w1k, "chains": chains}[case]
    else:
        p, ef = golden_mmp[case], golden[case + "_ef1"]
    ref = converged_reference(p, ef)
    g = OMMPSystem(p)
    g.set_solver_tol(1e-10)
    g.set_precision("mixed")
    g.set_inner_preconditioner(precond)
    g.set_external_field(ef)
    assert rel(g.ipd, ref.ipd) < 1e-7
    assert g.residual_history(0)[-1] < 1e-10


def test_block_preconditioner_saves_inner_iterations(w1k):
    p, ef = w1k
    counts = {}
    for precond in ("diagonal", "block", "near"):
        g = OMMPSystem(p)
        g.set_solver_tol(1e-10)
        g.set_precision("mixed")
        g.set_inner_preconditioner(precond)
        g.set_external_field(ef)
        counts[precond] = g.counter(1)
    assert counts["block"] < counts["diagonal"]
    assert counts["near"] <= counts["block"]  # the Neumann step over the near field


@pytest.mark.parametrize("case", ["w1k", "1crn_amoeba", "chains"])
def test_symmetric_fp32_operator_two_columns_and_determinism(case, w1k, chains, golden_mmp):
    """The symmetric FP32 kernel (each unordered pair once, fixed-point sums):
    two columns in one launch equal to the columns one at a time within FP32
    rounding, both within 1e-5 of FP64, and bitwise repeatable."""
    p = {"w1k": w1k[0], "chains": chains[0]}.get(case) or golden_mmp[case]
    g = OMMPSystem(p)
    g.set_fp32_kernel("symmetric")
    x = np.random.default_rng(5).standard_normal((2, g.pol_atoms, 3)) * 0.05
    y2 = g.tmatvec_fp32(x)
    assert np.array_equal(y2, g.tmatvec_fp32(x))
    y64 = g.tmatvec(x)
    assert rel(y2, y64) < 1e-5
    for c in range(2):
        assert rel(g.tmatvec_fp32(x[c]), y64[c]) < 1e-5


@pytest.mark.parametrize("kernel", ["pairwise", "tiled", "symmetric", "auto"])
def test_mixed_solve_with_each_fp32_kernel(kernel, chains):
    p, ef = chains
    ref = converged_reference(p, ef).ipd
    g = OMMPSystem(p)
    g.set_fp32_kernel(kernel)
    g.set_solver_tol(1e-10)
    g.set_precision("mixed")
    assert g.fp32_shape(1) is None  # nothing tuned before the first solve
    g.set_external_field(ef)
    assert rel(g.ipd, ref) < 1e-7
    shape = g.fp32_shape(1)
    assert shape is not None and shape[1] == 1 and shape[2] >= 1
    assert shape[0] == kernel if kernel != "auto" else shape[0] in ("pairwise", "tiled", "symmetric")


def test_chain_system_wang_exclusions(chains):
    p, ef = chains
    g = OMMPSystem(p)
    o = OracleSystem(p)
    assert rel(g.e_m2d(), o.e_m2d()) < 1e-12
    x = np.random.default_rng(4).standard_normal((o.pol_atoms, 3))
    assert rel(g.tmatvec(x), o.tmatvec(x)) < 1e-12
    g.set_solver_tol(1e-10)
    o.set_tol(1e-10)
    g.set_external_field(ef)
    o.set_external_field(ef)
    assert rel(g.ipd, o.ipd) < 1e-9
    ref = converged_reference(p, ef).ipd
    g.clear_guess()
    g.set_precision("mixed")
    g.set_external_field(ef)
    assert rel(g.ipd, ref) < 1e-7


def test_solver_not_converged_reports_status(golden, golden_mmp):
    from openmmpol_gb300 import OMMPError
    g = OMMPSystem(golden_mmp["1crn_amoeba"])
    g.set_solver_maxiter(2)
    with pytest.raises(OMMPError) as e:
        g.set_external_field(golden["1crn_amoeba_ef1"])
    assert e.value.status == 2
    # the system stays usable
    g.set_solver_maxiter(200)
    g.set_external_field(golden["1crn_amoeba_ef1"])
    np.testing.assert_allclose(g.ipd.reshape(-1, 3), golden["1crn_amoeba_ipd1"], rtol=1e-6, atol=1e-5)
