"""Batched right-hand sides (ommp_gpu_set_external_fields_batch): each field's
result must equal the single-field solve of the same field from a zero guess.

FP64 mode runs the reference CG per column with shared products, so it must
agree with the single solves to 1e-9 (relative); mixed mode must stay within
1e-7 of a converged FP64 oracle.  Covers AMOEBA with different D and P
right-hand sides (protein), AMOEBA water (identical D and P: one set of
columns), Wang-AL (one set), and graph capture on and off.
"""
import numpy as np
import pytest

from openmmpol_gb300 import OMMPSystem, set_verbose, synth
from oracle.oracle import SOLVER_DIIS, OracleSystem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def fields_for(s, nf, seed):
    rng = np.random.default_rng(seed)
    base = rng.standard_normal((s.pol_atoms, 3)) * 1e-3
    return np.stack([base * (1 + 0.3 * k) + rng.standard_normal((s.pol_atoms, 3)) * 2e-4 for k in range(nf)])


def singles(path, fields, precision):
    g = OMMPSystem(path)
    g.set_precision(precision)
    g.set_solver_tol(1e-10)
    out, en = [], []
    for f in fields:
        g.clear_guess()
        g.set_external_field(f)
        out.append(g.ipd)
        en.append(g.get_polelec_energy())
    return np.stack(out), np.array(en)


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


@pytest.fixture(scope="module")
def water(tmp_path_factory):
    w = synth.water_cluster(700, seed=4)
    return synth.write_mmp(str(tmp_path_factory.mktemp("wb") / "w.mmp"), w)


@pytest.mark.parametrize("case", ["1crn_amoeba", "1crn_wang", "nma_amoeba"])
def test_batch_fp64_equals_single_solves(case, golden_mmp):
    p = golden_mmp[case]
    g = OMMPSystem(p)
    g.set_solver_tol(1e-10)
    fields = fields_for(g, 5, 1)
    ipd, en = g.set_external_fields_batch(fields)
    ref, ren = singles(p, fields, "fp64")
    for k in range(len(fields)):
        assert rel(ipd[k], ref[k]) < 1e-9
    np.testing.assert_allclose(en, ren, rtol=1e-9)


@pytest.mark.parametrize("case", ["1crn_amoeba", "1crn_wang"])
@pytest.mark.parametrize("graphs", [True, False])
def test_batch_mixed_within_1e7_of_converged_oracle(case, graphs, golden_mmp):
    p = golden_mmp[case]
    g = OMMPSystem(p)
    g.set_solver_tol(1e-10)
    g.set_precision("mixed")
    g.set_use_graphs(graphs)
    fields = fields_for(g, 4, 2)
    ipd, en = g.set_external_fields_batch(fields)
    for k in range(len(fields)):
        o = OracleSystem(p)
        o.set_tol(1e-12)
        o.set_default_solver(SOLVER_DIIS)
        o.set_external_field(fields[k])
        assert rel(ipd[k], o.ipd) < 1e-7
        assert abs(en[k] - o.get_polelec_energy()) <= 1e-7 * abs(o.get_polelec_energy())


def test_batch_water_identical_sets_and_system_state_untouched(water):
    g = OMMPSystem(water)
    g.set_solver_tol(1e-10)
    g.set_precision("mixed")
    cmm = g.cmm
    fields = np.stack([synth.point_charge_field(g.cpol, cmm.mean(0) / synth.ANG2AU, seed=s,
                                                all_sites_bohr=cmm)[0] for s in range(6)])
    g.set_external_field(fields[0])
    before = g.ipd
    ipd, en = g.set_external_fields_batch(fields)
    assert np.array_equal(g.ipd, before)  # the batch leaves the system's dipoles alone
    assert np.array_equal(ipd[:, 0], ipd[:, 1])  # water: D and P systems coincide
    # single mixed solves converge to the same 1e-10 residual
    ref, ren = singles(water, fields, "mixed")
    for k in range(len(fields)):
        assert rel(ipd[k], ref[k]) < 1e-7
    np.testing.assert_allclose(en, ren, rtol=1e-7)


def test_batch_fp64_water_four_column_groups(water):
    """2,100 sites: the symmetric FP64 product runs the 6 columns of the batch
    as a 4-column and a 2-column group (one pair geometry per group); the CG
    per column must still equal the single-field solves to 1e-9."""
    g = OMMPSystem(water)
    g.set_solver_tol(1e-10)
    cmm = g.cmm
    fields = np.stack([synth.point_charge_field(g.cpol, cmm.mean(0) / synth.ANG2AU, seed=20 + s,
                                                all_sites_bohr=cmm)[0] for s in range(6)])
    ipd, en = g.set_external_fields_batch(fields)
    ref, ren = singles(water, fields, "fp64")
    for k in range(len(fields)):
        assert rel(ipd[k], ref[k]) < 1e-9
    np.testing.assert_allclose(en, ren, rtol=1e-9)


@pytest.mark.parametrize("case,precision", [("water", "mixed"), ("1crn_amoeba", "mixed"), ("water", "mixed-ds"),
                                            ("chains", "mixed")])
def test_block_cg_inner_solve(case, precision, water, golden_mmp, tmp_path):
    """Batches of at least 4 columns share one Krylov space in the FP32
    inner solve (block CG): the results equal the independent per-column
    inner solves within 1e-7, the block needs no more inner iterations than
    the independent columns do, and the outer refinement still ends below the
    1e-10 residual (checked against single solves)."""
    if case == "water":
        p = water
    elif case == "chains":
        c = synth.chain_system(n_chains=10, chain_len=40, n_waters=600, seed=2)
        p = synth.write_mmp(str(tmp_path / "c.mmp"), c)
    else:
        p = golden_mmp[case]
    res = {}
    for block in (True, False):
        g = OMMPSystem(p)
        g.set_solver_tol(1e-10)
        g.set_precision(precision)
        g.set_block_cg(block)
        cmm = g.cmm
        fields = np.stack([synth.point_charge_field(g.cpol, cmm.mean(0) / synth.ANG2AU, seed=40 + s,
                                                    all_sites_bohr=cmm)[0] for s in range(8)])
        ipd, en = g.set_external_fields_batch(fields)
        res[block] = (ipd, en, g.counter(3), g.counter(1))
    ipd_b, en_b, inner_b, prod_b = res[True]
    ipd_i, en_i, inner_i, prod_i = res[False]
    for k in range(8):
        assert rel(ipd_b[k], ipd_i[k]) < 1e-7
    np.testing.assert_allclose(en_b, en_i, rtol=1e-7)
    assert inner_b <= inner_i and prod_b <= prod_i
    ref, _ = singles(p, fields[:2], precision)
    for k in range(2):
        assert rel(ipd_b[k], ref[k]) < 1e-7


@pytest.mark.parametrize("precision", ["mixed", "mixed-ds"])
def test_batch_residual_update_matches_recompute(precision, water):
    """A batch whose later refinement residuals are updated by the FP32
    product of the step's correction reaches the dipoles of one that
    recomputes every residual (the iterates are the same, only the residual
    that certifies convergence differs) with fewer residual products, and
    both stay within 1e-7 of the single solves."""
    res = {}
    for mode in ("update", "recompute"):
        g = OMMPSystem(water)
        g.set_solver_tol(1e-10)
        g.set_precision(precision)
        g.set_residual_update(mode)
        cmm = g.cmm
        fields = np.stack([synth.point_charge_field(g.cpol, cmm.mean(0) / synth.ANG2AU, seed=70 + s,
                                                    all_sites_bohr=cmm)[0] for s in range(6)])
        ipd, en = g.set_external_fields_batch(fields)
        res[mode] = (ipd, en, g.counter(2), g.counter(5), g.counter(0) + g.counter(4))
    ipd_u, en_u, outer_u, upd_u, prod_u = res["update"]
    ipd_r, en_r, outer_r, upd_r, prod_r = res["recompute"]
    assert upd_u >= 1 and upd_r == 0
    assert prod_u < prod_r
    if outer_u == outer_r:
        assert rel(ipd_u, ipd_r) < 1e-12
    ref, _ = singles(water, fields[:2], precision)
    for k in range(2):
        assert rel(ipd_u[k], ref[k]) < 1e-7

