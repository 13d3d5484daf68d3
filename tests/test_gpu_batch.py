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
