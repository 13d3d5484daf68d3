"""Full-size parity on the 90,000-site water box (the benchmark geometry).

The oracle's full solve takes ~7 minutes on 8 cores, so its result is a
committed fixture (tests/golden/w30k_seed103.npz, made by
tests/golden/make_w30k_reference.py): energy, dipole norms and sums, and the
dipoles of 3,000 sampled sites.  Size-independent checks complement it: the
residual E - T mu of the GPU dipoles on sampled rows, recomputed by the
oracle.  Tolerances: FP64 1e-9 relative (plain-method contract); mixed
precision 1e-7 relative.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from openmmpol_gb300 import OMMPSystem, set_verbose, synth
from oracle.oracle import OracleSystem

pytestmark = pytest.mark.gpu

FIX = os.path.join(GOLDEN_DIR, "w30k_seed103.npz")


@pytest.fixture(scope="module")
def w30k(tmp_path_factory):
    set_verbose(0)
    w = synth.water_cluster(30000, seed=1)
    p = synth.write_mmp(str(tmp_path_factory.mktemp("w30k") / "w30k.mmp"), w)
    g = OMMPSystem(p)
    cmm = g.cmm
    ef, _, _ = synth.point_charge_field(g.cpol, w.box_center(), seed=103, all_sites_bohr=cmm)
    g.center = w.box_center()
    return p, g, ef


@pytest.fixture(scope="module")
def w30k_oracle(w30k):
    return OracleSystem(w30k[0])


def _check_against_fixture(g, ref, tol):
    ipd = g.ipd
    assert abs(g.get_polelec_energy() - float(ref["energy"])) <= tol * abs(float(ref["energy"]))
    np.testing.assert_allclose(np.linalg.norm(ipd.reshape(2, -1), axis=1), ref["norms"], rtol=tol)
    samp = ipd[:, ref["idx"], :]
    assert np.linalg.norm(samp - ref["ipd_sample"]) <= tol * np.linalg.norm(ref["ipd_sample"])


def _sampled_residual(p, g, ef, nrows=256, ipd_d=None, o=None):
    """max over sampled rows of |E - T mu| / max |E| for the D set, via the oracle."""
    o = o or OracleSystem(p)
    ipd_d = g.ipd[0] if ipd_d is None else ipd_d
    rows = np.sort(np.random.default_rng(11).choice(g.pol_atoms, nrows, replace=False)).astype(np.int32)
    tmu = o.tmatvec_rows(ipd_d, rows)
    rhs = g.e_m2d()[0][rows] + ef[rows]
    return np.abs(rhs - tmu).max() / np.abs(rhs).max()


@pytest.mark.skipif(not os.path.exists(FIX), reason="full-size fixture not generated")
def test_w30k_fp64_matches_oracle_fixture(w30k):
    p, g, ef = w30k
    ref = np.load(FIX)
    g.set_precision("fp64")
    g.set_solver_tol(1e-10)
    g.clear_guess()
    g.set_external_field(ef)
    assert [g.iterations(0), g.iterations(1)] == list(ref["iters"])
    np.testing.assert_allclose(g.residual_history(0), ref["hist_d"], rtol=1e-6)
    _check_against_fixture(g, ref, 1e-9)
    assert _sampled_residual(p, g, ef) < 1e-7


@pytest.mark.skipif(not os.path.exists(FIX), reason="full-size fixture not generated")
def test_w30k_mixed_precision_matches_oracle_fixture(w30k):
    p, g, ef = w30k
    ref = np.load(FIX)
    g.set_precision("mixed")
    g.set_solver_tol(1e-10)
    g.clear_guess()
    g.set_external_field(ef)
    _check_against_fixture(g, ref, 1e-7)
    assert g.residual_history(0)[-1] < 1e-10
    assert _sampled_residual(p, g, ef) < 1e-7


def test_w30k_mixed_ds_matches_oracle_fixture(w30k):
    p, g, ef = w30k
    ref = np.load(FIX)
    g.set_precision("mixed-ds")
    g.set_solver_tol(1e-10)
    g.clear_guess()
    g.set_external_field(ef)
    _check_against_fixture(g, ref, 1e-7)
    assert g.residual_history(0)[-1] < 1e-10
    assert g.counter(0) == 0 and g.counter(4) >= 1
    assert _sampled_residual(p, g, ef) < 1e-7
    g.set_precision("fp64")


def test_b64_full_batch_columns_pinned_by_oracle(w30k, w30k_oracle):
    """The batching configuration at its full size: 64 fields of 30 point
    charges (seeds 1000..1063) on the 90,000-site box in one batched strict
    mixed solve.  Three columns are checked against the oracle's residual rows
    (E - T mu on 256 sampled rows below 1e-7 of max |E|) and against single
    plain-FP64 solves of the same fields (1e-7 relative)."""
    p, g, _ = w30k
    fields = np.stack([synth.point_charge_field(g.cpol, g.center, seed=1000 + r, all_sites_bohr=g.cmm)[0]
                       for r in range(64)])
    g.set_precision("mixed")
    g.set_solver_tol(1e-10)
    ipd, en = g.set_external_fields_batch(fields)
    assert np.array_equal(ipd[:, 0], ipd[:, 1])  # water: D and P coincide
    g.set_precision("fp64")
    for r in (0, 31, 63):
        assert _sampled_residual(p, g, fields[r], ipd_d=ipd[r, 0], o=w30k_oracle) < 1e-7
        g.clear_guess()
        g.set_external_field(fields[r])
        assert np.linalg.norm(ipd[r] - g.ipd) <= 1e-7 * np.linalg.norm(g.ipd)
        assert abs(en[r] - g.get_polelec_energy()) <= 1e-7 * abs(g.get_polelec_energy())
