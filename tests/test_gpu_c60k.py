"""Full-size parity on the 60,000-site Wang-AL chain system (the precision
configuration: 150 self-avoiding chains of 200 sites in 10,000 waters,
linear Thole damping, 1-2/1-3 exclusions; synth.chain_system(seed=3)).

The oracle's full solve is a committed fixture (tests/golden/c60k_seed7.npz,
made by tests/golden/make_c60k_reference.py): energy, iteration count and
residual history, dipole norm and sum, and the dipoles and permanent field of
3,000 sampled sites.  Size-independent check beside it: the residual E - T mu
of the GPU dipoles on sampled rows, recomputed by the oracle.  Tolerances:
FP64 1e-9 relative (plain-method contract), permanent field 1e-12 (FP64) and
1e-11 (double-single); mixed precision 1e-7 relative.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from openmmpol_gb300 import OMMPSystem, set_verbose, synth
from oracle.oracle import OracleSystem

pytestmark = pytest.mark.gpu

FIX = os.path.join(GOLDEN_DIR, "c60k_seed7.npz")


@pytest.fixture(scope="module")
def c60k(tmp_path_factory):
    set_verbose(0)
    c = synth.chain_system(seed=3)
    p = synth.write_mmp(str(tmp_path_factory.mktemp("c60k") / "c60k.mmp"), c)
    g = OMMPSystem(p)
    ef, _, _ = synth.point_charge_field(g.cpol, c.box_center(), seed=7, all_sites_bohr=g.cmm)
    return p, g, ef, OracleSystem(p)


def _sampled_residual(o, g, ipd, ef, nrows=256):
    rows = np.sort(np.random.default_rng(13).choice(g.pol_atoms, nrows, replace=False)).astype(np.int32)
    tmu = o.tmatvec_rows(ipd[0], rows)
    rhs = g.e_m2d()[0][rows] + ef[rows]
    return np.abs(rhs - tmu).max() / np.abs(rhs).max()


def _check(g, ref, tol):
    ipd = g.ipd
    assert ipd.shape[1] == int(ref["pol_atoms"])
    assert abs(g.get_polelec_energy() - float(ref["energy"])) <= tol * abs(float(ref["energy"]))
    assert abs(np.linalg.norm(ipd) - float(ref["norm"])) <= tol * float(ref["norm"])
    samp = ipd[:, ref["idx"], :]
    assert np.linalg.norm(samp - ref["ipd_sample"]) <= tol * np.linalg.norm(ref["ipd_sample"])


@pytest.mark.skipif(not os.path.exists(FIX), reason="full-size fixture not generated")
@pytest.mark.parametrize("precision,tol,ftol", [("fp64", 1e-9, 1e-12), ("mixed", 1e-7, 1e-12),
                                                ("mixed-ds", 1e-7, 1e-11)])
def test_c60k_matches_oracle_fixture(c60k, precision, tol, ftol):
    p, g, ef, o = c60k
    ref = np.load(FIX)
    g.set_precision(precision)
    g.set_solver_tol(1e-10)
    g.clear_guess()
    g.set_external_field(ef)
    e = g.e_m2d()[:, ref["idx"], :]
    assert np.linalg.norm(e - ref["e_m2d_sample"]) <= ftol * np.linalg.norm(ref["e_m2d_sample"])
    _check(g, ref, tol)
    if precision == "fp64":
        # the reference's CG, iterate for iterate
        assert g.iterations(0) == int(ref["iters"][0])
        np.testing.assert_allclose(g.residual_history(0), ref["hist"], rtol=1e-6)
    else:
        assert g.residual_history(0)[-1] < 1e-10
    assert _sampled_residual(o, g, g.ipd, ef) < 1e-7
