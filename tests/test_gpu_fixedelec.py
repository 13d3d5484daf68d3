"""Interaction energy of the static multipoles on the GPU
(ommp_get_fixedelec_energy, energy_MM_MM src/mod_electrostatics.F90:899-941)
against the reference's EM goldens (printed to 13 digits: 1e-11 relative) and
against the oracle on a synthetic water box and after a coordinate update
(1e-9: the water total is ~1,000 times smaller than its largest site terms,
whose FP64 sums differ in order between the two)."""
import numpy as np
import pytest

from openmmpol_gb300 import OMMPSystem, set_verbose, synth
from oracle.oracle import OracleSystem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


@pytest.mark.parametrize("case", ["nma_amoeba", "nma_wang", "1crn_amoeba", "1crn_wang", "1ao6cut_wang",
                                  "1ubq_amoeba", "1ubq_wang"])
def test_static_energy_matches_golden(case, golden, golden_mmp):
    g = OMMPSystem(golden_mmp[case])
    ref = float(golden[case + "_em"])
    assert abs(g.get_fixedelec_energy() - ref) <= 1e-11 * abs(ref) + 1e-14


def test_static_energy_water_and_update(tmp_path):
    p = synth.write_mmp(str(tmp_path / "w.mmp"), synth.water_cluster(1500, seed=4))
    g, o = OMMPSystem(p), OracleSystem(p)
    e = g.get_fixedelec_energy()
    assert abs(e - o.get_fixedelec_energy()) <= 1e-9 * abs(e)
    assert g.get_fixedelec_energy() == e  # cached per geometry
    c = g.cmm + np.random.default_rng(2).normal(scale=0.05, size=(g.mm_atoms, 3))
    g.update_coordinates(c)
    o.update_coordinates(c)
    e2 = g.get_fixedelec_energy()
    assert e2 != e
    assert abs(e2 - o.get_fixedelec_energy()) <= 1e-9 * abs(e2)
