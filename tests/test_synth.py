"""Synthetic workload generator: determinism, geometry, and that the .mmp
files it writes load in the oracle with the expected topology."""
import numpy as np

from openmmpol_gb300 import synth
from oracle.oracle import OracleSystem


def test_water_cluster_geometry_and_determinism(tmp_path):
    a = synth.water_cluster(200, seed=5)
    b = synth.water_cluster(200, seed=5)
    np.testing.assert_array_equal(a.coords, b.coords)
    O, H1, H2 = a.coords[0::3], a.coords[1::3], a.coords[2::3]
    np.testing.assert_allclose(np.linalg.norm(H1 - O, axis=1), 0.9572, atol=1e-12)
    np.testing.assert_allclose(np.linalg.norm(H2 - O, axis=1), 0.9572, atol=1e-12)
    ang = np.degrees(np.arccos(np.sum((H1 - O) * (H2 - O), 1) / 0.9572 ** 2))
    np.testing.assert_allclose(ang, 104.52, atol=1e-9)
    d = np.linalg.norm(O[:, None] - O[None], axis=-1) + np.eye(len(O)) * 10
    assert d.min() >= 2.5


def test_water_mmp_loads_with_molecular_groups(tmp_path):
    w = synth.water_cluster(50, seed=2)
    p = synth.write_mmp(str(tmp_path / "w.mmp"), w)
    s = OracleSystem(p)
    assert s.is_amoeba and s.mm_atoms == 150 and s.pol_atoms == 150
    ri, ci, sc = s.screening(1)  # D-field list: whole molecule, scale 0
    assert len(ci) == 150 * 3 and np.all(sc == 0)
    ri, ci, sc = s.screening(2)  # AMOEBA u-scale is 1 everywhere
    assert len(ci) == 0


def test_chain_system_small(tmp_path):
    c = synth.chain_system(n_chains=4, chain_len=20, n_waters=200, seed=1)
    p = synth.write_mmp(str(tmp_path / "c.mmp"), c)
    s = OracleSystem(p)
    assert not s.is_amoeba and s.pol_atoms == 80 + 600
    xyz = c.coords[:80].reshape(4, 20, 3)
    np.testing.assert_allclose(np.linalg.norm(np.diff(xyz, axis=1), axis=2), 1.53, atol=1e-9)
    ri, ci, sc = s.screening(2)  # 1-2 and 1-3 exclusions
    assert np.all(sc == 0) and len(ci) > 0


def test_point_charge_field_guard():
    w = synth.water_cluster(100, seed=1)
    c = w.coords * synth.ANG2AU
    E, q, pos = synth.point_charge_field(c, w.box_center(), seed=4, all_sites_bohr=c)
    assert E.shape == c.shape and len(q) == 30
    assert np.all(np.abs(q) <= 0.5)
    d = np.linalg.norm(c[:, None] - pos[None], axis=-1)
    assert d.min() >= 1.0 * synth.ANG2AU - 1e-12
