"""The oracle's potential and field at external points (the reference's
ommp_{potential,field}_{mmpol,mm,pol}2ext, src/mod_electrostatics.F90:3067-3336).

The reference ships no golden file for these, so the restatement is pinned by
physics and by independent formulas:
* the static-multipole field is minus the gradient of the static potential
  (central finite differences, AMOEBA multipoles and Wang-AL charges);
* the induced-dipole potential and field equal a numpy evaluation of the
  point-dipole formulas on the oracle's own dipoles (D set for the potential,
  (P + D) / 2 for the AMOEBA field, as the reference does);
* for a charge-only system the static field equals the point-charge field
  used to build external fields (openmmpol_gb300.synth);
* results are added into the caller's array, and the induced part refuses to
  run before a solve.
"""
import numpy as np
import pytest

from openmmpol_gb300 import synth
from oracle.oracle import OracleError, OracleSystem


def points_around(o, n, seed):
    rng = np.random.default_rng(seed)
    c = o.cmm
    lo, hi = c.min(0) - 8.0, c.max(0) + 8.0
    pts = []
    while len(pts) < n:
        p = rng.uniform(lo, hi)
        if np.min(np.linalg.norm(c - p, axis=1)) > 1.5:
            pts.append(p)
    return np.array(pts)


@pytest.mark.parametrize("case", ["1crn_amoeba", "1crn_wang", "nma_amoeba", "1ao6cut_wang"])
def test_static_field_is_minus_gradient_of_potential(case, golden_mmp):
    o = OracleSystem(golden_mmp[case])
    pts = points_around(o, 24, 1)
    e = o.field_ext(1, pts)
    h = 1e-4
    g = np.zeros_like(pts)
    for c in range(3):
        d = np.zeros(3)
        d[c] = h
        g[:, c] = -(o.potential_ext(1, pts + d) - o.potential_ext(1, pts - d)) / (2 * h)
    assert np.abs(g - e).max() <= 1e-6 * np.abs(e).max()


@pytest.mark.parametrize("case", ["1crn_amoeba", "1crn_wang"])
def test_induced_potential_and_field_match_point_dipoles(case, golden_mmp):
    o = OracleSystem(golden_mmp[case])
    pts = points_around(o, 16, 2)
    with pytest.raises(OracleError):
        o.potential_ext(2, pts)
    ef = np.random.default_rng(3).standard_normal((o.pol_atoms, 3)) * 1e-3
    o.set_external_field(ef)
    ipd = o.ipd
    cpol = o.cmm[o.polar_mm]
    mu_v = ipd[0]
    mu_e = 0.5 * (ipd[0] + ipd[1]) if o.is_amoeba else ipd[0]
    dr = pts[:, None, :] - cpol[None, :, :]
    r = np.linalg.norm(dr, axis=2)
    v_ref = (np.einsum("jik,ik->ji", dr, mu_v) / r ** 3).sum(1)
    mdr = np.einsum("jik,ik->ji", dr, mu_e)
    e_ref = (3 * mdr[:, :, None] * dr / r[:, :, None] ** 5 - mu_e[None] / r[:, :, None] ** 3).sum(1)
    v = o.potential_ext(2, pts)
    e = o.field_ext(2, pts)
    assert np.abs(v - v_ref).max() <= 1e-12 * np.abs(v_ref).max()
    assert np.abs(e - e_ref).max() <= 1e-12 * np.abs(e_ref).max()
    # which = 0 is the sum of the two parts, added into the caller's array
    v0 = np.arange(len(pts), dtype=float)
    tot = o.potential_ext(0, pts, v0)
    assert np.allclose(tot, v0 + o.potential_ext(1, pts) + v, rtol=1e-13, atol=1e-13)
    e0 = np.ones((len(pts), 3))
    tot = o.field_ext(0, pts, e0)
    assert np.allclose(tot, e0 + o.field_ext(1, pts) + e, rtol=1e-13, atol=1e-13)


def test_charge_only_field_is_the_point_charge_field(tmp_path):
    c = synth.chain_system(n_chains=3, chain_len=20, n_waters=40, seed=5)
    p = synth.write_mmp(str(tmp_path / "c.mmp"), c)
    o = OracleSystem(p)
    assert not o.is_amoeba
    pts = points_around(o, 12, 4)
    e = o.field_ext(1, pts)
    q = o.q[:, 0]
    dr = pts[:, None, :] - o.cmm[None, :, :]
    r = np.linalg.norm(dr, axis=2)
    e_ref = (q[None, :, None] * dr / r[:, :, None] ** 3).sum(1)
    assert np.abs(e - e_ref).max() <= 1e-12 * np.abs(e_ref).max()
