"""Potential and field at external points on the GPU (the reference's
ommp_{potential,field}_{mmpol,mm,pol}2ext) against the oracle and against a
numpy evaluation of the point-dipole formulas on the GPU's own dipoles.

Tolerances: static multipoles against the oracle 1e-12 (same FP64 formulas,
different summation order); the induced part against numpy on the same
dipoles 1e-12, and against the oracle (whose dipoles agree with the GPU's to
the plain-solver contract) 1e-8.  Results are added into the caller's array.
"""
import ctypes as C

import numpy as np
import pytest

from openmmpol_gb300 import OMMPError, OMMPSystem, _lib, set_verbose, synth
from oracle.oracle import OracleSystem

pytestmark = pytest.mark.gpu


def maxrel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / np.abs(b).max()


def points_around(cmm, n, seed, guard=1.5):
    rng = np.random.default_rng(seed)
    lo, hi = cmm.min(0) - 8.0, cmm.max(0) + 8.0
    pts = []
    while len(pts) < n:
        p = rng.uniform(lo, hi, size=(4 * n, 3))
        for q in p:
            if np.min(np.linalg.norm(cmm - q, axis=1)) > guard:
                pts.append(q)
                if len(pts) == n:
                    break
    return np.array(pts)


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


@pytest.mark.parametrize("case", ["1crn_amoeba", "1crn_wang", "nma_amoeba", "1ubq_amoeba", "1ao6cut_wang"])
def test_external_points_match_oracle(case, golden_mmp):
    p = golden_mmp[case]
    g, o = OMMPSystem(p), OracleSystem(p)
    pts = points_around(o.cmm, 300, 7)
    # static multipoles: no solve needed
    assert maxrel(g.potential_mm2ext(pts), o.potential_ext(1, pts)) < 1e-12
    assert maxrel(g.field_mm2ext(pts), o.field_ext(1, pts)) < 1e-12
    # the induced part refuses to run before a solve
    with pytest.raises(OMMPError) as e:
        g.potential_pol2ext(pts)
    assert e.value.status == 1
    ef = np.random.default_rng(8).standard_normal((g.pol_atoms, 3)) * 1e-3
    g.set_solver_tol(1e-10)
    o.set_tol(1e-10)
    g.set_external_field(ef)
    o.set_external_field(ef)
    ipd = g.ipd
    cpol = g.cpol
    mu_v = ipd[0]
    mu_e = 0.5 * (ipd[0] + ipd[1]) if g.is_amoeba else ipd[0]
    dr = pts[:, None, :] - cpol[None, :, :]
    r = np.linalg.norm(dr, axis=2)
    v_np = (np.einsum("jik,ik->ji", dr, mu_v) / r ** 3).sum(1)
    mdr = np.einsum("jik,ik->ji", dr, mu_e)
    e_np = (3 * mdr[:, :, None] * dr / r[:, :, None] ** 5 - mu_e[None] / r[:, :, None] ** 3).sum(1)
    assert maxrel(g.potential_pol2ext(pts), v_np) < 1e-12
    assert maxrel(g.field_pol2ext(pts), e_np) < 1e-12
    assert maxrel(g.potential_pol2ext(pts), o.potential_ext(2, pts)) < 1e-8
    assert maxrel(g.field_pol2ext(pts), o.field_ext(2, pts)) < 1e-8
    assert maxrel(g.potential_mmpol2ext(pts), o.potential_ext(0, pts)) < 1e-8
    assert maxrel(g.field_mmpol2ext(pts), o.field_ext(0, pts)) < 1e-8


def test_legacy_calls_add_into_the_callers_array(golden_mmp):
    p = golden_mmp["1crn_amoeba"]
    g = OMMPSystem(p)
    g.set_external_field(np.zeros((g.pol_atoms, 3)))
    pts = np.ascontiguousarray(points_around(g.cmm, 50, 9))
    L = _lib.load()
    dp = _lib._dp
    v = np.full(len(pts), 2.5)
    L.ommp_potential_mmpol2ext(g._h, len(pts), pts.ctypes.data_as(dp), v.ctypes.data_as(dp))
    assert np.allclose(v, 2.5 + g.potential_mmpol2ext(pts), rtol=1e-14, atol=1e-14)
    e = np.full((len(pts), 3), -1.0)
    L.ommp_field_pol2ext(g._h, len(pts), pts.ctypes.data_as(dp), e.ctypes.data_as(dp))
    assert np.allclose(e, -1.0 + g.field_pol2ext(pts), rtol=1e-14, atol=1e-14)
    # which = all equals the sum of its parts
    assert np.allclose(g.field_mmpol2ext(pts), g.field_mm2ext(pts) + g.field_pol2ext(pts), rtol=1e-12,
                       atol=1e-15)


def test_many_points_water(tmp_path):
    w = synth.water_cluster(1000, seed=1)
    p = synth.write_mmp(str(tmp_path / "w.mmp"), w)
    g, o = OMMPSystem(p), OracleSystem(p)
    pts = points_around(o.cmm, 4000, 11, guard=1.0)
    assert maxrel(g.potential_mm2ext(pts), o.potential_ext(1, pts)) < 1e-12
    assert maxrel(g.field_mm2ext(pts), o.field_ext(1, pts)) < 1e-12
