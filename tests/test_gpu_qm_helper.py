"""QM helper on the GPU (ommp_init_qm_helper, ommp_prepare_qm_ele_ene /
_grd and the getters, src/mod_qm_helper.F90:80-161,356-520) against the
oracle: the nuclear fields (orc_nuclei_fields) and the MM-side potential /
field at the nuclei (orc_potential_ext / orc_field_ext, the oracle evaluated
on the GPU's own dipoles), 1e-12 relative; and the helper's bookkeeping
(what is available when, what update_coord resets) as the reference has it.
"""
import numpy as np
import pytest

from openmmpol_gb300 import OMMPError, OMMPQmHelper, OMMPSystem, set_verbose
from oracle.oracle import OracleSystem

pytestmark = pytest.mark.gpu


def maxrel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


def nuclei_near(cmm, n, seed, guard=2.0):
    rng = np.random.default_rng(seed)
    lo, hi = cmm.min(0) - 4.0, cmm.max(0) + 4.0
    out = []
    while len(out) < n:
        p = rng.uniform(lo, hi)
        if np.min(np.linalg.norm(cmm - p, axis=1)) > guard:
            out.append(p)
    z = rng.integers(1, 9, n).astype(np.int32)
    return np.array(out), z.astype(np.float64), z


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


@pytest.mark.parametrize("case", ["1crn_amoeba", "1crn_wang", "nma_amoeba", "1ubq_amoeba"])
def test_qm_helper_matches_oracle(case, golden_mmp):
    p = golden_mmp[case]
    g, o = OMMPSystem(p), OracleSystem(p)
    cqm, qqm, zqm = nuclei_near(o.cmm, 12, 3)
    qm = OMMPQmHelper(cqm, qqm, zqm)
    assert qm.qm_atoms == 12 and qm.npol == 0 and qm.nmm == 0
    np.testing.assert_array_equal(qm.cqm, cqm)
    with pytest.raises(AttributeError):
        qm.E_n2p
    # energy quantities; no dipoles yet, so no V_p2n
    qm.prepare_qm_ele_ene(g)
    assert qm.npol == g.pol_atoms
    assert maxrel(qm.E_n2p, o.nuclei_fields(cqm, qqm)) < 1e-12
    assert maxrel(qm.V_m2n, o.potential_ext(1, cqm)) < 1e-12
    with pytest.raises(AttributeError):
        qm.V_p2n
    # the nuclei polarize the system; then the induced part
    g.set_solver_tol(1e-10)
    g.set_external_field(qm.E_n2p)
    qm.prepare_qm_ele_ene(g)
    o.set_ipd(g.ipd)
    assert maxrel(qm.V_p2n, o.potential_ext(2, cqm)) < 1e-12
    # gradient quantities
    qm.prepare_qm_ele_grd(g)
    E, G, H = o.nuclei_fields(cqm, qqm, grad=True)
    assert qm.nmm == g.mm_atoms
    assert maxrel(qm.E_n2m, E) < 1e-12
    assert maxrel(qm.G_n2m, G) < 1e-12
    assert maxrel(qm.H_n2m, H) < 1e-12
    np.testing.assert_array_equal(qm.G_n2p, qm.G_n2m[g.polar_mm])
    assert maxrel(qm.E_m2n, o.field_ext(1, cqm)) < 1e-12
    assert maxrel(qm.E_p2n, o.field_ext(2, cqm)) < 1e-12
    qm.close()


def test_update_coord_resets_like_the_reference(golden_mmp):
    p = golden_mmp["1crn_amoeba"]
    g, o = OMMPSystem(p), OracleSystem(p)
    cqm, qqm, zqm = nuclei_near(o.cmm, 6, 5)
    qm = OMMPQmHelper(cqm, qqm, zqm)
    g.set_external_field(np.zeros((g.pol_atoms, 3)))
    qm.prepare_qm_ele_ene(g)
    qm.prepare_qm_ele_grd(g)
    vp = qm.V_p2n
    c2 = cqm + 0.3
    qm.update_coord(c2)
    for name in ("E_n2p", "G_n2p", "E_n2m", "G_n2m", "H_n2m", "V_m2n", "E_m2n"):
        with pytest.raises(AttributeError):
            getattr(qm, name)
    # V_p2n and E_p2n keep their flags (src/mod_qm_helper.F90:143-149)
    np.testing.assert_array_equal(qm.V_p2n, vp)
    qm.E_p2n
    qm.prepare_qm_ele_ene(g)
    assert maxrel(qm.E_n2p, o.nuclei_fields(c2, qqm)) < 1e-12
    assert maxrel(qm.V_m2n, o.potential_ext(1, c2)) < 1e-12
    np.testing.assert_array_equal(qm.V_p2n, vp)  # not recomputed, as in the reference
    qm.prepare_qm_ele_grd(g)  # recomputed at every call
    o.set_ipd(g.ipd)
    assert maxrel(qm.E_p2n, o.field_ext(2, c2)) < 1e-12


def test_qm_helper_errors(golden_mmp):
    p = golden_mmp["nma_wang"]
    g = OMMPSystem(p)
    cqm, qqm, zqm = nuclei_near(g.cmm, 3, 7)
    qm = OMMPQmHelper(cqm, qqm, zqm)
    # the induced field at the nuclei needs dipoles
    with pytest.raises(OMMPError) as e:
        qm.prepare_qm_ele_grd(g)
    assert e.value.status == 1
    # a nucleus on top of an MM site
    c = cqm.copy()
    c[0] = g.cmm[2]
    qm.update_coord(c)
    with pytest.raises(OMMPError) as e:
        qm.prepare_qm_ele_ene(g)
    assert e.value.status == 4
