"""The oracle's QM-helper nuclear fields (electrostatic_for_ene / _grad,
src/mod_qm_helper.F90:356-520, q_elec_prop src/mod_electrostatics.F90:
1097-1176) pinned by numpy and by central finite differences: the field of
the nuclei is the point-charge formula, the reference's field gradient is
G_ab = -dE_a/dx_b and its Hessian H_abc = -dG_ab/dx_c (derivatives with
respect to the MM site's position), h = 1e-4 bohr.
"""
import numpy as np
import pytest

from oracle.oracle import OracleSystem

G6 = [(0, 0), (0, 1), (1, 1), (0, 2), (1, 2), (2, 2)]
H10 = [(0, 0, 0), (0, 0, 1), (0, 0, 2), (0, 1, 1), (0, 1, 2), (0, 2, 2), (1, 1, 1), (1, 1, 2), (1, 2, 2),
       (2, 2, 2)]


def nuclei(cmm, n, seed):
    rng = np.random.default_rng(seed)
    return cmm.mean(0) + rng.normal(scale=4.0, size=(n, 3)), rng.uniform(1.0, 8.0, n)


@pytest.mark.parametrize("case", ["1crn_wang", "nma_amoeba"])
def test_nuclear_field_matches_point_charges(case, golden_mmp):
    o = OracleSystem(golden_mmp[case])
    cqm, q = nuclei(o.cmm, 7, 1)
    d = o.cmm[o.polar_mm][:, None, :] - cqm[None]
    r = np.linalg.norm(d, axis=2)
    ref = (q[None, :, None] * d / r[..., None] ** 3).sum(1)
    assert np.abs(o.nuclei_fields(cqm, q) - ref).max() < 1e-14 * np.abs(ref).max()
    E, _, _ = o.nuclei_fields(cqm, q, grad=True)
    assert np.array_equal(E[o.polar_mm], o.nuclei_fields(cqm, q))


def test_gradient_and_hessian_are_derivatives(golden_mmp):
    o = OracleSystem(golden_mmp["1crn_wang"])
    cqm, q = nuclei(o.cmm, 5, 2)
    c0 = o.cmm.copy()
    _, G, H = o.nuclei_fields(cqm, q, grad=True)
    h = 1e-4
    for site in (0, 100, 400):
        dE, dG = np.zeros((3, 3)), np.zeros((3, 6))
        for b in range(3):
            cp, cm = c0.copy(), c0.copy()
            cp[site, b] += h
            cm[site, b] -= h
            o.update_coordinates(cp)
            Ep, Gp, _ = o.nuclei_fields(cqm, q, grad=True)
            o.update_coordinates(cm)
            Em, Gm, _ = o.nuclei_fields(cqm, q, grad=True)
            dE[:, b] = (Ep[site] - Em[site]) / (2 * h)
            dG[b] = (Gp[site] - Gm[site]) / (2 * h)
        o.update_coordinates(c0)
        g_fd = np.array([-dE[a, b] for a, b in G6])
        h_fd = np.array([-dG[c][G6.index((a, b))] for a, b, c in H10])
        assert np.abs(g_fd - G[site]).max() < 1e-7 * np.abs(G[site]).max()
        assert np.abs(h_fd - H[site]).max() < 1e-7 * np.abs(H[site]).max()
