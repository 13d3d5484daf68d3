"""Solves of uneven systems advanced together (ommp_gpu_solve_multi,
csrc/multisolve.cu): the pair products of all systems that need one share a
persistent multi-system launch per product kind, large products spread over
several rounds.

Checks: every system's dipoles and energy equal its own single-system solve
within the mixed-precision tolerance (1e-7 relative) and a converged oracle
for a protein; a system's result is bit-for-bit the same solved alone
through the engine and in the mix (fixed-point sums: slicing a product over
rounds does not change it); launches served two or more systems of
different size, and the large product was spread over several rounds.
"""
import numpy as np
import pytest

import openmmpol_gb300 as og
from openmmpol_gb300 import OMMPSystem, set_verbose, synth
from oracle.oracle import SOLVER_DIIS, OracleSystem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


@pytest.fixture(scope="module")
def mix(tmp_path_factory, golden_mmp):
    d = tmp_path_factory.mktemp("mix")
    paths = [golden_mmp["1crn_amoeba"], golden_mmp["1crn_wang"]]
    for nw, seed in ((300, 3), (2000, 4), (10000, 5)):
        paths.append(synth.write_mmp(str(d / f"w{nw}.mmp"), synth.water_cluster(nw, seed=seed)))
    c = synth.chain_system(n_chains=10, chain_len=40, n_waters=600, seed=2)
    paths.append(synth.write_mmp(str(d / "chains.mmp"), c))
    return paths


def _fields(systems, seed0):
    out = []
    for k, s in enumerate(systems):
        cmm = s.cmm
        out.append(synth.point_charge_field(s.cpol, cmm.mean(0) / synth.ANG2AU, seed=seed0 + k, all_sites_bohr=cmm)[0])
    return out


def _systems(paths, precision):
    out = []
    for p in paths:
        g = OMMPSystem(p)
        g.set_solver_tol(1e-10)
        g.set_precision(precision)
        out.append(g)
    return out


@pytest.mark.parametrize("precision", ["mixed", "mixed-ds"])
def test_solve_multi_matches_single_solves(mix, precision):
    systems = _systems(mix, precision)
    fields = _fields(systems, 60)
    en, st = og.solve_multi(systems, fields)
    assert st["max_systems_per_launch"] >= 2 and st["shared_launches"] >= 1
    assert st["spread_products"] >= 1  # the 30,000-site products took several rounds
    # mixed-ds updates its later refinement residuals by FP32 products
    assert any(g.counter(5) >= 1 for g in systems) == (precision == "mixed-ds")
    singles = _systems(mix, precision)
    for g, s1, f, e in zip(systems, singles, fields, en):
        s1.set_external_field(f)
        assert rel(g.ipd, s1.ipd) < 1e-7
        assert abs(e - s1.get_polelec_energy()) <= 1e-7 * abs(s1.get_polelec_energy())
        assert abs(e - g.get_polelec_energy()) <= 1e-12 * abs(e)
        assert g.residual_history(0)[-1] < 1e-10
    # the protein against a converged oracle (different D and P sets)
    o = OracleSystem(mix[0])
    o.set_tol(1e-12)
    o.set_default_solver(SOLVER_DIIS)
    o.set_external_field(fields[0])
    assert rel(systems[0].ipd, o.ipd) < 1e-7


def test_solve_multi_result_is_the_same_alone_and_in_the_mix(mix):
    systems = _systems(mix, "mixed-ds")
    fields = _fields(systems, 80)
    og.solve_multi(systems, fields)
    for k in (0, 3, 4):
        alone = _systems([mix[k]], "mixed-ds")[0]
        og.solve_multi([alone], [fields[k]])
        assert np.array_equal(alone.ipd, systems[k].ipd)


def test_solve_multi_follow_up_warm_start(mix):
    """A second round of solves starts from the resident dipoles (the
    reference's ipd_use_guess) and needs fewer refinement steps."""
    systems = _systems(mix[2:4], "mixed")
    fields = _fields(systems, 90)
    og.solve_multi(systems, fields)
    outer0 = [g.counter(2) for g in systems]
    fields2 = [f * (1.0 + 0.01 * np.random.default_rng(3).standard_normal(f.shape)) for f in fields]
    og.solve_multi(systems, fields2)
    for k, (g, f, o0) in enumerate(zip(systems, fields2, outer0)):
        ref = _systems([mix[2 + k]], "mixed")[0]
        ref.set_external_field(f)
        assert rel(g.ipd, ref.ipd) < 1e-7
        assert g.counter(2) <= o0


def test_solve_multi_residual_update_matches_recompute(mix):
    """In the engine too, updating the later refinement residuals by the
    FP32 product of the correction changes only the convergence certificate:
    the dipoles equal those of recomputed residuals, with fewer
    double-single products."""
    out = {}
    for mode in ("update", "recompute"):
        systems = _systems(mix, "mixed-ds")
        for g in systems:
            g.set_residual_update(mode)
        fields = _fields(systems, 90)
        og.solve_multi(systems, fields)
        out[mode] = systems
    for gu, gr in zip(out["update"], out["recompute"]):
        assert gr.counter(5) == 0
        assert gu.counter(4) <= gr.counter(4)
        if gu.counter(2) == gr.counter(2):
            assert rel(gu.ipd, gr.ipd) < 1e-12
        assert gu.residual_history(0)[-1] < 1e-10
    assert sum(g.counter(5) for g in out["update"]) >= 1

