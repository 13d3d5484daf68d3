"""The near-field couplings of the inner preconditioner's Neumann step
(build_near_field, openmmpol_gb300/csrc/precond.cpp), built on the host by a
CPU harness (tests/host/dump_near.cpp; no CUDA call): every pair of sites in
different runs of the block preconditioner within the cutoff is listed once
per row and no other, and the 3x3 blocks are symmetric (N_ij = N_ji^T), so
the preconditioner B^-1 - B^-1 N B^-1 is symmetric."""
import os
import subprocess

import numpy as np
import pytest

from openmmpol_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("host") / "dump_near")
    subprocess.run(["g++", "-O1", "-std=c++17", "-pthread", "-I", "/usr/local/cuda/include", "-o", exe,
                    os.path.join(ROOT, "tests", "host", "dump_near.cpp"),
                    os.path.join(ROOT, "openmmpol_gb300", "csrc", "setup.cpp"),
                    os.path.join(ROOT, "openmmpol_gb300", "csrc", "precond.cpp")], check=True)
    return exe


def run(exe, path):
    out = subprocess.run([exe, path], check=True, capture_output=True, text=True).stdout
    sites, edges, zero, rc = {}, {}, set(), None
    for line in out.splitlines():
        t = line.split()
        if t[0] == "N":
            rc = float(t[2])
        elif t[0] == "S":
            sites[int(t[1])] = (int(t[2]), np.array([float(v) for v in t[3:6]]))
        elif t[0] == "Z":
            zero.add((int(t[1]), int(t[2])))
        elif t[0] == "E":
            edges[(int(t[1]), int(t[2]))] = np.array([float(v) for v in t[3:12]]).reshape(3, 3)
    return rc, sites, edges, zero


@pytest.mark.parametrize("case", ["water", "1crn_amoeba", "1crn_wang"])
def test_near_field_pairs_and_symmetry(case, harness, golden_mmp, tmp_path):
    if case == "water":
        path = synth.write_mmp(str(tmp_path / "w.mmp"), synth.water_cluster(300, seed=5))
    else:
        path = golden_mmp[case]
    rc, sites, edges, zero = run(harness, path)
    n = len(sites)
    run_id = np.array([sites[j][0] for j in range(n)])
    x = np.stack([sites[j][1] for j in range(n)])
    d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    want = (d2 < rc * rc) & (run_id[:, None] != run_id[None, :])
    got = np.zeros_like(want)
    for (j, i) in edges:
        got[j, i] = True
    # every listed pair is a cross-run pair within the cutoff; the listed set
    # is the brute-force set less the pairs whose D2D scale factor is zero
    # (Wang-AL exclusions of bonded neighbours in different runs)
    assert not (got & ~want).any()
    missing = want & ~got
    assert {(int(j), int(i)) for j, i in zip(*np.nonzero(missing))} <= zero
    assert not any(got[j, i] for (j, i) in zero)
    assert (got == got.T).all()
    for (j, i), b in edges.items():
        np.testing.assert_allclose(b, edges[(i, j)].T, rtol=1e-6, atol=1e-9)
        np.testing.assert_allclose(b, b.T, rtol=1e-6, atol=1e-9)
    if case == "water":
        assert not missing.any()  # water: no scaled inter-molecular pairs
        assert 5 < len(edges) / n < 30
