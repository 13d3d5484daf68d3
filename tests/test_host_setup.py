"""Host setup of the GPU library (its own .mmp reader, BFS connectivity,
screening scales, multipole rotation) against the oracle, on CPU.

The library's setup code is compiled here with a host-only driver
(tests/host/dump_setup.cpp); no CUDA call is made."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT
from openmmpol_gb300 import synth
from oracle.oracle import OracleSystem


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("host") / "dump_setup")
    cuda_inc = "/usr/local/cuda/include"
    subprocess.run(["g++", "-O1", "-std=c++17", "-pthread", "-I", cuda_inc, "-o", exe,
                    os.path.join(ROOT, "tests", "host", "dump_setup.cpp"),
                    os.path.join(ROOT, "openmmpol_gb300", "csrc", "setup.cpp")], check=True)
    return exe


def parse(out):
    M, U, Q, P = {}, {}, {}, {}
    for line in out.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "M":
            M[(int(t[1]), int(t[2]))] = (float(t[3]), float(t[4]))
        elif t[0] == "U":
            U[(int(t[1]), int(t[2]))] = float(t[3])
        elif t[0] == "Q":
            Q[int(t[1])] = [float(x) for x in t[2:]]
        elif t[0] == "P":
            P[int(t[1])] = (int(t[2]), float(t[3]), float(t[4]))
    return M, U, Q, P


def oracle_pairs(o):
    pm = o.polar_mm
    ref = {}
    for which in ((0, 1) if o.is_amoeba else (0,)):
        ri, ci, sc = o.screening(which)
        for i in range(o.mm_atoms):
            for k in range(ri[i], ri[i + 1]):
                jp = int(ci[k])
                if pm[jp] == i:
                    continue
                d = ref.setdefault((jp, i), [1.0, 1.0])
                d[which] = sc[k]
                if not o.is_amoeba:
                    d[1] = sc[k]
    uref = {}
    ri, ci, sc = o.screening(2)
    for i in range(o.pol_atoms):
        for k in range(ri[i], ri[i + 1]):
            uref[(int(ci[k]), i)] = sc[k]  # target-major: (target, source)
    return ref, uref


def systems(golden_mmp, tmp_path):
    out = dict(golden_mmp)
    out["water"] = synth.write_mmp(str(tmp_path / "w.mmp"), synth.water_cluster(60, seed=3))
    out["chains"] = synth.write_mmp(str(tmp_path / "c.mmp"),
                                    synth.chain_system(n_chains=3, chain_len=25, n_waters=120, seed=4))
    return out


@pytest.mark.parametrize("case", GOLDEN_CASES + ["water", "chains"])
def test_host_setup_matches_oracle(case, harness, golden_mmp, tmp_path):
    path = systems(golden_mmp, tmp_path)[case]
    r = subprocess.run([harness, path], capture_output=True, text=True, check=True)
    M, U, Q, P = parse(r.stdout)
    o = OracleSystem(path)
    ref, uref = oracle_pairs(o)
    assert set(M) == set(ref)
    for k, v in ref.items():
        assert M[k] == pytest.approx(tuple(v), abs=1e-15)
    assert set(U) == set(uref)
    for k, v in uref.items():
        assert U[k] == pytest.approx(v, abs=1e-15)
    q = np.array([Q[i] for i in range(o.mm_atoms)])
    np.testing.assert_allclose(q, o.q, rtol=0, atol=1e-13)
    pm = np.array([P[k][0] for k in range(o.pol_atoms)])
    np.testing.assert_array_equal(pm, o.polar_mm)
    np.testing.assert_allclose([P[k][1] for k in range(o.pol_atoms)], o.pol, rtol=1e-15)
    np.testing.assert_allclose([P[k][2] for k in range(o.pol_atoms)], o.thole[o.polar_mm], rtol=1e-14)


def test_host_reader_rejects_bad_revision(harness, tmp_path):
    p = tmp_path / "bad.mmp"
    p.write_text("7\n")
    r = subprocess.run([harness, str(p)], capture_output=True, text=True)
    assert r.returncode == 1 and "version 2 or 3" in r.stdout


def test_host_reader_list_directed_forms(harness, tmp_path):
    # the same system written with list-directed variations: a record split
    # over two lines, commas, D exponents, r*c repeat counts, extra values
    # after a read; the reader takes its general (sequential) path for these
    # and must give exactly what the plain file gives
    w = synth.water_cluster(40, seed=9)
    plain = synth.write_mmp(str(tmp_path / "plain.mmp"), w)
    lines = open(plain).read().split("\n")
    mm = int(lines[22])
    base = 24 + mm  # first coordinate record
    c, mp, pol, conn, grp = base, base + 2 * mm, base + 3 * mm, base + 4 * mm, base + 5 * mm
    x, y, z = lines[c + 5].split()
    lines[c + 5] = x + " " + y
    lines.insert(c + 6, "  " + z)  # atom 5 continues on the next record
    off = 1
    lines[c + 7 + off - 1] = ", ".join(lines[c + 7 + off - 1].split())
    q = [float(v) for v in lines[mp + 3 + off].split()]
    lines[mp + 3 + off] = " ".join(("%.17E" % v).replace("E", "D") for v in q)
    lines[pol + 2 + off] = lines[pol + 2 + off] + " 9.9 trailing"
    t = lines[conn + 7 + off].split()
    nz = [v for v in t if v != "0"]
    lines[conn + 7 + off] = " ".join(nz + ["%d*0" % (len(t) - len(nz))])
    t = lines[grp + 4 + off].split()
    nz = [v for v in t if v != "0"]
    lines[grp + 4 + off] = " ".join(nz + ["%d*0" % (len(t) - len(nz))])
    varied = tmp_path / "varied.mmp"
    varied.write_text("\n".join(lines))
    a = subprocess.run([harness, plain], capture_output=True, text=True, check=True).stdout
    b = subprocess.run([harness, str(varied)], capture_output=True, text=True, check=True).stdout
    assert a == b
