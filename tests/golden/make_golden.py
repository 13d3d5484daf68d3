"""Regenerate the golden fixtures in tests/golden/ from the reference's own tests.

Run in a checkout that has the OpenMMPol sources next to it:

    python tests/golden/make_golden.py /path/to/OpenMMPol

For every direct-path golden case of the reference test-suite
(tests/test_list:6-18 N-methylacetamide, :29-38 1crn, :64-72 1ao6 cut,
:45-53 1ubq) it copies the ``.mmp`` input (gzip-compressed) and stores the
reference outputs in ``golden.npz``:

* ``<case>_ipd0`` / ``<case>_ipd1``: induced dipoles ``[n_ipd*pol_atoms, 3]``
  from ``IPD_0_*.ref`` (no external field) and ``IPD_1_*.ref`` (with EF_1.txt);
* ``<case>_ep0`` / ``<case>_ep1``: the ``EP`` line of ``ENE_{0,1}_*.ref``;
* ``<case>_em``: the ``EM`` line (static multipole energy; the same in both
  files, the external field does not enter it);
* ``<case>_ef1``: ``EF_1.txt`` gathered at the polarizable sites in the order of
  ``polar_mm`` (tests/test_programs/C/test_SI_potential.c:112-125 does the same
  gather), so fixtures stay small.

Tolerances are the reference's: ipd rtol 1e-6 / atol 1e-5, energy 1e-6 / 1e-6
(tests/generate_cmake_tests.py:8-9,95-100); 1ubq goldens were produced with the
fast multipole method and are compared at atol 1e-3 (tests/test_list:50-53).
"""
import gzip
import os
import sys

import numpy as np

CASES = {
    # name: (mmp, ipd pattern, ene pattern or None, EF file, atol_ipd)
    "nma_amoeba": ("N-methylacetamide/input_AMOEBA.mmp", "N-methylacetamide/IPD_%d_AMOEBA.ref",
                   "N-methylacetamide/ENE_%d_AMOEBA.ref", "N-methylacetamide/EF_1.txt", 1e-5),
    "nma_amoeba_cut": ("N-methylacetamide/input_AMOEBA_CUT.mmp",
                       "N-methylacetamide/IPD_%d_AMOEBA_CUT.ref", None,
                       "N-methylacetamide/EF_1.txt", 1e-5),
    "nma_wang": ("N-methylacetamide/input_WANG_AL.mmp", "N-methylacetamide/IPD_%d_WANG_AL.ref",
                 "N-methylacetamide/ENE_%d_WANG_AL.ref", "N-methylacetamide/EF_1.txt", 1e-5),
    "nma_wang_cut": ("N-methylacetamide/input_WANG_AL_CUT.mmp",
                     "N-methylacetamide/IPD_%d_WANG_AL_CUT.ref", None,
                     "N-methylacetamide/EF_1.txt", 1e-5),
    "1crn_amoeba": ("1crn/input_AMOEBA.mmp", "1crn/IPD_%d_AMOEBA.ref", "1crn/ENE_%d_AMOEBA.ref",
                    "1crn/EF_1.txt", 1e-5),
    "1crn_wang": ("1crn/input_WANG_AL.mmp", "1crn/IPD_%d_WANG_AL.ref", "1crn/ENE_%d_WANG_AL.ref",
                  "1crn/EF_1.txt", 1e-5),
    "1ao6cut_wang": ("1ao6/input_WANG_AL_CUT10.mmp", "1ao6/IPD_%d_WANG_AL_CUT10.ref",
                     "1ao6/ENE_%d_WANG_AL_CUT10.ref", "1ao6/EF_1.txt", 1e-5),
    "1ubq_amoeba": ("1ubq/input_AMOEBA.mmp", "1ubq/IPD_%d_AMOEBA.ref", "1ubq/ENE_%d_AMOEBA.ref",
                    "1ubq/EF_1.txt", 1e-3),
    "1ubq_wang": ("1ubq/input_WANG_AL.mmp", "1ubq/IPD_%d_WANG_AL.ref", "1ubq/ENE_%d_WANG_AL.ref",
                  "1ubq/EF_1.txt", 1e-3),
}


def read_term(path, tag):
    with open(path) as f:
        for line in f:
            if line.startswith(tag):
                return float(line.split()[-1])
    raise ValueError(f"no {tag} line in {path}")


def read_ep(path):
    return read_term(path, "EP")


def polar_mm_of(mmp_path):
    """Polarizable atoms are those with alpha > 1e-8 (mod_inputloader.F90:155-163)."""
    with open(mmp_path) as f:
        lines = f.read().split("\n")
    rev = int(lines[0].split()[0])
    hdr = 3 + 2 + (17 if rev == 3 else 15)
    mm = int(lines[hdr].split()[0])
    amoeba = int(lines[3].split()[0]) == 1
    ld = 10 if amoeba else 1
    pos = hdr + 1 + mm + 1 + mm + mm
    # multipoles: list-directed, ld values per atom
    vals_needed = ld
    for _ in range(mm):
        got = 0
        while got < vals_needed:
            got += len(lines[pos].split())
            pos += 1
    pol = np.array([float(lines[pos + i].split()[0].replace("D", "e")) for i in range(mm)])
    return np.nonzero(pol > 1e-8)[0]


def main(ref_root):
    tests = os.path.join(ref_root, "tests")
    out_dir = os.path.dirname(os.path.abspath(__file__))
    arrays = {}
    for name, (mmp, ipd, ene, ef, atol) in CASES.items():
        src = os.path.join(tests, mmp)
        dst = os.path.join(out_dir, name + ".mmp.gz")
        with open(src, "rb") as f:
            data = f.read()
        if not os.path.exists(dst) or gzip.open(dst).read() != data:  # keep unchanged fixtures
            with gzip.GzipFile(dst, "wb", 9, mtime=0) as g:
                g.write(data)
        pm = polar_mm_of(src)
        efm = np.loadtxt(os.path.join(tests, ef)).reshape(-1, 3)
        arrays[name + "_ef1"] = efm[pm]
        for k in (0, 1):
            arrays[f"{name}_ipd{k}"] = np.loadtxt(os.path.join(tests, ipd % k)).reshape(-1, 3)
            if ene:
                arrays[f"{name}_ep{k}"] = np.array(read_ep(os.path.join(tests, ene % k)))
        if ene:
            arrays[name + "_em"] = np.array(read_term(os.path.join(tests, ene % 0), "EM"))
        arrays[name + "_atol"] = np.array(atol)
    np.savez_compressed(os.path.join(out_dir, "golden.npz"), **arrays)
    print("wrote", len(CASES), "cases to", out_dir)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
