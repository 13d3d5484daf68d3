"""ommp_gpu_tmatvec_noalloc: the allocation-free T.mu entry point.

Hosts that own all GPU memory (a QM program's SCF loop with its own memory
pool, an MD engine whose step must not stall) cannot let the library call
cudaMalloc while they run, because allocation synchronises the device and may
fail mid-run.  This entry point takes caller-owned device buffers and keeps
its scratch in a static device array.  The test calls it through the C ABI
twice in a row on different inputs and checks each result against the
regular entry point ommp_gpu_tmatvec, at the relative tolerance the other
T.mu tests use (1e-12).  It lives in its own file, collected last, and works
both alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from openmmpol_gb300 import OMMPSystem, _lib, set_verbose, synth

pytestmark = pytest.mark.gpu


def _dev_buffer(L, nbytes):
    p = C.c_void_p()
    assert L.ommp_gpu_device_alloc(nbytes, C.byref(p)) == 0
    return p


@pytest.mark.parametrize("case,nrhs,dodiag", [("1crn_wang", 1, 1), ("1ubq_amoeba", 2, 1), ("1crn_amoeba", 1, 0),
                                              ("w900", 1, 1), ("w900", 2, 0)])
def test_noalloc_tmatvec_matches_regular_entry_point(case, nrhs, dodiag, golden_mmp, tmp_path):
    # w900: 2,700 sites, the symmetric product with its fixed-point sums in
    # the static scratch
    set_verbose(0)
    L = _lib.load()
    if case == "w900":
        s = OMMPSystem(synth.write_mmp(str(tmp_path / "w900.mmp"), synth.water_cluster(900, seed=8)))
    else:
        s = OMMPSystem(golden_mmp[case])
    n = s.pol_atoms
    nbytes = nrhs * n * 3 * 8
    xd, yd = _dev_buffer(L, nbytes), _dev_buffer(L, nbytes)
    try:
        for call in range(2):  # two calls in a row share (and reuse) the static scratch
            x = np.random.default_rng(100 + call).standard_normal((nrhs, n, 3))
            assert L.ommp_gpu_copy_to_device(xd, x.ctypes.data, nbytes) == 0
            st = L.ommp_gpu_tmatvec_noalloc(s._h, xd, yd, nrhs, dodiag)
            assert st == 0, L.ommp_gpu_last_error()
            y = np.empty_like(x)
            assert L.ommp_gpu_copy_to_host(y.ctypes.data, yd, nbytes) == 0
            ref = s.tmatvec(x if nrhs > 1 else x[0], dodiag=bool(dodiag)).reshape(nrhs, n, 3)
            assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)
    finally:
        L.ommp_gpu_device_free(xd)
        L.ommp_gpu_device_free(yd)


def test_noalloc_rejects_bad_column_count(golden_mmp):
    L = _lib.load()
    s = OMMPSystem(golden_mmp["nma_wang"])
    xd = _dev_buffer(L, 8 * 3 * s.pol_atoms * 3)
    try:
        assert L.ommp_gpu_tmatvec_noalloc(s._h, xd, xd, 3, 1) == 3
        assert b"nrhs" in L.ommp_gpu_last_error()
    finally:
        L.ommp_gpu_device_free(xd)
