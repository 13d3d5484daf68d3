"""ommp_gpu_tmatvec_noalloc: the allocation-free T.mu entry point.

Hosts that own all GPU memory (a QM program's SCF loop with its own memory
pool, an MD engine whose step must not stall) cannot let the library call
cudaMalloc while they run, because allocation synchronises the device and may
fail mid-run.  This entry point takes caller-owned device buffers and keeps
its scratch in a static device array.  The tests call it through the C ABI
twice in a row on different inputs and check each result against the
regular entry point ommp_gpu_tmatvec, at the relative tolerance the other
T.mu tests use (1e-12); check that the device's free memory does not change
across a call; and check the rejections (too many columns, a system too
large for the static scratch, overlapping x and y).  The file is collected
last and works both alone in a fresh process and after the other tests.
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


def _free_bytes(L):
    f, t = C.c_int64(), C.c_int64()
    assert L.ommp_gpu_device_mem_info(C.byref(f), C.byref(t)) == 0
    return f.value


@pytest.mark.parametrize("case,nrhs,dodiag", [("1crn_wang", 1, 1), ("1ubq_amoeba", 2, 1), ("1crn_amoeba", 1, 0),
                                              ("w900", 1, 1), ("w900", 2, 0), ("w40000", 2, 1)])
def test_noalloc_tmatvec_matches_regular_entry_point(case, nrhs, dodiag, golden_mmp, tmp_path):
    # w900: 2,700 sites, the symmetric product with its fixed-point sums in
    # the static scratch.  w40000: 120,000 sites, where two columns of
    # fixed-point sums (2,160,002 doubles) no longer fit, so the target-outer
    # kernel runs with its split partials in the static scratch instead.
    set_verbose(0)
    L = _lib.load()
    if case.startswith("w"):
        nmol = int(case[1:])
        s = OMMPSystem(synth.write_mmp(str(tmp_path / f"{case}.mmp"), synth.water_cluster(nmol, seed=8)))
    else:
        s = OMMPSystem(golden_mmp[case])
    n = s.pol_atoms
    nbytes = nrhs * n * 3 * 8
    xd, yd = _dev_buffer(L, nbytes), _dev_buffer(L, nbytes)
    try:
        for call in range(2):  # two calls in a row share (and reuse) the static scratch
            x = np.random.default_rng(100 + call).standard_normal((nrhs, n, 3))
            assert L.ommp_gpu_copy_to_device(xd, x.ctypes.data, nbytes) == 0
            free0 = _free_bytes(L)
            st = L.ommp_gpu_tmatvec_noalloc(s._h, xd, yd, nrhs, dodiag)
            assert st == 0, L.ommp_gpu_last_error()
            if call == 1:  # from the second call on, no module load either
                assert _free_bytes(L) == free0
            y = np.empty_like(x)
            assert L.ommp_gpu_copy_to_host(y.ctypes.data, yd, nbytes) == 0
            ref = s.tmatvec(x if nrhs > 1 else x[0], dodiag=bool(dodiag)).reshape(nrhs, n, 3)
            assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)
    finally:
        L.ommp_gpu_device_free(xd)
        L.ommp_gpu_device_free(yd)


def test_noalloc_rejects_bad_column_count_and_overlap(golden_mmp):
    L = _lib.load()
    s = OMMPSystem(golden_mmp["nma_wang"])
    n = s.pol_atoms
    xd = _dev_buffer(L, 8 * 3 * n * 3)
    try:
        assert L.ommp_gpu_tmatvec_noalloc(s._h, xd, xd, 3, 1) == 3
        assert b"nrhs" in L.ommp_gpu_last_error()
        # y starting inside x (and x inside y): no in-place product
        base = xd.value
        assert L.ommp_gpu_tmatvec_noalloc(s._h, C.c_void_p(base), C.c_void_p(base), 1, 1) == 3
        assert b"overlap" in L.ommp_gpu_last_error()
        assert L.ommp_gpu_tmatvec_noalloc(s._h, C.c_void_p(base), C.c_void_p(base + 8 * 3 * (n - 1)), 1, 1) == 3
        assert L.ommp_gpu_tmatvec_noalloc(s._h, C.c_void_p(base + 8 * 3 * (n - 1)), C.c_void_p(base), 1, 1) == 3
        # adjacent, disjoint ranges are accepted
        assert L.ommp_gpu_tmatvec_noalloc(s._h, C.c_void_p(base), C.c_void_p(base + 8 * 3 * n), 1, 1) == 0
    finally:
        L.ommp_gpu_device_free(xd)


def test_noalloc_rejects_system_beyond_static_scratch(tmp_path):
    # 351,000 sites x 2 columns need 2,106,000 doubles of partials even with
    # one source split: more than the 16 MiB (2,097,152 doubles) scratch
    set_verbose(0)
    L = _lib.load()
    s = OMMPSystem(synth.write_mmp(str(tmp_path / "w117k.mmp"), synth.water_cluster(117000, seed=9)))
    n = s.pol_atoms
    assert n == 351000
    xd, yd = _dev_buffer(L, 8 * 2 * n * 3), _dev_buffer(L, 8 * 2 * n * 3)
    try:
        assert L.ommp_gpu_tmatvec_noalloc(s._h, xd, yd, 2, 1) == 3
        msg = L.ommp_gpu_last_error()
        assert b"exceed the 16 MiB static scratch" in msg and b"349525" in msg
    finally:
        L.ommp_gpu_device_free(xd)
        L.ommp_gpu_device_free(yd)
