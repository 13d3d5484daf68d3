"""CPU-side checks of the C-ABI library: it builds, loads, and exports every
symbol declared in include/openmmpol_gb300.h (no compute calls without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "openmmpol_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(ommp_[A-Za-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib_path():
    from openmmpol_gb300 import build
    return build.build()


def test_header_declares_reference_subset():
    names = declared_functions()
    for must in ["ommp_init_mmp", "ommp_set_external_field", "ommp_set_external_field_nomm",
                 "ommp_get_ipd", "ommp_get_polelec_energy", "ommp_set_default_solver",
                 "ommp_set_default_matv", "ommp_terminate", "ommp_get_pol_atoms",
                 "ommp_update_coordinates"]:
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(lib_path):
    from openmmpol_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)
    _lib.load(lib_path)


def test_library_targets_sm103a(lib_path):
    # the fatbin carries sm_103a code: the ELF holds the arch string
    data = open(lib_path, "rb").read()
    assert b"sm_103a" in data or b"sm_103" in data


def test_missing_library_fails_loudly(tmp_path):
    from openmmpol_gb300 import _lib
    with pytest.raises(_lib.LibraryMissing):
        # a fresh loader state pointed at a path that does not exist
        saved = _lib._lib
        _lib._lib = None
        try:
            _lib.load(str(tmp_path / "nope.so"))
        finally:
            _lib._lib = saved


def test_server_host_admission_without_gpu(lib_path, tmp_path, golden_mmp):
    """Server bookkeeping that needs no device: argument checks, a file that
    does not parse, and a system larger than the whole budget are refused
    (host setup only; nothing is allocated on a device)."""
    from openmmpol_gb300 import OMMPError, Server, _lib
    _lib.load(lib_path)
    with pytest.raises(OMMPError):
        Server(0, slots=1)
    with pytest.raises(OMMPError):
        Server(1 << 20, slots=0)
    srv = Server(4096, slots=2, precision="mixed")
    with pytest.raises(OMMPError, match="mmp|open|read"):
        srv.wait(srv.submit(str(tmp_path / "missing.mmp"), [[0.0, 0.0, 0.0]], 1))
    import numpy as np
    with pytest.raises(OMMPError, match="budget"):
        srv.wait(srv.submit(golden_mmp["nma_amoeba"], np.zeros((18, 3)), 2))
    assert not srv.cancel(12345)  # unknown request
    st = srv.stats()
    srv.close()
    assert st["completed"] == 2 and st["resident"] == 0 and st["bytes_in_use"] == 0
