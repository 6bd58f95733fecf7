"""The C-ABI library builds, loads and exports every entry point that
include/supermc.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

from conftest import REPO


def declared_functions():
    text = open(os.path.join(REPO, "include", "supermc.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"\b(smc_[a-z_0-9]+)\s*\(", text)


def test_library_exports_header_symbols():
    from supermc_gb300.build import build
    from supermc_gb300 import _lib
    path = build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert set(_lib.EXPORTS) == set(names)
    for n in names:
        assert hasattr(lib, n), n


def test_status_strings_without_device():
    from supermc_gb300 import _lib
    lib = _lib.load()
    for s in range(9):
        assert lib.smc_status_string(s)


def test_cuda_error_string_format():
    """smc_cuda_error_string names the pending CUDA runtime error as
    "<name>: <description>" (here, without a device, whatever the runtime
    reports), and an SMC_ERR_CUDA raised by the Python layer carries it."""
    from supermc_gb300 import _lib
    lib = _lib.load()
    text = lib.smc_cuda_error_string().decode()
    assert text.startswith("cuda") and ": " in text
    try:
        _lib.check(_lib.SMC_ERR_CUDA, "probe")
    except _lib.SmcError as e:
        assert "probe (cuda" in str(e) and e.status == _lib.SMC_ERR_CUDA
    else:
        raise AssertionError("SMC_ERR_CUDA did not raise")
