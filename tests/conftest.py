import os
import platform
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "oracle"))

ORACLE_SO = ROOT / "oracle" / "_build" / "libpfref.so"
REF_SHIM_SO = ROOT / "oracle" / "_ref" / "libpf_shim.so"
REF_ASIS_SO = ROOT / "oracle" / "_ref" / "libpf_asis.so"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    from pixelforge_gb300.abi import PixelForgeLib
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "pfref"], check=True)
    return PixelForgeLib(str(ORACLE_SO))


@pytest.fixture(scope="session")
def ref_shim():
    """The reference compiled from its own sources with exact rcp/rsqrt.

    Only on x86-64 with the reference sources present (``PF_REFERENCE_SRC``;
    they include <immintrin.h> unconditionally); skipped elsewhere."""
    from pixelforge_gb300.abi import PixelForgeLib
    if not REF_SHIM_SO.exists() and platform.machine() in ("x86_64", "AMD64"):
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref-if-present"], check=True)
    if not REF_SHIM_SO.exists():
        pytest.skip("reference build unavailable on this host")
    return PixelForgeLib(str(REF_SHIM_SO))


@pytest.fixture(scope="session")
def gpu():
    from pixelforge_gb300 import load_library
    return load_library()
