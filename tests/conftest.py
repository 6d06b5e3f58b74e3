"""Test configuration: the gpu marker, import paths, and session builds.

CPU tests (-m "not gpu") check the oracle against the golden vectors made from the
reference's own code, the host-side logic, and that libvrt.so loads and exports every
symbol include/vrt.h declares.  GPU tests (-m gpu) compare the CUDA path, called
through the C ABI, with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("voxel-rt_gb300", "oracle", "tests"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libvrt.so and the oracle once per session (quick when up to date)."""
    import build as vbuild
    import vrt_oracle
    vbuild.build()
    vrt_oracle.build()


@pytest.fixture(scope="session")
def vrt_lib():
    import build as vbuild
    import vrt
    vbuild.build()
    vrt.lib()
    return vrt


@pytest.fixture(scope="session")
def oracle():
    import vrt_oracle
    vrt_oracle.build()
    return vrt_oracle


@pytest.fixture(scope="session")
def cuda(vrt_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
