import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hydrocode-fusion_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    """The oracle's C restatement (built on demand; test infrastructure only)."""
    import oracle as orc

    if not os.path.exists(orc.PORT_SO):
        orc.build()
    return orc.Oracle("port")


@pytest.fixture(scope="session")
def ref():
    """The reference compiled from its own sources, where the reference tree exists."""
    import oracle as orc

    if not os.path.exists(orc.REF_SO):
        if not orc.reference_available():
            pytest.skip("reference tree not given (set HYDRO_REFERENCE)")
        orc.build(ref=True)
    return orc.Oracle("reference")


@pytest.fixture(scope="session")
def ref_g2d():
    """The reference built with GRP_2D_flux calling its genuinely-2D solver
    (oracle/Makefile), where the reference tree exists."""
    import oracle as orc

    if not os.path.exists(orc.REF_G2D_SO):
        if not orc.reference_available():
            pytest.skip("reference tree not given (set HYDRO_REFERENCE)")
        orc.build(ref=True)
    return orc.Oracle("reference_g2d")


@pytest.fixture(scope="session")
def ref_mf():
    """GRP_2D_flux of the reference's two-component build (MULTIFLUID_BASICS),
    where the reference tree exists."""
    import oracle as orc

    if not os.path.exists(orc.REF_MF_SO):
        if not orc.reference_available():
            pytest.skip("reference tree not given (set HYDRO_REFERENCE)")
        orc.build(ref=True)
    return orc.Oracle("reference_mf")


@pytest.fixture(scope="session")
def gpu_lib():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hydro_gb300 as hg

    if not os.path.exists(hg.LIB_PATH):
        hg.build()
    hg.lib()
    return hg
