import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libkura.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build_oracle, kora
    if not os.path.exists(os.path.join(kora.BUILD, "libkora.so")) or not os.path.exists(kora.cli_path(True)):
        build_oracle.build()
    return kora


@pytest.fixture(scope="session")
def native():
    import kuramoto_gb300 as kg
    if not os.path.exists(kg.lib_path()) or not os.path.exists(kg.cli_path()):
        from kuramoto_gb300 import build
        build.build()
    kg.lib()
    return kg
