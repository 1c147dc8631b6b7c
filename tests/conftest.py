import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgfe")
    # the oracle is test infrastructure: build it for the suite
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def gg():
    import __graft_entry__ as ge
    lib = ROOT / "gridap.jl_gb300" / "_build" / "libgfe.so"
    if not lib.exists():
        ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def kats():
    import json
    return json.loads((ROOT / "tests" / "golden" / "gridap_kats.json").read_text())
