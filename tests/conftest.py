import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "reina-vk_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def reference_dir(sub: str = "") -> Path | None:
    """A checkout of the reference (reina-vk) named by the REINA_REFERENCE_DIR environment variable, or None
    when the variable is unset or the directory is absent; tests that read the reference's own files skip
    then."""
    env = os.environ.get("REINA_REFERENCE_DIR")
    if not env:
        return None
    p = Path(env) / sub
    return p if p.exists() else None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def R():
    """The trace-path library binding, built if needed (nvcc cross-compiles without a GPU)."""
    import build as pkg_build

    pkg_build.build()
    import reina_gb300

    reina_gb300.load_library()
    return reina_gb300


@pytest.fixture(scope="session")
def O():
    from oracle import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx(R):
    ctx = R.Context(0)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def host_ctx(R):
    ctx = R.Context(-1)
    yield ctx
    ctx.close()
