import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs on the GPU box")


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from native import ORACLE_SO, Oracle
    if not ORACLE_SO.exists():
        import __graft_entry__
        __graft_entry__.build()
    return Oracle()


@pytest.fixture(scope="session")
def ref():
    from native import Ref, have_ref
    if not have_ref():
        pytest.skip("the reference build (oracle/_ref) is only present where its sources are")
    return Ref()


@pytest.fixture(scope="session")
def gtc():
    import __graft_entry__
    return __graft_entry__.load_package().gtc


@pytest.fixture(scope="session")
def ctx(gtc):
    c = gtc.Context(0)
    yield c
    c.close()
