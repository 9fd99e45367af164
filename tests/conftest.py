import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def pkg():
    entry.build()
    return entry.load_package()


@pytest.fixture(scope="session")
def stq(pkg):
    return pkg.stq


@pytest.fixture(scope="session")
def oracle(pkg):
    return entry.load_oracle()


@pytest.fixture(scope="session")
def kat():
    return json.loads((GOLDEN / "kat.json").read_text())


@pytest.fixture(scope="session")
def cloth_fixture():
    return dict(np.load(GOLDEN / "cloth_g12.npz"))


def decode_boxes(entries, dtype):
    """KAT boxes (float bit patterns) -> structured array of the 44-byte layout."""
    out = np.zeros(len(entries), dtype)
    for i, b in enumerate(entries):
        out[i]["id"] = b["id"]
        out[i]["min"] = np.array(b["min"], np.uint32).view(np.float32)
        out[i]["max"] = np.array(b["max"], np.uint32).view(np.float32)
        out[i]["vertex_ids"] = b["vertex_ids"]
        out[i]["ref_id"] = b["ref_id"]
    return out


def decode_mesh(m):
    V0 = np.array([[float.fromhex(x) for x in r] for r in m["V0"]], np.float64)
    V1 = np.array([[float.fromhex(x) for x in r] for r in m["V1"]], np.float64)
    E = np.array(m["E"], np.int32).reshape(-1, 2)
    F = np.array(m["F"], np.int32).reshape(-1, 3)
    return V0, V1, E, F


def expected_pairs(lst):
    return np.array(lst, np.int32).reshape(-1, 2)


@pytest.fixture(scope="session")
def cuda():
    import torch

    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return torch.device("cuda:0")


@pytest.fixture()
def ctx(stq, cuda):
    import torch

    c = stq.Context(0, torch.cuda.current_stream(cuda).cuda_stream)
    yield c
    c.close()
