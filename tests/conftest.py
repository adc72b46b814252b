import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


def load_golden(name):
    with np.load(GOLDEN / f"{name}.npz", allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def golden_cases(name):
    """Split a stage archive into per-case dicts: {name, inputs{...}, outputs{...}}."""
    g = load_golden(name)
    cases = []
    for i in range(int(g["count"])):
        p = f"c{i}_"
        case = {"name": str(g[p + "name"]), "in": {}, "out": {}}
        for k, v in g.items():
            if not k.startswith(p) or k == p + "name":
                continue
            key = k[len(p):]
            if key.startswith("in_"):
                case["in"][key[3:]] = v
            else:
                case["out"][key] = v
        cases.append(case)
    return cases


@pytest.fixture(scope="session")
def oracle_backend():
    from oracle import oracle
    return oracle.OracleBackend()
