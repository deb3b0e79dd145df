import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine's kernels")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the engine library and the CPU oracle once per session."""
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def alarm():
    z = np.load(os.path.join(GOLDEN, "alarm_s5000.npz"))
    return [str(s) for s in z["names"]], z["cols"], z["card"]


def read_sepsets(path):
    from oracle import oracle as O
    return O.read_sepsets(path)


def read_tests(path):
    """Golden per-test vectors: list of (x, y, z tuple, hash, df, g2, p, indep)."""
    out = []
    with open(path) as f:
        for line in f:
            a, b = line.split("|")
            t = [int(v) for v in a.split()]
            x, y, d = t[0], t[1], t[2]
            z = tuple(t[3:3 + d])
            h, df, g2, p, ind = b.split()
            out.append((x, y, z, int(h, 16), int(df), float(g2), float(p), int(ind)))
    return out


def sepset_arrays(seps):
    keys = sorted(seps)
    removed = np.array(keys, dtype=np.int32).reshape(-1, 2)
    off = np.zeros(len(keys) + 1, dtype=np.int32)
    vs = []
    for k, key in enumerate(keys):
        vs += list(seps[key])
        off[k + 1] = len(vs)
    return removed, off, np.array(vs, dtype=np.int32)
