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


def tiny_table_cases():
    """Known-answer CI tests on hand-built tables, G^2 and p in closed form:
    (name, raw [n_vars, S] uint8 with columns x, y, z..., d, G^2, df, p).
    G^2 = 2 sum O ln(O / E) per stratum; p = erfc(sqrt(G^2 / 2)) at df 1, exp(-G^2 / 2) at
    df 2, 1 at df 0 (the reference calls a test with df 0 independent)."""
    import math

    def data(rows):  # rows of (count, x, y, z...)
        cols = [[] for _ in range(len(rows[0]) - 1)]
        for c, *vals in rows:
            for j, v in enumerate(vals):
                cols[j] += [v] * c
        return np.array(cols, dtype=np.uint8)

    cases = []
    g2 = 4 * (3 * math.log(1.5) + math.log(0.5))  # 2x2 [[3,1],[1,3]], E = 2
    cases.append(("2x2", data([(3, 0, 0), (1, 0, 1), (1, 1, 0), (3, 1, 1)]), 0, g2, 1, math.erfc(math.sqrt(g2 / 2))))
    g2 = 32 * math.log(2)  # 2x2 [[8,0],[0,8]]: dependent
    cases.append(("2x2 dependent", data([(8, 0, 0), (8, 1, 1)]), 0, g2, 1, math.erfc(math.sqrt(g2 / 2))))
    g2 = 20 * math.log(5 / 3) - 4 * math.log(3)  # 3x2 [[5,1],[1,5],[3,3]], E = 3
    cases.append(("3x2", data([(5, 0, 0), (1, 0, 1), (1, 1, 0), (5, 1, 1), (3, 2, 0), (3, 2, 1)]), 0, g2, 2,
                  math.exp(-g2 / 2)))
    g2 = 8 * math.log(2)  # z=0: [[2,0],[0,2]] (df 1, G^2 8 ln 2); z=1: [[1,1],[1,1]] (df 1, G^2 0)
    cases.append(("2x2|z", data([(2, 0, 0, 0), (2, 1, 1, 0), (1, 0, 0, 1), (1, 0, 1, 1), (1, 1, 0, 1),
                                 (1, 1, 1, 1)]), 1, g2, 2, math.exp(-g2 / 2)))
    # x constant within each stratum: every stratum has one nonzero row, df 0
    cases.append(("df 0", data([(3, 0, 0, 0), (2, 0, 1, 0), (2, 1, 0, 1), (4, 1, 1, 1)]), 1, 0.0, 0, 1.0))
    return cases
