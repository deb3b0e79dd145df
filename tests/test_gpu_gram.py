"""Level 0 on the tensor cores: pair tables from the Gram matrix of the one-hot samples.

The engine decides level 0 of a single dataset from G = H H^T (gram.cu: TMA-staged E4M3
one-hot tiles, tcgen05.mma with FP32 accumulation in TMEM, exact for counts below 2^24).
These tests hold it to the counting kernels (FPGM_GRAM=0) and to the oracle: every pair's
decision at level 0 (depth 1) at several alphas, over sample counts that are not multiples
of the 128-sample K block, row counts that are not multiples of the 128-row tile, the
split-K path (few tiles) and the one-CTA-per-tile path (many tiles).
"""
import numpy as np
import pytest

from oracle import oracle as O
import fastpgm_gb300 as F

pytestmark = pytest.mark.gpu


def _level0(raw, alpha, gram, monkeypatch):
    monkeypatch.setenv("FPGM_GRAM", "1" if gram else "0")
    e = F.Engine(0)
    monkeypatch.delenv("FPGM_GRAM")
    try:
        e.upload(raw)
        st = e.pc_skeleton(alpha=alpha, depth=1).to_dict()
        return st, e.result()
    finally:
        e.close()


@pytest.mark.parametrize("n,S,card,seed", [(12, 1, (2, 3), 1), (20, 17, (2, 5), 2), (30, 1000, (2, 9), 3),
                                           (40, 4099, (3, 12), 4), (70, 20000, (2, 21), 5), (600, 2000, (2, 10), 6)])
def test_level0_gram_equals_counting_kernels_and_oracle(monkeypatch, n, S, card, seed):
    raw, _, _ = F.generate(n_nodes=n, n_samples=S, seed=seed, avg_indegree=1.5, max_indegree=3, card=card,
                           dirichlet=0.5)
    cols, cd = O.relabel(raw)
    for alpha in (0.05, 0.5, 1e-6):
        sg, rg = _level0(raw, alpha, True, monkeypatch)
        sc, rc = _level0(raw, alpha, False, monkeypatch)
        assert sg["gram_tests"] == n * (n - 1) // 2, "level 0 did not take the tensor-core path"
        assert sc["gram_tests"] == 0
        assert np.array_equal(rg["adj"], rc["adj"])
        assert rg["sepsets"] == rc["sepsets"]
        assert sg["tests"] == sc["tests"] and sg["edges_after"] == sc["edges_after"]
        ref = O.pc_skeleton(cols, cd, alpha=alpha, depth=1, threads=8)
        assert np.array_equal(rg["adj"], ref["adj"])
        assert rg["sepsets"] == ref["sepsets"]


def test_level0_gram_on_the_c4_shape(monkeypatch):
    """1,041 variables with up to 21 states (7,000+ one-hot rows, thousands of 128x128 tiles,
    one CTA per tile) on 8,192 samples: level-0 decisions equal the counting kernels'."""
    raw, _, _ = F.make_config("c4", n_samples=8192)
    sg, rg = _level0(raw, 0.05, True, monkeypatch)
    sc, rc = _level0(raw, 0.05, False, monkeypatch)
    assert sg["gram_tests"] == 1041 * 1040 // 2
    assert np.array_equal(rg["adj"], rc["adj"])
    assert sg["gram_flops"] > 0 and sg["gram_ms"] > 0
