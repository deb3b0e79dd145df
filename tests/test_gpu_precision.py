"""FP32 G^2 against the FP64 oracle on the benchmark workloads (c2, c4).

The batched engine computes G^2 terms in FP32 with compensated summation and decides by
FP64 band tables; only tests inside the band around alpha are recomputed in FP64.  Here a
seeded sample of random tests per |Z| is run through the batched kernels and the oracle:
counts (df) and decisions must be identical, and the largest relative G^2 error and the
largest p-value difference of the FP32 tests are printed (pytest -s) and bounded by the
tolerance the other parity tests use (2e-5 relative G^2)."""
import numpy as np
import pytest

from oracle import oracle as O
import fastpgm_gb300 as F

pytestmark = pytest.mark.gpu

G2_RTOL, G2_ATOL = 2e-5, 2e-3


@pytest.mark.parametrize("name,ds,per_d", [("c2", (0, 1, 2, 3, 4, 5), 200), ("c4", (0, 1, 2, 4, 6, 8), 60)])
def test_fp32_g2_error_on_workloads(name, ds, per_d):
    raw, _, _ = F.make_config(name)
    cols, card = O.relabel(raw)
    n = raw.shape[0]
    rng = np.random.default_rng(2024)
    worst_rel, worst_dp, fp32_tests, rechecked = 0.0, 0.0, 0, 0
    with F.Engine(0) as eng:
        eng.upload(raw)
        for d in ds:
            tests = np.array([rng.choice(n, size=2 + d, replace=False) for _ in range(per_d)], dtype=np.int32)
            got = eng.ci_test_batch(tests, d)
            exp = O.ci_tests(cols, card, tests, d, threads=16)
            for g, o in zip(got, exp):
                assert g.df == o.df and g.independent == o.independent, (name, d, g.df, o.df)
                if g.rechecked:
                    rechecked += 1
                    assert abs(g.p_value - o.p_value) <= 1e-10
                    continue
                fp32_tests += 1
                err = abs(g.g2 - o.g2)
                assert err <= max(G2_ATOL, G2_RTOL * abs(o.g2)), (name, d, g.g2, o.g2)
                if o.g2 > 1.0:
                    worst_rel = max(worst_rel, err / o.g2)
                worst_dp = max(worst_dp, abs(g.p_value - o.p_value))
    print("\n%s: %d FP32 tests, %d rechecked in FP64: max |dG2|/G2 = %.3g, max |dp| = %.3g"
          % (name, fp32_tests, rechecked, worst_rel, worst_dp))
