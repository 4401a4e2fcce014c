"""Host-side checks of the uneven-batch workload definition (no GPU)."""
import math

import numpy as np

from muxi_spmv_gb300 import batch as B
from muxi_spmv_gb300 import api


def test_uneven_specs_follow_the_workload_laws():
    specs = B.uneven_specs(1024, seed=0)
    assert len(specs) == 1024
    rows = np.array([s.spec.numRows for s in specs])
    assert rows.min() >= 1024 and rows.max() <= 262144
    # log-uniform rows: the mean of log(rows) sits mid-way between the bounds
    mid = 0.5 * (math.log(1024) + math.log(262144))
    assert abs(np.log(rows).mean() - mid) < 0.15
    means = np.array([s.mean_target for s in specs])
    assert means.min() >= 2.0 and means.max() <= 64.0
    laws = [s.law for s in specs]
    assert 400 < laws.count("zipf") < 624
    for s in specs:
        assert s.spec.numCols == s.spec.numRows
        if s.law == "zipf":
            assert s.spec.kind == api.GEN_ZIPF_UNIFORM and s.spec.p0 == 2.0
        else:
            assert s.spec.kind == api.GEN_POISSON_UNIFORM and s.spec.p0 == s.mean_target
    # seeded: same seed, same specs; another seed, other specs
    again = B.uneven_specs(1024, seed=0)
    assert all(a.spec == b.spec for a, b in zip(specs, again))
    assert any(a.spec != b.spec for a, b in zip(specs, B.uneven_specs(1024, seed=1)))


def test_zipf_batch_lengths_reach_the_target_mean():
    """Zipf(2.0) lengths truncated at the clip plus the per-row offset have
    the target mean (host generator, small rows)."""
    import muxi_spmv_gb300 as mx
    for s in B.uneven_specs(64, seed=5):
        if s.law != "zipf" or s.spec.numRows > 20000:
            continue
        rp, _, _ = mx.generate(s.spec)
        mean = rp[-1] / s.spec.numRows
        assert abs(mean - s.mean_target) < 0.1 * s.mean_target + 0.6, (s.spec, mean)
