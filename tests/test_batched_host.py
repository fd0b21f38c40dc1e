"""Host logic of the many-model batch: schedule buckets and stream assignment."""

import pytest

from botorch_gb300 import testing as T
from botorch_gb300.batched import SCHEDULES, assign_streams, bucket_key


def test_bucket_key_rounds_n_up_to_a_power_of_two():
    assert bucket_key(100, 6) == (128, 6)
    assert bucket_key(128, 6) == (128, 6)
    assert bucket_key(129, 6) == (256, 6)
    assert bucket_key(4000, 30) == (4096, 30)
    assert bucket_key(1, 4) == (1, 4)


def test_assign_streams_longest_first():
    costs = [5.0, 1.0, 4.0, 3.0, 3.0, 2.0]
    lanes = assign_streams(costs, 2)
    loads = [sum(costs[i] for i in lane) for lane in lanes]
    assert sorted(i for lane in lanes for i in lane) == list(range(len(costs)))
    assert max(loads) == 9.0  # 5+3+1 / 4+3+2
    assert assign_streams([1.0], 4) == [[0], [], [], []]
    with pytest.raises(ValueError):
        assign_streams([1.0], 0)


def test_schedules_cover_both_gemm_forms():
    assert any(s[0] for s in SCHEDULES) and any(not s[0] for s in SCHEDULES)


def test_many_gps_generator():
    ws = T.many_gps(16, seed=3)
    assert len(ws) == 16
    for w in ws:
        n, d = w.train_X.shape
        assert 100 <= n <= 4000 and 4 <= d <= 30
        assert w.X.shape == (256, 2, d) and w.n_samples == 256
    assert T.many_gps(2, seed=3)[0].train_X.shape == ws[0].train_X.shape
