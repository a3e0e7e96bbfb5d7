"""Host logic of the continuous-batching server (no GPU): the admission rule and its sizing."""
from wbgpu.serve import admit, request_bytes


def test_admit_fifo_prefix_within_budget():
    assert admit([10, 10, 10], used_bytes=0, budget_bytes=25, free_slots=4) == 2
    assert admit([10, 30, 1], used_bytes=0, budget_bytes=35, free_slots=4) == 1  # no overtaking
    assert admit([10, 10, 10], used_bytes=0, budget_bytes=100, free_slots=2) == 2  # slots bound
    assert admit([5], used_bytes=20, budget_bytes=22, free_slots=3) == 0
    assert admit([], used_bytes=0, budget_bytes=10, free_slots=3) == 0


def test_admit_oversize_request_runs_alone():
    assert admit([50, 1], used_bytes=0, budget_bytes=10, free_slots=4) == 1
    assert admit([50], used_bytes=1, budget_bytes=10, free_slots=4) == 0


def test_request_bytes_scale():
    a = request_bytes(32, 13824, 1, {'V', 'A', 'Od'}, 'mixed')
    assert request_bytes(32, 13824, 2, {'V', 'A', 'Od'}, 'mixed') == 2 * a
    assert request_bytes(32, 13824, 1, {'V', 'A', 'Od'}, 'fp64') > a
    assert request_bytes(64, 13824, 1, {'V', 'A', 'Od'}, 'mixed') > 3 * a
