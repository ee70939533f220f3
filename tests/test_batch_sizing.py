"""Arena sizing from a device-memory budget (pihm_batch_arena_bytes,
pihm_batch_limits_for_memory): host arithmetic over pihm_batch_create's own
allocation list, no device needed."""
import os

import pytest


@pytest.fixture(scope="module")
def B():
    from pihm_gpu import capi
    if not os.path.exists(capi.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    from pihm_gpu import batch
    return batch


def _lim(B, ne):
    lim = B.BatchLimits()
    lim.max_elem, lim.max_river, lim.max_edge, lim.max_record, lim.max_systems = ne, ne // 30 + 1, int(1.6 * ne) + 16, 100, 64
    return lim


def test_arena_bytes_grow_with_capacity(B):
    a, b = B.arena_bytes(_lim(B, 1_000_000)), B.arena_bytes(_lim(B, 2_000_000))
    per = (b - a) / 1_000_000
    # 24 state-vector slots of 3 values per element plus mesh, edge and scratch planes
    assert 24 * 3 * 8 < per < 4096, per
    assert a > 0


def test_limits_for_memory_is_the_largest_that_fits(B):
    budget = 3 * 1024 ** 3
    lim = B.limits_for_memory(budget, rivers_per_elem=0.03, edges_per_elem=1.6, records_per_elem=0.01, max_systems=64)
    assert B.arena_bytes(lim) <= budget
    bigger = B.limits_for_memory(budget, 0.03, 1.6, 0.01, 64)
    bigger.max_elem += 1
    bigger.max_river = int(0.03 * bigger.max_elem) + 1
    bigger.max_edge = int(1.6 * bigger.max_elem) + 16
    bigger.max_record = int(0.01 * bigger.max_elem) + 1
    assert B.arena_bytes(bigger) > budget
    assert lim.max_systems == 64 and lim.max_elem > 1_000_000


def test_limits_for_memory_rejects_a_budget_too_small(B):
    from pihm_gpu.capi import PihmGpuError
    with pytest.raises(PihmGpuError):
        B.limits_for_memory(1024)
