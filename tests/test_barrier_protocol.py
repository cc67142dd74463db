"""The arrival protocol of the persistent tetrahedral step's grid barrier
(`grid_barrier` in emsolvers_gb300/csrc/tetfem.cu), checked as a model on
the CPU: block 0 adds 2^31 - (expected - 1) to a 32-bit counter, every other
block adds 1, and a block waits until the counter's top bit differs from
the value its own add returned.  Under every interleaving of arrivals and
polls (fast blocks reaching the next barrier before slow ones have seen the
last flip), no block leaves a barrier before all blocks have arrived at it,
every block leaves it once they have, and the counter's low bits are zero
again after each barrier; with expected one higher than the grid (the
timeout test's setting) no block ever leaves."""
import numpy as np
import pytest

TOP = 0x80000000
MASK = 0xFFFFFFFF


def _run(nblocks, expected, rounds, seed, max_events=200000):
    rng = np.random.default_rng(seed)
    count = 0
    rnd = [0] * nblocks            # the barrier each block is at (or heading to)
    waiting = [False] * nblocks
    old = [0] * nblocks
    arrived = {}                   # barrier -> blocks that arrived
    left = {}
    for _ in range(max_events):
        if all(r >= rounds for r in rnd):
            break
        b = int(rng.integers(nblocks))
        if rnd[b] >= rounds:
            continue
        if not waiting[b]:
            add = (TOP - (expected - 1)) & MASK if b == 0 else 1
            old[b] = count
            count = (count + add) & MASK
            arrived[rnd[b]] = arrived.get(rnd[b], 0) + 1
            waiting[b] = True
        elif (count ^ old[b]) & TOP:
            assert arrived[rnd[b]] == nblocks, "a block left a barrier before all had arrived"
            left[rnd[b]] = left.get(rnd[b], 0) + 1
            waiting[b] = False
            rnd[b] += 1
    return count, rnd, arrived, left


@pytest.mark.parametrize("nblocks", [1, 2, 3, 7, 64])
def test_no_block_leaves_before_all_arrive_and_all_leave(nblocks):
    for seed in range(20):
        count, rnd, arrived, left = _run(nblocks, nblocks, 12, seed)
        assert all(r == 12 for r in rnd)
        assert all(left[r] == nblocks for r in range(12))
        assert count & (TOP - 1) == 0        # the low bits reset after every barrier


def test_the_grid_of_the_headline_mesh():
    count, rnd, _, left = _run(1125, 1125, 3, 0, max_events=3_000_000)
    assert all(r == 3 for r in rnd) and all(left[r] == 1125 for r in range(3))
    assert count & (TOP - 1) == 0


@pytest.mark.parametrize("nblocks", [1, 2, 5, 64])
def test_expecting_one_block_more_never_completes(nblocks):
    # the EMS_TET_BARRIER_PROBE setting: every wait must run out
    count, rnd, arrived, left = _run(nblocks, nblocks + 1, 2, 1, max_events=20000)
    assert all(r == 0 for r in rnd)
    assert arrived[0] == nblocks and not left
