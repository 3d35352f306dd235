"""CPU tests of the binomial checkpointing schedule used by the adjoint sweep."""
import math

import pytest

from samoa_gb300.adjoint import binomial_split, revolve


class FakeStepper:
    """State = step index; checks that adjoint(t) sees the state at step t."""

    def __init__(self, slots):
        self.state = 0
        self.slots = {}
        self.free = list(range(slots))
        self.max_live = 0
        self.forward = 0
        self.order = []

    def store(self, step):
        assert self.state == step
        slot = self.free.pop()
        self.slots[slot] = step
        self.max_live = max(self.max_live, len(self.slots))
        return slot

    def restore(self, slot, step):
        assert self.slots[slot] == step
        self.state = step

    def advance(self, k):
        self.state += k
        self.forward += k

    def adjoint(self, t):
        assert self.state == t
        self.order.append(t)
        self.state = t + 1  # the adjoint step runs the forward step t first
        self.forward += 1

    def release(self, slot):
        del self.slots[slot]
        self.free.append(slot)


@pytest.mark.parametrize("n,s", [(1, 1), (2, 1), (10, 1), (10, 2), (50, 3), (200, 8), (2000, 64), (777, 5)])
def test_revolve_reverses_every_step_with_bounded_snapshots(n, s):
    f = FakeStepper(s)
    revolve(n, s, f)
    assert f.order == list(range(n - 1, -1, -1))
    assert f.max_live <= s
    r = 0
    while math.comb(s + r, s) < n:
        r += 1
    # each step is computed at most r + 1 times (r recomputations plus the adjoint's own step)
    assert f.forward <= (r + 1) * n, (f.forward, r, n)


def test_binomial_split_bounds():
    for length in range(2, 300):
        for s in range(1, 8):
            m = binomial_split(length, s)
            assert 1 <= m <= length - 1
