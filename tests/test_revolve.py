"""The binomial checkpoint schedule (lsh_revolve.h through lsh_revolve_plan,
host code, no GPU): every step reversed once, in order, from the right
state, with the fewest forward steps -- checked against a brute-force
dynamic program over all split points."""
from functools import lru_cache

import pytest

from landslidehysea_gb300.solver import revolve_plan


@lru_cache(None)
def brute(n, s):
    """Fewest forward steps to reverse n steps with s state slots (the
    start's included): restore-and-advance with one slot, else the best
    first checkpoint j."""
    if n <= 1:
        return 0
    if s == 1:
        return n * (n - 1) // 2
    return min(j + brute(n - j, s - 1) + brute(j, s) for j in range(1, n))


@pytest.mark.parametrize("s", [1, 2, 3, 4, 5, 8])
def test_schedule_is_optimal(s):
    for n in range(1, 90):
        fw, opt = revolve_plan(n, s)
        assert fw == brute(n, s) == (opt if n > 1 else 0), (n, s, fw, opt)


def test_schedule_large():
    # enough slots: every state stored once, no recomputation beyond the descent
    fw, opt = revolve_plan(4000, 4000)
    assert fw == opt == 3999
    # the 1024^2 adjoint configuration's scale: 4000 steps in 250 slots
    fw, opt = revolve_plan(4000, 250)
    assert fw == opt
    assert fw < 3 * 4000
