"""Binomial checkpoint schedules (host code of the library, no device).

The schedule is checked three ways: replayed on a model of the state slots
(every action legal, every segment reversed once, last to first), its cost
against the minimum of the checkpointing recursion computed here by
dynamic programming, and against Griewank's closed form at sizes the
recursion cannot reach."""
from functools import lru_cache
from math import comb

import numpy as np
import pytest

from fwi_cuda_gb300 import engine

SAVE_MAIN, RESTORE, ADVANCE, SAVE_WORK, REVERSE = 1, 2, 3, 4, 5


@lru_cache(maxsize=None)
def min_advances(n, s):
    """Fewest segment advances to reverse n segments with s state slots, the
    state at segment 0 held in one of them."""
    if n <= 1:
        return 0
    if s <= 1:
        return n * (n - 1) // 2
    return min(m + min_advances(n - m, s - 1) + min_advances(m, s) for m in range(1, n))


def replay(actions, n, slots):
    """Run the actions on a model of the slots; returns (advances, spine)
    where spine is how far the forward pass carried its saves."""
    live = {}
    work = None
    done = []
    fwd = actions[actions[:, 0] == SAVE_MAIN]
    assert fwd[0, 1] == 0 and np.all(np.diff(fwd[:, 1]) > 0)
    for _, seg, slot in fwd:
        assert 0 <= slot < slots and slot not in live
        live[slot] = seg
    advances = 0
    for op, seg, slot in actions[len(fwd):]:
        assert op != SAVE_MAIN
        if op == RESTORE:
            assert live[slot] == seg
            work = seg
        elif op == ADVANCE:
            assert work == seg
            work = seg + 1
            advances += 1
        elif op == SAVE_WORK:
            # a later RESTORE names the segment it expects, so a slot
            # overwritten while still needed fails there
            assert work == seg and 0 <= slot < slots
            live[slot] = seg
        elif op == REVERSE:
            assert work == seg
            done.append(seg)
            work = None
        else:
            raise AssertionError(op)
    assert done == list(range(n - 1, -1, -1))
    return advances, int(fwd[-1, 1])


@pytest.mark.parametrize("n", [1, 2, 3, 5, 10, 17, 31])
@pytest.mark.parametrize("slots", [1, 2, 3, 4, 6])
def test_schedule_is_legal_and_optimal(n, slots):
    a, adv = engine.checkpoint_schedule(n, slots)
    got, spine = replay(a, n, min(slots, n))
    assert got == adv
    # the forward pass's saves stand for the spine's advances
    assert adv + spine == min_advances(n, min(slots, n))


def test_enough_slots_is_the_two_level_scheme():
    a, adv = engine.checkpoint_schedule(12, 12)
    assert adv == 0
    assert list(a[a[:, 0] == SAVE_MAIN][:, 1]) == list(range(12))
    assert (a[:, 0] == RESTORE).sum() == 12  # one restore per segment, no saves of the working state
    assert not (a[:, 0] == SAVE_WORK).any()


@pytest.mark.parametrize("n,slots", [(4000, 90), (3334, 20), (1000, 3), (12000, 400)])
def test_large_schedules_meet_the_closed_form(n, slots):
    a, adv = engine.checkpoint_schedule(n, slots)
    got, spine = replay(a, n, slots)
    assert got == adv
    t = 0
    while comb(slots + t, t) < n:
        t += 1
    assert adv + spine == t * n - comb(slots + t, t - 1)


def test_schedule_rejects_bad_arguments():
    from fwi_cuda_gb300 import _lib
    with pytest.raises(_lib.PSVError):
        engine.checkpoint_schedule(0, 3)
    with pytest.raises(_lib.PSVError):
        engine.checkpoint_schedule(5, 0)


def test_schedules_beyond_the_advance_cap_are_refused_before_they_are_built():
    # one action per segment advance: a few slots forced on a very long
    # record would list 10^8..10^10 actions; the closed form refuses them at
    # once (2^26 advances at most)
    import time
    from fwi_cuda_gb300 import _lib

    def F(n, s):  # Griewank's closed form
        if n <= 1:
            return 0
        if s == 1:
            return n * (n - 1) // 2
        t = 0
        while comb(s + t, t) < n:
            t += 1
        return t * n - comb(s + t, t - 1)

    assert all(F(n, s) == min_advances(n, s) for n in range(1, 40) for s in range(1, 6))
    for n, slots in ((100000, 1), (11586, 1), (10 ** 6, 3)):
        assert F(n, slots) > 2 ** 26
        t = time.time()
        with pytest.raises(_lib.PSVError) as e:
            engine.checkpoint_schedule(n, slots)
        assert e.value.status == _lib.PSV_ERR_ARG and time.time() - t < 1.0
    assert F(11585, 1) <= 2 ** 26 and F(3334, 1) == 3334 * 3333 // 2
