"""The adjoint's schedules (hmf_adjoint_schedule, host only: no GPU needed).

Every schedule is replayed on a model of the state slots: a forward
iteration must read x_t and write a different slot, the loss must see x_T,
and the backward steps must run from T-1 down to 0, each finding x_t and
x_{t+1} in the slots it names.  The fewest-forward-iterations schedule is
checked against an exhaustive shortest-path search over all slot contents
for small cases (the search knows nothing of the recursion)."""
import heapq

import pytest

from robartsvtk_gb300 import adjoint_schedule

FWD, LOSS, BWD = 0, 1, 2


def replay(actions, T, max_slots):
    """Checks a schedule; returns (slots used, forward iterations)."""
    held = {0: 0}  # slot -> t of the state it holds
    next_bwd = T - 1
    loss_seen = False
    n_fwd = 0
    used = {0}
    for kind, t, a, b in actions:
        for s in (a, b):
            if s >= 0:
                assert s < max_slots, (kind, t, a, b)
                used.add(s)
        if kind == FWD:
            assert held.get(a) == t and a != b and 0 <= t < T, (kind, t, a, b)
            held[b] = t + 1
            n_fwd += 1
        elif kind == LOSS:
            assert not loss_seen and t == T and held.get(a) == T
            loss_seen = True
        else:
            assert loss_seen and t == next_bwd, (kind, t, next_bwd)
            assert held.get(a) == t and held.get(b) == t + 1, (kind, t, a, b, held)
            next_bwd -= 1
    assert loss_seen and next_bwd == -1
    return len(used), n_fwd


def fewest_by_search(T, S):
    """Fewest forward iterations over S slots, by Dijkstra over (slot
    contents, next backward step, loss done); None when unreachable."""
    start = (tuple([0] + [-1] * (S - 1)), T - 1, False)
    dist = {start: 0}
    heap = [(0, start)]
    while heap:
        d, st = heapq.heappop(heap)
        if dist[st] < d:
            continue
        slots, nb, loss = st
        if nb < 0:
            return d
        moves = []
        if not loss and T in slots:
            moves.append((0, (slots, nb, True)))
        if loss and nb in slots and nb + 1 in slots:
            moves.append((0, (slots, nb - 1, True)))
        for a in range(S):
            t = slots[a]
            if 0 <= t < T:
                for b in range(S):
                    if b != a:
                        ns = list(slots)
                        ns[b] = t + 1
                        moves.append((1, (tuple(ns), nb, loss)))
        for c, s2 in moves:
            if d + c < dist.get(s2, 1 << 60):
                dist[s2] = d + c
                heapq.heappush(heap, (d + c, s2))
    return None


@pytest.mark.parametrize("T", [0, 1, 2, 7, 13, 30])
@pytest.mark.parametrize("k", [1, 2, 3, 5, 30])
def test_fixed_interval_schedule(T, k):
    acts = adjoint_schedule(T, checkpoint_every=k)
    kk = max(1, min(k, max(T, 1)))
    n_ckpt = max(1, -(-T // kk))
    slots, n_fwd = replay(acts, T, n_ckpt + kk)
    # every iteration once, then the inner states of every segment but the last again
    assert n_fwd == T + (n_ckpt - 1) * (kk - 1)


@pytest.mark.parametrize("T", range(1, 7))
@pytest.mark.parametrize("S", [2, 3, 4, 5])
def test_fewest_schedule_is_optimal(T, S):
    acts = adjoint_schedule(T, S)
    best = fewest_by_search(T, S)
    if best is None:
        assert acts is None
        return
    slots, n_fwd = replay(acts, T, S)
    assert n_fwd == best


@pytest.mark.parametrize("T", [1, 10, 57, 300])
def test_fewest_schedule_costs(T):
    costs = []
    for S in list(range(3, 12)) + [T // 2 + 1, T, T + 1, T + 5]:
        acts = adjoint_schedule(T, S)
        if acts is None:
            assert S <= 2  # three slots reach any T (x_0 plus a ping-pong pair)
            costs.append(None)
            continue
        slots, n_fwd = replay(acts, T, S)
        costs.append((S, n_fwd))
        if S >= T + 1:
            assert n_fwd == T  # every state kept: each iteration runs once
    got = [c for c in costs if c is not None]
    for (s1, c1), (s2, c2) in zip(got, got[1:]):
        if s2 >= s1:
            assert c2 <= c1  # more slots never cost more


def test_large_workload_schedule():
    """400 iterations (the 512x512x384 workload) over five slots: about
    nine forward passes."""
    acts = adjoint_schedule(400, 5)
    slots, n_fwd = replay(acts, 400, 5)
    assert slots == 5 and 400 < n_fwd < 10 * 400
    assert adjoint_schedule(400, 2) is None
