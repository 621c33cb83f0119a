"""
The time blocking of the forward group kernels (run_group and
run_group_pipelined in csrc/tvbg_lanes.cuh) simulated on the host, no GPU:
a history ring of nh slots (slot s at s mod nh), blocks of K steps whose
delayed sums are all gathered before the block's updates write x(t + 1)
into slot t + 1.

The recursion keeps the kernels' data flow (a linear stand-in for a model):
x_j(t + 1) = a x_j(t) + sum_{in-edges j <- i, delay d} w x_i(t - d) + g_j(t),
zero history before t = 0 (slot 0 holds x(0)).

- One team: with every delay >= K - 1 the blocked schedule equals the
  step-by-step recursion, and a block's own writes never reach its gathers
  while nh >= d_max + 1 + K (on the device other threads write while a
  thread still gathers).
- Two teams (the pipelined kernel): block b + 1 is gathered while block b
  runs; with every delay >= 2K - 1 the gather may run before or after block
  b's writes, with the same result.
- Where a condition fails, the schedules differ.
"""

import numpy as np


def problem(N=6, dmin=15, dmax=40, T=150, seed=0):
    rng = np.random.default_rng(seed)
    edges = [(j, i, int(rng.integers(dmin, dmax + 1)), float(rng.normal()) / N)
             for j in range(N) for i in range(N) if i != j and rng.random() < 0.6]
    j, i, _, w = edges[0]
    edges[0] = (j, i, dmin, w)
    return edges, rng.normal(size=(T, N)), rng.normal(size=N)


def differs(x, y):
    return float(np.abs(x - y).max()) > 1e-6 * float(np.abs(y).max())


def step_by_step(edges, g, x0, a=0.5):
    T, N = g.shape
    x = np.zeros((T + 1, N))
    x[0] = x0
    past = lambda t: x[t] if t >= 0 else np.zeros(N)   # noqa: E731
    for t in range(T):
        s = np.zeros(N)
        for j, i, d, w in edges:
            s[j] += w * past(t - d)[i]
        x[t + 1] = a * x[t] + s + g[t]
    return x[T]


def blocked(edges, g, x0, K, nh, order=None, a=0.5):
    """order None: one team; 'racy': whether a block's gather would change
    if it ran after the block's own writes; 'before' / 'after': two teams,
    block b + 1 gathered before / after block b's writes."""
    T, N = g.shape
    ring = np.zeros((N, nh))
    ring[:, 0] = x0
    x = x0.copy()

    def gather(tb):
        sums = {}
        for t in range(tb, min(T, tb + K)):
            s = np.zeros(N)
            for j, i, d, w in edges:
                s[j] += w * ring[i, (t - d) % nh]
            sums[t] = s
        return sums

    def update(tb, sums):
        nonlocal x
        for t in range(tb, min(T, tb + K)):
            x = a * x + sums[t] + g[t]
            ring[:, (t + 1) % nh] = x

    starts = list(range(0, T, K))
    if order in (None, 'racy'):
        racy = False
        for tb in starts:
            sums = gather(tb)
            update(tb, sums)
            if order == 'racy':
                late = gather(tb)
                racy = racy or any(not np.array_equal(sums[t], late[t]) for t in sums)
        return racy if order == 'racy' else x
    nxt = gather(starts[0])
    for b, tb in enumerate(starts):
        cur = nxt
        if b + 1 < len(starts) and order == 'before':
            nxt = gather(starts[b + 1])
        update(tb, cur)
        if b + 1 < len(starts) and order == 'after':
            nxt = gather(starts[b + 1])
    return x


def test_one_team_blocking():
    for seed in range(3):
        edges, g, x0 = problem(dmin=7, dmax=40, seed=seed)
        ref = step_by_step(edges, g, x0)
        assert np.array_equal(blocked(edges, g, x0, K=8, nh=64), ref)
        assert not blocked(edges, g, x0, K=8, nh=64, order='racy')
    edges, g, x0 = problem(dmin=5, dmax=40, seed=1)       # a delay below K - 1
    assert differs(blocked(edges, g, x0, K=8, nh=64), step_by_step(edges, g, x0))
    edges, g, x0 = problem(dmin=7, dmax=40, seed=2)       # nh = d_max + 1 + K: race-free
    assert not blocked(edges, g, x0, K=8, nh=49, order='racy')
    edges[1] = edges[1][:2] + (41, edges[1][3])           # one more: a block's writes reach it
    assert blocked(edges, g, x0, K=8, nh=49, order='racy')


def test_two_team_blocking():
    for seed in range(3):
        edges, g, x0 = problem(dmin=15, dmax=40, seed=seed)
        ref = step_by_step(edges, g, x0)
        for order in ('before', 'after'):
            assert np.array_equal(blocked(edges, g, x0, K=8, nh=64, order=order), ref), order
    edges, g, x0 = problem(dmin=12, dmax=40, seed=4)      # a delay below 2K - 1
    ref = step_by_step(edges, g, x0)
    assert np.array_equal(blocked(edges, g, x0, K=8, nh=64, order='after'), ref)
    assert differs(blocked(edges, g, x0, K=8, nh=64, order='before'), ref)
