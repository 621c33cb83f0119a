"""
The time blocking of the reverse-time kernel on groups (adjoint_group_kernel
in csrc/tvbg_adjoint.cu) simulated on the host, no GPU: the adjoint ring of
nh slots (slot s at s mod nh), blocks of K reverse steps whose out-edge sums
are all gathered before the block's updates write mu(t + 1) into slot t + 1.

The recursion keeps the kernel's data flow (a linear stand-in for the MPR
terms): lambda_j(t) = a lambda_j(t+1) + sum_{edges j->i, delay d} w
mu_i(t + d + 1) + g_j(t), mu = lambda, zero beyond T.

- One team: with every delay >= K and nh >= d_max + K, the blocked schedule
  equals the step-by-step recursion.
- Two teams: block b + 1 is gathered while block b runs; with every delay
  >= 2K the gather may run entirely before or entirely after block b's ring
  writes, and both give the step-by-step result.
- Where a condition fails, the schedules differ (the check has teeth).
- The ring size: the slots a block writes alias none of its reads while
  nh >= d_max + K (on the device the other threads of a block write while
  a thread gathers).
"""

import numpy as np


def problem(N=6, dmin=16, dmax=40, T=150, seed=0):
    """Random out-edges with delays in [dmin, dmax] (dmin itself always
    present), weights scaled so that the recursion contracts."""
    rng = np.random.default_rng(seed)
    edges = [(j, i, int(rng.integers(dmin, dmax + 1)), float(rng.normal()) / N)
             for j in range(N) for i in range(N) if i != j and rng.random() < 0.6]
    j, i, _, w = edges[0]
    edges[0] = (j, i, dmin, w)
    g = rng.normal(size=(T, N))
    lam_T = rng.normal(size=N)
    return edges, g, lam_T


def differs(x, y):
    return float(np.abs(x - y).max()) > 1e-6 * float(np.abs(y).max())


def step_by_step(edges, g, lam_T, a=0.5):
    T, N = g.shape
    lam = np.zeros((T + 1, N))
    lam[T] = lam_T
    mu = lambda t: lam[t] if t <= T else np.zeros(N)   # noqa: E731
    for t in range(T - 1, -1, -1):
        coup = np.zeros(N)
        for j, i, d, w in edges:
            coup[j] += w * mu(t + d + 1)[i]
        lam[t] = a * lam[t + 1] + coup + g[t]
    return lam[0]


def blocked(edges, g, lam_T, K, nh, order=None, a=0.5):
    """order None: one team (gather block b, then its updates); 'racy':
    the same, returning whether any block's gather would change if it ran
    after the block's own ring writes (another thread's, on the device);
    'before' / 'after': two teams, block b + 1 gathered before / after block
    b's ring writes."""
    T, N = g.shape
    ring = np.zeros((N, nh))
    lam = lam_T.copy()

    def gather(tb):
        coup = {}
        for t in range(tb, max(-1, tb - K), -1):
            c = np.zeros(N)
            for j, i, d, w in edges:
                c[j] += w * ring[i, (t + d + 1) % nh]
            coup[t] = c
        return coup

    def update(tb, coup):
        nonlocal lam
        for t in range(tb, max(-1, tb - K), -1):
            ring[:, (t + 1) % nh] = lam          # mu(t + 1)
            lam = a * lam + coup[t] + g[t]

    tops = list(range(T - 1, -1, -K))
    if order in (None, 'racy'):
        racy = False
        for tb in tops:
            coup = gather(tb)
            update(tb, coup)
            if order == 'racy':
                # on the device other threads write their block-b slots while
                # a thread still gathers block b: the gather must not see them
                late = gather(tb)
                racy = racy or any(not np.array_equal(coup[t], late[t]) for t in coup)
        return racy if order == 'racy' else lam
    nxt = gather(tops[0])
    for b, tb in enumerate(tops):
        cur = nxt
        if b + 1 < len(tops):
            if order == 'before':
                nxt = gather(tops[b + 1])
                update(tb, cur)
            else:
                update(tb, cur)
                nxt = gather(tops[b + 1])
        else:
            update(tb, cur)
    return lam


def test_one_team_blocking():
    for seed in range(3):
        edges, g, lam_T = problem(dmin=8, dmax=40, seed=seed)
        ref = step_by_step(edges, g, lam_T)
        # the same additions in the same order: equal
        assert np.array_equal(blocked(edges, g, lam_T, K=8, nh=48), ref)
        assert np.array_equal(blocked(edges, g, lam_T, K=8, nh=64), ref)
    # a delay below K reads a slot the block has not written yet
    edges, g, lam_T = problem(dmin=5, dmax=40, seed=1)
    assert differs(blocked(edges, g, lam_T, K=8, nh=64), step_by_step(edges, g, lam_T))
    # the other threads' writes of a block never reach its gathers while
    # nh >= d_max + K; with nh < d_max + K they do
    edges, g, lam_T = problem(dmin=8, dmax=40, seed=2)
    assert not blocked(edges, g, lam_T, K=8, nh=48, order='racy')
    edges[1] = edges[1][:2] + (41, edges[1][3])
    assert blocked(edges, g, lam_T, K=8, nh=48, order='racy')


def test_two_team_blocking():
    for seed in range(3):
        edges, g, lam_T = problem(dmin=16, dmax=40, seed=seed)
        ref = step_by_step(edges, g, lam_T)
        for order in ('before', 'after'):
            got = blocked(edges, g, lam_T, K=8, nh=64, order=order)
            assert np.array_equal(got, ref), (seed, order)
    # with a delay below 2K the early gather misses slots block b writes
    edges, g, lam_T = problem(dmin=10, dmax=40, seed=4)
    ref = step_by_step(edges, g, lam_T)
    assert np.array_equal(blocked(edges, g, lam_T, K=8, nh=64, order='after'), ref)
    assert differs(blocked(edges, g, lam_T, K=8, nh=64, order='before'), ref)
