"""
The continuous-batching server: requests of different models, sizes,
instance counts and step counts admitted while others run; each request's
result is the same alone and in the mix (bit-exact: chunk boundaries are
exact and every request keeps its own Philox key and launch shape), the
HBM budget is respected, and latencies are recorded.
"""

import numpy as np
import pytest

from tvb_hpc import network, serve

pytestmark = pytest.mark.gpu


def conns():
    out = []
    for k, (N, dens) in enumerate([(68, 0.3), (84, 0.3), (192, 0.15)]):
        w, ln = network.synthetic_connectome(N, dens, seed=k)
        out.append(network.Connectivity.from_dense(w, ln))
    return out


def requests(seed=0, n=6):
    rng = np.random.default_rng(seed)
    return serve.random_requests(n, rate=1e6, rng=rng, conns=conns(), inst=(1, 24),
                                 steps=(300, 2500), grad_frac=0.0)


def test_alone_equals_in_the_mix(cuda):
    reqs = requests()
    srv = serve.Server(chunk=700)
    for r in reqs:
        srv.submit(r)
    done = {r.rid: r for r in srv.run()}
    assert len(done) == len(reqs)
    assert {r.model for r in reqs} >= {'Kuramoto', 'G2DO'}
    for r in requests():          # the same requests, one server each
        solo = serve.Server(chunk=700)
        solo.submit(r)
        (a, ) = solo.run()
        assert np.array_equal(a.state, done[r.rid].state), r.model
    st = srv.stats()
    assert st['requests'] == len(reqs) and st['p99_s'] >= st['p50_s'] > 0


def test_admission_respects_budget(cuda):
    reqs = requests(seed=1, n=5)
    need = [serve.footprint(r) for r in reqs]
    budget = max(need) * 1.5       # at most one or two requests at a time
    srv = serve.Server(hbm_budget=budget, chunk=500)
    for r in reqs:
        srv.submit(r)
    peak = 0
    while srv.queue or srv.active:
        srv.tick()
        peak = max(peak, srv.used + sum(x.nbytes for x in []))
        assert srv.used <= budget
    assert len(srv.done) == len(reqs)


def test_late_arrivals_join_running_work(cuda):
    "A request arriving while another runs is admitted at the next tick."
    reqs = requests(seed=2, n=2)
    t = [0.0]
    srv = serve.Server(chunk=200, clock=lambda: t[0])
    reqs[0].arrival, reqs[1].arrival = 0.0, 0.5
    reqs[0].nsteps = reqs[1].nsteps = 1000
    for r in reqs:
        srv.submit(r)
    srv.tick()
    assert [r.rid for r in srv.active] == [reqs[0].rid]
    t[0] = 1.0
    srv.tick()
    assert {r.rid for r in srv.active} == {reqs[0].rid, reqs[1].rid}
    while srv.queue or srv.active:
        t[0] += 1.0
        srv.tick()
    assert all(r.steps_done == r.nsteps for r in srv.done)


def test_poll_and_cancel(cuda):
    "A queued and an active request are cancelled; the rest finish unchanged."
    reqs = requests(seed=3, n=4)
    for r in reqs:
        r.nsteps = max(r.nsteps, 1500)
    srv = serve.Server(chunk=500)
    for r in reqs:
        srv.submit(r)
    assert srv.poll(reqs[0].rid) == 'queued' and srv.poll(12345) is None
    srv.tick()
    assert srv.poll(reqs[1].rid) == 'active'
    used = srv.used
    assert srv.cancel(reqs[1].rid)
    assert srv.used == used - reqs[1].nbytes
    assert srv.poll(reqs[1].rid) == 'cancelled'
    assert not srv.cancel(reqs[1].rid)
    done = {r.rid: r for r in srv.run()}
    assert reqs[1].rid not in done and len(done) == len(reqs) - 1
    for r in requests(seed=3, n=4):
        if r.rid == reqs[1].rid:
            continue
        r.nsteps = max(r.nsteps, 1500)
        solo = serve.Server(chunk=500)
        solo.submit(r)
        (a, ) = solo.run()
        assert np.array_equal(a.state, done[r.rid].state)


def test_native_pool_equals_groups(cuda):
    """The C++ serving pool (tvbg_serve_*): every request's final state is
    bit-identical to lane-interleaved groups of the same inputs run alone,
    with requests of different models and sizes in the mix."""
    from tvb_hpc import groups, model as mdl, scheme as sch
    reqs = [r for r in requests(seed=5, n=8)]
    pool = serve.NativeServer(chunk=600)
    for r in reqs:
        pool.submit(r)
    assert pool.poll(reqs[0].rid) == 'queued'
    done = {r.rid: r for r in pool.run()}
    assert len(done) == len(reqs)
    for r in requests(seed=5, n=8):
        M, C, noise = serve.MODELS[r.model]
        m = M()
        scm = sch.EulerMaryuyamaStep(r.dt) if noise else sch.EulerStep(r.dt)
        gs = groups.GroupSet(m, C(m), scm, r.conn, r.dt, couplings=r.couplings, speeds=r.speeds,
                             state0=r.x0, nparam=r.nparam, seed=r.seed)
        gs.run(r.nsteps)
        ref = gs.state.cpu().numpy()
        got = done[r.rid].state
        if C is serve.cpl.Diff:   # in-edge weight sums: the pool sums sequentially
            assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), r.model
        else:
            assert np.array_equal(got, ref), r.model
    assert pool.used() == 0


def test_native_pool_budget_cancel(cuda):
    reqs = requests(seed=6, n=4)
    for r in reqs:
        r.nsteps = max(r.nsteps, 1500)
    probe = serve.NativeServer(chunk=500)
    for r in reqs:
        probe.submit(r)
    fp = [probe.footprint(r.rid) for r in reqs]
    probe.close()
    pool = serve.NativeServer(hbm_budget=1.5 * max(fp), chunk=500)   # one or two at a time
    for r in reqs:
        pool.submit(r)
    a, q = pool.tick()
    assert a >= 1 and a + q == len(reqs) and pool.used() <= 1.5 * max(fp)
    # issued steps: those taken plus the chunk running now (<= one chunk ahead)
    for r in reqs:
        d, i = pool.steps_done(r.rid), pool.steps_issued(r.rid)
        assert d <= i <= min(r.nsteps, d + 500)
    assert pool.cancel(reqs[-1].rid) and pool.poll(reqs[-1].rid) == 'cancelled'
    assert not pool.cancel(reqs[-1].rid)
    rest = pool.run()
    assert {r.rid for r in rest} == {r.rid for r in reqs[:-1]}
    assert pool.used() == 0


def test_server_with_native_pool(cuda):
    """Server(native=True): requests without gradients run in the C++ pool,
    the gradient requests on the Python path, in the same ticks; every
    result equals the same request served alone."""
    rng = np.random.default_rng(9)
    reqs = serve.random_requests(8, rate=1e6, rng=rng, conns=conns(), inst=(1, 16),
                                 steps=(300, 1500), grad_frac=1.0)
    assert any(r.want_grad for r in reqs) and not all(r.want_grad for r in reqs)
    srv = serve.Server(chunk=500, native=True)
    for r in reqs:
        srv.submit(r)
    done = {r.rid: r for r in srv.run()}
    assert len(done) == len(reqs) and not srv.busy
    assert srv.native.used() == 0
    for r in serve.random_requests(8, rate=1e6, rng=np.random.default_rng(9), conns=conns(),
                                   inst=(1, 16), steps=(300, 1500), grad_frac=1.0):
        solo = serve.Server(chunk=500, native=True)
        solo.submit(r)
        (a, ) = solo.run()
        assert np.array_equal(a.state, done[r.rid].state), r.model
        if r.want_grad:
            assert all(np.array_equal(x, y) for x, y in zip(a.grad, done[r.rid].grad))
    st = srv.stats()
    assert st['requests'] == len(reqs) and st['p99_s'] >= st['p50_s'] > 0


def test_hybrid_server_shares_the_budget(cuda):
    """Server(native=True): the Python path (gradient requests) and the
    native pool admit against one budget; at every tick the bytes both hold
    stay within it.  A request larger than the budget fails instead of
    waiting forever."""
    rng = np.random.default_rng(21)
    reqs = serve.random_requests(10, rate=1e6, rng=rng, conns=conns(), inst=(4, 24),
                                 steps=(800, 2000), grad_frac=0.5)
    assert any(r.want_grad for r in reqs) and not all(r.want_grad for r in reqs)
    need = [serve.footprint(r) for r in reqs]
    budget = 2.2 * max(need)
    srv = serve.Server(hbm_budget=budget, chunk=400, native=True)
    # an MPR gradient request (the Python path, where its footprint is checked)
    big = serve.random_requests(1, rate=1e6, rng=np.random.default_rng(3), conns=conns()[2:],
                                models=('MPR', ), inst=(4000, 4000), steps=(500, 500),
                                grad_frac=1.0)[0]
    big.rid = 999
    assert big.want_grad and serve.footprint(big) > budget
    for r in reqs + [big]:
        srv.submit(r)
    peak = 0
    for _ in range(10000):
        if not srv.busy:
            break
        srv.tick()
        held = srv.used + srv.native.used()
        peak = max(peak, held)
        assert held <= budget
    srv._collect(wait=True)
    assert not srv.busy
    assert srv.poll(999) == 'failed' and 'exceeds the budget' in big.error
    assert {r.rid for r in srv.done} == {r.rid for r in reqs}
    assert peak > 0
