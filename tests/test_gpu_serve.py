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
