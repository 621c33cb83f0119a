"""
The drop-in executor: transforms.network_time_step called exactly as
tvb_hpc/examples/hackathon.py:48-54 calls the fused loopy kernel
(kwargs, numpy arrays updated in place, nstep=10 chunks with i_step_0).
  - parity with the oracle in Track-A order over 1000 steps (normalised
    weights, so the dynamics are not chaotic and 1e-4 is meaningful);
  - the hackathon FC-SC known-answer test (hackathon.py:88-89) on hcp0.
"""

import os

import numpy as np
import pytest

from conftest import GOLDEN, circ_rel_err

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, transforms

pytestmark = pytest.mark.gpu


def make_knl(dt=1.0, omega=10.0 * 2.0 * np.pi / 1e3):
    "hackathon.py:23-33, with the coupling a as a kernel argument."
    osc = model.Kuramoto()
    osc.dt = dt
    osc.const['omega'] = omega
    cfun = coupling.Kuramoto(osc)
    cfun.param['a'] = 'a'
    scm = scheme.EulerStep(osc.dt)
    knl = transforms.network_time_step(osc, cfun, scm)
    return knl, osc


def test_executor_numpy_kwargs_parity(cuda):
    w, ln = network.synthetic_connectome(84, 0.3, seed=21)
    c = network.Connectivity.from_dense(w, ln)
    knl, osc = make_knl(dt=0.1)
    speed, a = 4.0, 2.5
    lnz = c.delays(speed, osc.dt, 'trunc').astype(np.uintc)
    np.random.seed(5)
    state, input, param, drift, diffs, _ = osc.prep_arrays(c.nnode)
    state0 = state.copy()
    obsrv = np.zeros((lnz.max() + 3 + 1000, c.nnode, 2), np.float32)
    for i in range(100):
        knl(nstep=10, nnode=c.nnode, ntime=obsrv.shape[0], state=state, input=input,
            param=param, drift=drift, diffs=diffs, obsrv=obsrv, nnz=c.nnz, delays=lnz,
            row=c.row, col=c.col, weights=c.wnz, a=a, i_step_0=i * 10)
    ntime = obsrv.shape[0]
    ref = orc.run(0, 2, c.row, c.col, c.wnz, ntime, 1000, 0.1, lnz[None].astype(np.int32), [a],
                  param[None, :, 0], state0[None], flags=orc.F_TRACKA, trace_every=1,
                  trace_len=ntime, trace_nobs=2)
    assert circ_rel_err(state, ref['state'][0]) < 1e-4
    assert circ_rel_err(obsrv[:1000, :, 0], ref['trace'][0, :1000, :, 0]) < 1e-4
    assert np.abs(obsrv[:1000, :, 1] - ref['trace'][0, :1000, :, 1]).max() < 1e-4


def test_executor_batched_form(cuda):
    "Leading nsubj axis on state/param/obsrv (examples/hcp100.py:75-80)."
    torch = cuda
    w, ln = network.synthetic_connectome(50, 0.3, seed=22)
    c = network.Connectivity.from_dense(w, ln)
    knl, osc = make_knl(dt=0.1)
    lnz = c.delays(5.0, 0.1, 'ceil').astype(np.uintc)
    S = 4
    rng = np.random.default_rng(0)
    st = rng.uniform(0, 2 * np.pi, (S, 50, 1)).astype(np.float32)
    pa = np.full((S, 50, 1), 0.0628, np.float32)
    ntime = int(lnz.max()) + 1 + 300
    ob = torch.zeros((ntime, S, 50, 2), device='cuda')
    st_d = torch.from_numpy(st).cuda()
    a = np.array([0.5, 1.0, 2.0, 4.0], np.float32)
    for i in range(30):
        knl(nstep=10, nnode=50, ntime=ntime, state=st_d, input=None,
            param=torch.from_numpy(pa).cuda(), drift=None, diffs=None, obsrv=ob, nnz=c.nnz,
            delays=lnz, row=c.row, col=c.col, weights=c.wnz, a=a, i_step_0=i * 10)
    ref = orc.run(0, 2, c.row, c.col, c.wnz, ntime, 300, 0.1,
                  np.broadcast_to(lnz.astype(np.int32), (S, lnz.size)), a, pa[:, :, 0], st,
                  flags=orc.F_TRACKA, trace_every=1, trace_len=ntime, trace_nobs=2)
    assert circ_rel_err(st_d.cpu().numpy(), ref['state']) < 1e-4
    got = ob.cpu().numpy()[:300, :, :, 0].transpose(1, 0, 2)
    assert circ_rel_err(got, ref['trace'][:, :300, :, 0]) < 1e-4


@pytest.mark.parametrize('seed', [0, 1])
def test_hackathon_known_answer_gpu(cuda, seed):
    "hackathon.py:58-89 through the drop-in executor, batched over couplings."
    torch = cuda
    c = network.Connectivity.hcp0(os.path.join(GOLDEN, 'hcp0.npz'))
    knl, osc = make_knl()
    nc, ns = 8, 8
    couplings = np.logspace(0, 1.0, nc).astype(np.float32)
    speeds = np.logspace(0.0, 2.0, ns)
    theta0 = np.random.default_rng(seed).uniform(0, 2 * np.pi, (c.nnode, 1)).astype(np.float32)
    trace = np.zeros((nc * ns, 400, c.nnode), np.float32)
    for si, speed in enumerate(speeds):
        lnz = (c.lnz / np.float32(speed) / np.float32(osc.dt)).astype(np.uintc)
        st = torch.from_numpy(np.broadcast_to(theta0, (nc, c.nnode, 1)).copy()).cuda()
        pa = torch.full((nc, c.nnode, 1), osc.const['omega'], device='cuda')
        ntime = int(lnz.max()) + 3 + 4000
        ob = torch.zeros((ntime, nc, c.nnode, 2), device='cuda')
        for i in range(400):
            knl(nstep=10, nnode=c.nnode, ntime=ntime, state=st, input=None, param=pa,
                drift=None, diffs=None, obsrv=ob, nnz=c.nnz, delays=lnz, row=c.row, col=c.col,
                weights=c.wnz, a=couplings, i_step_0=i * 10)
        tr = ob[:4000, :, :, 0].cpu().numpy().reshape(400, 10, nc, c.nnode).sum(1)
        trace[si * nc:(si + 1) * nc] = tr.transpose(1, 0, 2)
    import test_oracle_pins as pins
    ds, dc = pins.hackathon_derr(lambda s, cc: trace[list(speeds).index(s) * nc:
                                                     (list(speeds).index(s) + 1) * nc],
                                 c.weights)
    assert ds > 350.0, ds
    assert dc < -500.0, dc
