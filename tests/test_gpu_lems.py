"""
Kernels generated from LEMS-XML model files (tvb_hpc.lems), on the GPU:
against the LEMS oracle for every bundled model (1e-4 relative, circular
for phases), against the engine's hand-written kernels for the models both
have (the reference's own check of templated vs hand-written kernels,
dsl/dsl_cuda/example/cuda_setup.py:161-169), chunked runs bit-exact with
one run, the exposures and the run_simulation layout, and the noise path by
its statistics (one state variable, and six through the wide path).
"""

import numpy as np
import pytest

from conftest import rel_err, circ_rel_err

import lems_oracle as lo
from tvb_hpc import lems, network, model, coupling, scheme, engine
import tvb_hpc._native as nat

pytestmark = pytest.mark.gpu

TOL = 1e-4


def conn_of(N=60, seed=3):
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    return network.Connectivity.from_dense(w, ln)


def state0_of(name, N, seed=0):
    rng = np.random.default_rng(seed)
    if name == 'Kuramoto':
        return rng.uniform(0, 2 * np.pi, (N, 1)).astype(np.float32)
    if name == 'Oscillator':
        return rng.uniform(-0.5, 0.5, (N, 2)).astype(np.float32)
    if name == 'Rwongwang':
        return rng.uniform(0.1, 0.4, (N, 1)).astype(np.float32)
    if name == 'Epileptor':
        x = np.zeros((N, 6), np.float32)
        x[:, 0] = rng.uniform(-1.8, -1.2, N)
        x[:, 1] = rng.uniform(-15, -12, N)
        x[:, 2] = rng.uniform(2.8, 3.2, N)
        x[:, 3] = rng.uniform(-1.2, -0.8, N)
        x[:, 4] = rng.uniform(0, 0.2, N)
        x[:, 5] = rng.uniform(-0.1, 0.1, N)
        return x
    raise KeyError(name)


PARAMS = np.array([[2.0, 0.05], [5.0, 0.4], [12.0, 1.5]], np.float32)


@pytest.mark.parametrize('name,steps,single,kind', [
    ('Kuramoto', 400, False, 'sweep'), ('Oscillator', 400, False, 'sweep'),
    ('Rwongwang', 400, False, 'sweep'), ('Epileptor', 300, False, 'sweep'),
    ('Oscillator', 400, True, 'sweep'), ('Epileptor', 300, True, 'sweep'),
    ('Kuramoto', 400, False, 'groups'), ('Oscillator', 400, False, 'groups'),
    ('Epileptor', 300, False, 'groups'), ('Epileptor', 300, True, 'groups')])
def test_lems_matches_oracle(cuda, name, steps, single, kind):
    conn = conn_of()
    N = conn.nnode
    x0 = state0_of(name, N)
    m = lems.load_model(name)
    Set = lems.LemsSweep if kind == 'sweep' else lems.LemsGroupSet
    sw = Set(m, conn, 0.1, PARAMS, state0=x0, single=single)
    sw.run(steps)
    got = sw.state.cpu().numpy()
    ref = lo.run(lems.lems_file(name), name, conn.row, conn.col, conn.wnz, conn.lnz, PARAMS, 0.1,
                 steps, x0)
    assert np.isfinite(ref['state']).all()
    err = circ_rel_err if name == 'Kuramoto' else rel_err
    assert err(got, ref['state']) < TOL
    ex = sw.exposures().cpu().numpy()
    assert ex.shape == ref['expo'].shape
    assert err(ex, ref['expo']) < TOL


def test_lems_kuramoto_matches_hand_written_kernel(cuda):
    "The generated Kuramoto against the engine's own (fmod wrap, 'dsl' delays)."
    conn = conn_of(68, seed=1)
    N = conn.nnode
    x0 = state0_of('Kuramoto', N, seed=4)
    m = lems.load_model('Kuramoto')
    sw = lems.LemsSweep(m, conn, 0.1, PARAMS, state0=x0)
    sw.run(500)
    omega = lo.ceval('2.0 * M_PI_F * 0.01', {}).astype(np.float32)
    km = model.Kuramoto()
    hw = engine.Sweep(km, coupling.Kuramoto(km), scheme.EulerStep(0.1), conn, 0.1,
                      couplings=PARAMS[:, 1], speeds=PARAMS[:, 0], rounding='dsl', state0=x0,
                      nparam=np.full((N, 1), omega, np.float32), flags=nat.F_WRAP_FMOD)
    hw.run(500)
    assert circ_rel_err(sw.state.cpu().numpy(), hw.state.cpu().numpy()) < 1e-5


def test_lems_oscillator_and_rww_match_hand_written_kernels(cuda):
    conn = conn_of(50, seed=2)
    N = conn.nnode
    # 2-D oscillator, mean sine coupling
    x0 = state0_of('Oscillator', N, seed=5)
    sw = lems.LemsSweep(lems.load_model('Oscillator'), conn, 0.1, PARAMS, state0=x0)
    sw.run(400)
    g = model.Generic2dOscillator()
    hw = engine.Sweep(g, coupling.Kuramoto(g), scheme.EulerStep(0.1), conn, 0.1,
                      couplings=PARAMS[:, 1], speeds=PARAMS[:, 0], rounding='dsl', state0=x0)
    hw.run(400)
    assert rel_err(sw.state.cpu().numpy(), hw.state.cpu().numpy()) < TOL
    # reduced Wong-Wang, linear coupling, zero delays
    x0 = state0_of('Rwongwang', N, seed=6)
    sw = lems.LemsSweep(lems.load_model('Rwongwang'), conn, 0.1, PARAMS, state0=x0)
    sw.run(400)
    r = model.RWW()
    hw = engine.Sweep(r, coupling.Linear(r), scheme.EulerStep(0.1), conn, 0.1,
                      couplings=PARAMS[:, 1], delays=np.zeros(conn.nnz, np.int32), state0=x0)
    hw.run(400)
    assert rel_err(sw.state.cpu().numpy(), hw.state.cpu().numpy()) < TOL


@pytest.mark.parametrize('name', ['Epileptor', 'Ou6'])
def test_lems_chunks_bit_exact(cuda, name):
    conn = conn_of(40, seed=8)
    N = conn.nnode
    m = lems.load_model(name)
    x0 = state0_of(name, N) if name == 'Epileptor' else None
    a = lems.LemsSweep(m, conn, 0.1, PARAMS, state0=x0, seed=11)
    b = lems.LemsSweep(m, conn, 0.1, PARAMS, state0=x0, seed=11)
    a.run(300)
    for n in (1, 137, 162):
        b.run(n)
    assert np.array_equal(a.state.cpu().numpy(), b.state.cpu().numpy())
    assert np.array_equal(a.ring.cpu().numpy(), b.ring.cpu().numpy())


@pytest.mark.parametrize('name', ['Ou', 'Ou6'])
def test_lems_noise_statistics(cuda, name):
    """Uncoupled OU nodes (global_coupling 0): after 2000 steps every
    variable is stationary with variance nsig^2 / (1 - (1 - k dt)^2), the
    variables uncorrelated; seeds give different, reproducible streams."""
    conn = conn_of(200, seed=9)
    N = conn.nnode
    m = lems.load_model(name)
    params = np.array([[4.0, 0.0]] * 8, np.float32)
    sw = lems.LemsSweep(m, conn, 0.1, params, state0=np.zeros((N, m.ns), np.float32), seed=5)
    sw.run(2000)
    x = sw.state.cpu().numpy().reshape(-1, m.ns).astype(np.float64)
    nsig = np.sqrt(np.float32(0.1)) * np.float32(0.1)
    var = nsig ** 2 / (1 - (1 - 0.5 * 0.1) ** 2)
    n = x.shape[0]
    for v in range(m.ns):
        assert abs(x[:, v].mean()) < 5 * np.sqrt(var / n)
        assert abs(x[:, v].var() / var - 1) < 5 * np.sqrt(2.0 / n)
    if m.ns > 1:
        c = np.corrcoef(x.T)
        assert np.abs(c - np.eye(m.ns)).max() < 5 / np.sqrt(n)
    again = lems.LemsSweep(m, conn, 0.1, params, state0=np.zeros((N, m.ns), np.float32), seed=5)
    again.run(2000)
    assert np.array_equal(again.state.cpu().numpy(), sw.state.cpu().numpy())
    other = lems.LemsSweep(m, conn, 0.1, params, state0=np.zeros((N, m.ns), np.float32), seed=6)
    other.run(2000)
    assert not np.array_equal(other.state.cpu().numpy(), again.state.cpu().numpy())


def test_run_simulation_layout(cuda):
    "tavg (nstep, n_nodes * nexpo, n_work) after each launch, as cuda_run.py returns it."
    w, ln = network.synthetic_connectome(30, 0.3, seed=4)
    m = lems.load_model('Kuramoto')
    tavg, sw = lems.run_simulation(m, w, ln, PARAMS, 0.1, nstep=3, n_inner_steps=50, noise=False)
    assert tavg.shape == (3, 30 * 2, 3)
    conn = network.Connectivity.from_dense(w, ln)
    ref = lo.run(lems.lems_file('Kuramoto'), 'Kuramoto', conn.row, conn.col, conn.wnz, conn.lnz,
                 PARAMS, 0.1, 150)
    # sin(theta) rows of the last launch
    np.testing.assert_allclose(tavg[-1, 30:, :].T, ref['expo'][:, :, 1], atol=1e-4)


def test_lems_groups_take_separable_and_sine_couplings(cuda):
    """The group kernel runs separable couplings with pre applied at the ring
    write (here the linear OU coupling with a nonzero per-work-item scale)
    and falls back to the per-step kernel for zero delays."""
    conn = conn_of(50, seed=12)
    N = conn.nnode
    m = lems.load_model('Ou')
    x0 = np.random.default_rng(3).uniform(-0.5, 0.5, (N, 1)).astype(np.float32)
    params = np.array([[4.0, 0.02], [4.0, 0.05], [9.0, 0.1]], np.float32)
    gs = lems.LemsGroupSet(m, conn, 0.1, params, state0=x0, noise=False)
    gs.run(500)
    ref = lo.run(lems.lems_file('Ou'), 'Ou', conn.row, conn.col, conn.wnz, conn.lnz, params, 0.1,
                 500, x0)
    assert rel_err(gs.state.cpu().numpy(), ref['state']) < TOL
    kur = lems.make_set(lems.load_model('Kuramoto'), conn, 0.1, PARAMS)
    assert isinstance(kur, lems.LemsGroupSet) and kur.channels == 2
    # a coupling the group kernel cannot take falls back to the per-step kernel
    edge = lems.parse(open(lems.lems_file('Ou')).read().replace('expression="x_j"',
                                                               'expression="tanh(x_j - x)"'))
    assert isinstance(lems.make_set(edge, conn, 0.1, params), lems.LemsSweep)


@pytest.mark.parametrize('name,speed,k', [('Rwongwang', 1.0, 1), ('Kuramoto', 60.0, 2),
                                          ('Epileptor', 60.0, 2)])
def test_lems_groups_short_blocks(cuda, name, speed, k):
    "Zero delays (K = 1) and d_min = 1 (K = 2) on the group kernel, against the oracle."
    conn = conn_of(60, seed=13)
    N = conn.nnode
    x0 = state0_of(name, N)
    m = lems.load_model(name)
    params = np.array([[speed, 0.05], [speed, 0.4], [speed, 1.5]], np.float32)
    gs = lems.make_set(m, conn, 0.1, params, state0=x0)
    assert isinstance(gs, lems.LemsGroupSet) and set(gs.block_k.tolist()) == {k}
    gs.run(300)
    ref = lo.run(lems.lems_file(name), name, conn.row, conn.col, conn.wnz, conn.lnz, params, 0.1,
                 300, x0)
    err = circ_rel_err if name == 'Kuramoto' else rel_err
    assert err(gs.state.cpu().numpy(), ref['state']) < TOL


@pytest.mark.parametrize('name', ['Epileptor', 'Ou6'])
def test_lems_groups_chunks_bit_exact(cuda, name):
    conn = conn_of(40, seed=8)
    N = conn.nnode
    m = lems.load_model(name)
    x0 = state0_of(name, N) if name == 'Epileptor' else None
    a = lems.LemsGroupSet(m, conn, 0.1, PARAMS, state0=x0, seed=11)
    b = lems.LemsGroupSet(m, conn, 0.1, PARAMS, state0=x0, seed=11)
    a.run(300)
    for n in (1, 137, 162):
        b.run(n)
    assert np.array_equal(a.state.cpu().numpy(), b.state.cpu().numpy())
    assert np.array_equal(a.ring.cpu().numpy(), b.ring.cpu().numpy())


@pytest.mark.parametrize('name', ['Ou', 'Ou6'])
def test_lems_groups_noise_statistics(cuda, name):
    "The group kernel's noise (four and eight normals per step) by its statistics."
    conn = conn_of(200, seed=9)
    N = conn.nnode
    m = lems.load_model(name)
    params = np.array([[4.0, 0.0]] * 8, np.float32)
    gs = lems.LemsGroupSet(m, conn, 0.1, params, state0=np.zeros((N, m.ns), np.float32), seed=5)
    gs.run(2000)
    x = gs.state.cpu().numpy().reshape(-1, m.ns).astype(np.float64)
    nsig = np.sqrt(np.float32(0.1)) * np.float32(0.1)
    var = nsig ** 2 / (1 - (1 - 0.5 * 0.1) ** 2)
    n = x.shape[0]
    for v in range(m.ns):
        assert abs(x[:, v].mean()) < 5 * np.sqrt(var / n)
        assert abs(x[:, v].var() / var - 1) < 5 * np.sqrt(2.0 / n)
    if m.ns > 1:
        c = np.corrcoef(x.T)
        assert np.abs(c - np.eye(m.ns)).max() < 5 / np.sqrt(n)


def test_lems_hmje_two_inputs_matches_oracle(cuda, tmp_path):
    """tvb_hpc's HMJE (two coupled inputs: c1 from x1, c2 from x2) from its
    bundled LEMS file with the coupling constants on: one ring channel per
    input on the group kernel, against the LEMS oracle (itself pinned on
    tvb_hpc's model definition); x0, Iext, r swept per work item."""
    from test_lems import hmje_text, hmje_state0
    path = tmp_path / 'hmje_CUDA.xml'
    path.write_text(hmje_text())
    m = lems.parse(str(path), name='HMJE')
    assert m.coupling_class == 'sep2'
    conn = conn_of(60, seed=14)
    x0 = hmje_state0(conn.nnode)
    params = np.array([[3.0, 0.3, -1.6, 3.1, 0.00035], [6.0, 0.8, -2.2, 3.0, 0.001],
                       [6.0, 0.1, -1.9, 3.2, 0.0005]], np.float32)
    gs = lems.make_set(m, conn, 0.1, params, state0=x0, noise=False)
    assert isinstance(gs, lems.LemsGroupSet) and gs.channels == 2
    gs.run(400)
    ref = lo.run(str(path), 'HMJE', conn.row, conn.col, conn.wnz, conn.lnz, params, 0.1, 400, x0)
    assert rel_err(gs.state.cpu().numpy(), ref['state']) < TOL
    assert rel_err(gs.exposures().cpu().numpy(), ref['expo']) < TOL
    with pytest.raises(ValueError):          # two inputs: the group kernel only
        lems.LemsSweep(m, conn, 0.1, params, state0=x0)


@pytest.mark.parametrize('kind', ['groups', 'sweep'])
def test_lems_noise_scale_per_variable(cuda, kind):
    """noise="0" takes a state variable out of the noise: with zero initial
    state the silent variables of uncoupled OU nodes stay exactly zero
    (six variables: the wide path with its per-variable factors)."""
    text = open(lems.lems_file('Ou6')).read()
    for v in range(1, 6):
        text = text.replace('<StateVariable name="u%d" default="0" boundaries=""/>' % v,
                            '<StateVariable name="u%d" default="0" boundaries="" noise="0"/>' % v)
    m = lems.parse(text, name='Ou6')
    assert m.scales == [1, 0, 0, 0, 0, 0]
    conn = conn_of(100, seed=15)
    N = conn.nnode
    params = np.array([[4.0, 0.0]] * 8, np.float32)
    Set = lems.LemsGroupSet if kind == 'groups' else lems.LemsSweep
    sw = Set(m, conn, 0.1, params, state0=np.zeros((N, 6), np.float32), seed=3)
    sw.run(1000)
    x = sw.state.cpu().numpy().reshape(-1, 6)
    assert np.all(x[:, 1:] == 0)
    nsig = np.sqrt(np.float32(0.1)) * np.float32(0.1)
    var = nsig ** 2 / (1 - (1 - 0.5 * 0.1) ** 2)
    assert abs(x[:, 0].var() / var - 1) < 5 * np.sqrt(2.0 / x.shape[0])


def test_dsl_launcher_interface(cuda):
    """tvb_hpc.dsl.CudaRun.run_simulation with the DSL launcher's arguments
    (cuda_run.py:70-147; parameters from cuda_setup.py:88-101) runs the
    bundled Kuramoto file and returns its tavg layout."""
    import types
    from tvb_hpc import dsl
    w, ln = network.synthetic_connectome(30, 0.3, seed=6)
    couplings, speeds = dsl.setup_params(4, 2)
    params = dsl.expand_params(couplings * 1e-3, speeds * 2.0)
    args = types.SimpleNamespace(model='Kuramoto')
    tavg = dsl.CudaRun().run_simulation(w, ln, params, speeds, None, args, 30, 8, 2, 3, 40, 1024, 1,
                                        0.1, float(speeds.min()))
    assert tavg.shape == (3, 60, 8)
    conn = network.Connectivity.from_dense(w, ln)
    ref = lo.run(lems.lems_file('Kuramoto'), 'Kuramoto', conn.row, conn.col, conn.wnz, conn.lnz,
                 params, 0.1, 120)
    np.testing.assert_allclose(tavg[-1, 30:, :].T, ref['expo'][:, :, 1], atol=1e-4)
    with pytest.raises(ValueError):
        dsl.CudaRun().run_simulation(w, ln, params, speeds, None, args, 30, 8, 2, 3, 40, 1024, 2,
                                     0.1, 1.0)
