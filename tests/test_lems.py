"""
The LEMS-XML front-end without a GPU: the oracle's C-expression evaluator
against known C answers, the front-end's reading of every model file
(bundled, and the reference's dsl/dsl_cuda/XMLmodels when that tree is
present) against the oracle's independent reading, the generated host
code's derived parameters against the oracle bit for bit, and the LEMS
oracle pinned on the main oracle through the bundled Kuramoto, 2-D
oscillator and reduced Wong-Wang files (tvbg_oracle.c restates those models
from tvb_hpc).
"""

import math
import os

import numpy as np
import pytest

import lems_oracle as lo
import pyoracle as orc
from tvb_hpc import lems, network, model

# the reference's own model files, read where TVB_HPC_REFERENCE names a tvb-hpc checkout
REF_XML = os.path.join(os.environ.get('TVB_HPC_REFERENCE', '') or '/nonexistent',
                       'dsl', 'dsl_cuda', 'XMLmodels')
BUNDLED = ['Kuramoto', 'Oscillator', 'Rwongwang', 'Epileptor', 'Ou', 'Ou6', 'HMJE']
REFERENCE = ['Kuramoto', 'Oscillator', 'Rwongwang', 'Epileptor']


def ev(s, **env):
    return lo.ceval(s, env)


def test_c_expression_semantics():
    n = np.uint32(68)
    assert ev('1 / n_node', n_node=n) == 0 and ev('1 / n_node', n_node=n).dtype == np.uint32
    v = ev('1.0f / n_node', n_node=n)
    assert v.dtype == np.float32 and v == np.float32(1) / np.float32(68)
    assert ev('2.0 * 1e-5').dtype == np.float64
    dt = np.float32(0.1)
    assert ev('sqrt(dt)', dt=dt).dtype == np.float32
    assert ev('sqrt(2.0)', ).dtype == np.float64
    assert ev('powf(x, 3)', x=np.float32(2)) == 8 and ev('powf(x, 3)', x=np.float32(2)).dtype == np.float32
    assert ev('1 + 2 * 3 - 4 / 3') == 6
    assert ev('-7 / 2') == -3                      # C truncates toward zero
    assert ev('(float) 7 / 2') == 3.5
    assert ev('x < 0.0 && y >= 1', x=np.float32(-1), y=np.int32(1)) == 1
    assert ev('x < 0.0 || y > 1', x=np.float32(1), y=np.int32(1)) == 0
    assert ev('3.f').dtype == np.float32 and ev('.5').dtype == np.float64
    assert ev('M_PI_F') == np.float32(math.pi)
    with pytest.raises(ValueError):
        ev('nope + 1')


@pytest.mark.parametrize('name', BUNDLED)
def test_bundled_files_read_alike(name):
    m = lems.load_model(name)
    o = lo.read_model(lems.lems_file(name), name)
    assert m.params == o['params']
    assert [n for n, _ in m.derived_params] == list(o['derived'])
    assert m.states == o['states']
    assert len(m.time_derivs) == len(o['tders']) == m.ns
    assert m.noise == o['noise']
    src = lems.render_cuda(m)
    assert 'struct LemsModel' in src and 'tvbg_lems_sweep' in src


@pytest.mark.skipif(not os.path.isdir(REF_XML), reason='reference tree absent')
@pytest.mark.parametrize('name', REFERENCE)
def test_reference_files_parse_and_render(name):
    "The DSL's own model set is accepted by the front-end."
    m = lems.load_model(name, REF_XML)
    o = lo.read_model(lems.lems_file(name, REF_XML), name)
    assert m.params == o['params'] == ['global_speed', 'global_coupling']
    assert m.states == o['states']
    assert m.noise
    for single in (False, True):
        assert 'struct LemsModel' in lems.render_cuda(m, single)


def test_coupling_classes():
    "Which couplings the group kernel takes: separable or a sine difference."
    got = {n: lems.load_model(n).coupling_class for n in BUNDLED}
    assert got == {'Kuramoto': 'sc', 'Oscillator': 'sc', 'Epileptor': 'sc', 'Rwongwang': 'sep',
                   'Ou': 'sep', 'Ou6': 'sep', 'HMJE': 'sep2'}
    h = lems.load_model('HMJE')
    assert (h.cvar, h.cvar2) == (0, 3) and h.scales == [0, 0, 0, 1, 1, 0]
    base = open(lems.lems_file('Ou')).read()
    m = lems.parse(base.replace('expression="x_j"', 'expression="tanh(x_j - x)"'))
    assert m.coupling_class == 'edge'
    m = lems.parse(base.replace('expression="x_j"', 'expression="sinf(x_j - x)"'))
    assert m.coupling_class == 'sc'
    if os.path.isdir(REF_XML):
        ref = {n: lems.load_model(n, REF_XML).coupling_class for n in REFERENCE}
        assert ref == {'Kuramoto': 'sc', 'Oscillator': 'sc', 'Epileptor': 'sc', 'Rwongwang': 'sep'}


def test_to_single_and_names():
    assert lems.to_single('2.0 * x + 1e-5 - 3 + 4.0f') == '2.0f * x + 1e-5f - 3 + 4.0f'
    assert lems.names_in('powf(V, 3) + (float) a * sin(b_j)') == ['V', 'a', 'b_j']
    with pytest.raises(ValueError):
        lems.names_in('system(1)')


def test_front_end_rejects():
    base = open(lems.lems_file('Ou')).read()
    with pytest.raises(ValueError):        # an unknown name
        lems.parse(base.replace('-k * x + c_0', '-k * x + nope'))
    with pytest.raises(NotImplementedError):   # pre reads another state of node i
        lems.parse(base.replace('<StateVariable name="x" default="0" boundaries=""/>',
                                '<StateVariable name="x" default="0" boundaries=""/>'
                                '<StateVariable name="y" default="0" boundaries=""/>')
                   .replace('<TimeDerivative name="dx" expression="-k * x + c_0"/>',
                            '<TimeDerivative name="dx" expression="-k * x + c_0"/>'
                            '<TimeDerivative name="dy" expression="-y"/>')
                   .replace('expression="x_j"', 'expression="x_j - y"'))
    with pytest.raises(ValueError):        # noise on without nsig
        lems.parse(base.replace('<DerivedParameter name="nsig" expression="sqrtf(dt) * 0.1f"/>', ''))


def _libs_and_models():
    out = [('bundled', n, lems.load_model(n), lems.lems_file(n)) for n in ('Kuramoto', 'Epileptor')]
    if os.path.isdir(REF_XML):
        out += [('reference', n, lems.load_model(n, REF_XML), lems.lems_file(n, REF_XML))
                for n in ('Kuramoto', 'Rwongwang')]
    return out


def test_generated_host_derived_parameters_bit_exact():
    """tvbg_lems_derived (host C++ compiled by nvcc) against the oracle's
    evaluation: the same float32 slots, bit for bit."""
    params = np.array([[1.0, 0.01], [4.5, 0.3], [20.0, 2.0]], np.float32)
    for kind, n, m, path in _libs_and_models():
        L = lems.LemsLibrary(m)
        got = L.derived(params, 0.1, 68)
        o = lo.read_model(path, n)
        for b in range(params.shape[0]):
            _, slots = lo.derived_params(o, params[b], 0.1, 68)
            np.testing.assert_array_equal(got[b, :slots.size], slots, err_msg='%s %s' % (kind, n))
            assert np.all(got[b, slots.size:] == 0)
        assert L.info['ns'] == m.ns and L.info['nparams'] == 2
        assert L.info['group'] == {'sep': 1, 'sc': 2, 'edge': 0}[m.coupling_class]


def _conn(N=24, seed=3):
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    return network.Connectivity.from_dense(w, ln)


def _lems_run(name, conn, params, steps, state0):
    return lo.run(lems.lems_file(name), name, conn.row, conn.col, conn.wnz, conn.lnz, params, 0.1,
                  steps, state0)


def test_oracle_kuramoto_pinned_on_main_oracle():
    conn = _conn()
    N = conn.nnode
    rng = np.random.default_rng(0)
    th0 = rng.uniform(0, 2 * np.pi, (N, 1)).astype(np.float32)
    params = np.array([[2.0, 0.5], [6.0, 3.0]], np.float32)
    got = _lems_run('Kuramoto', conn, params, 200, th0)
    omega = lo.ceval('2.0 * M_PI_F * 0.01', {}).astype(np.float32)
    for b in range(2):
        d = network.delays_f32(conn.lnz, params[b, 0], 0.1, 'dsl')
        np.testing.assert_array_equal(d, got['delays'][b])
        nh = 1 << int(np.ceil(np.log2(d.max() + 2)))
        ref = orc.run(0, 2, conn.row, conn.col, conn.wnz, nh, 200, 0.1, d[None], [params[b, 1]],
                      np.full((1, N, 1), omega, np.float32), th0[None], flags=orc.F_WRAP_FMOD)
        diff = np.angle(np.exp(1j * (got['state'][b].astype(np.float64) - ref['state'][0])))
        assert np.abs(diff).max() < 1e-4
    # exposures: theta and sin(theta)
    np.testing.assert_array_equal(got['expo'][..., 0], got['state'][..., 0])
    np.testing.assert_allclose(got['expo'][..., 1], np.sin(got['state'][..., 0]), atol=1e-6)


def test_oracle_oscillator_pinned_on_main_oracle():
    conn = _conn(seed=5)
    N = conn.nnode
    rng = np.random.default_rng(1)
    x0 = rng.uniform(-0.5, 0.5, (N, 2)).astype(np.float32)
    params = np.array([[3.0, 0.2]], np.float32)
    got = _lems_run('Oscillator', conn, params, 300, x0)
    m = model.Generic2dOscillator()
    kid, consts, _ = m.engine_spec()
    d = network.delays_f32(conn.lnz, 3.0, 0.1, 'dsl')
    nh = 1 << int(np.ceil(np.log2(d.max() + 2)))
    ref = orc.run(kid, 2, conn.row, conn.col, conn.wnz, nh, 300, 0.1, d[None], [0.2],
                  m.node_params(N)[None], x0[None], consts=consts)
    err = np.abs(got['state'][0] - ref['state'][0]).max() / np.abs(ref['state'][0]).max()
    assert err < 1e-4


def test_oracle_rww_zero_delay_pinned_on_main_oracle():
    conn = _conn(seed=7)
    N = conn.nnode
    rng = np.random.default_rng(2)
    x0 = rng.uniform(0.1, 0.4, (N, 1)).astype(np.float32)
    params = np.array([[1.0, 0.1]], np.float32)
    got = _lems_run('Rwongwang', conn, params, 300, x0)
    assert np.all(got['delays'][0] == 0)
    m = model.RWW()
    kid, consts, _ = m.engine_spec()
    ref = orc.run(kid, 0, conn.row, conn.col, conn.wnz, 4, 300, 0.1, np.zeros((1, conn.nnz)), [0.1],
                  m.node_params(N)[None], x0[None], consts=consts)
    err = np.abs(got['state'][0] - ref['state'][0]).max() / np.abs(ref['state'][0]).max()
    assert err < 1e-4


HMJE_COUPLED = {'Kvf': '0.05f', 'Ks': '-0.1f', 'Kf': '0.02f'}


def hmje_text(consts=HMJE_COUPLED):
    "The bundled HMJE file with the coupling constants switched on."
    t = open(lems.lems_file('HMJE')).read()
    for k, v in consts.items():
        t = t.replace('<Constant name="%s" default="0.0f"/>' % k,
                      '<Constant name="%s" default="%s"/>' % (k, v))
    return t


def hmje_by_tvb_hpc(conn, x0, params, steps, dt=0.1, consts=HMJE_COUPLED):
    """The HMJE step from tvb_hpc's own model definition (model.HMJE's drift
    strings, model.py:185-206, evaluated with numpy in float32) with linear
    coupling on its two inputs c1 <- x1, c2 <- x2 (coupling.py:68-84,103-112)."""
    m = model.HMJE()
    const = {k: np.float32(v) for k, v in m.const.items()}
    const.update({k: np.float32(float(v.rstrip('f'))) for k, v in consts.items()})
    G, x0p, Iext, r = (np.float32(v) for v in params[1:5])
    const.update(x0=x0p, Iext=Iext, r=r)
    d = network.delays_f32(conn.lnz, params[0], dt, 'dsl').astype(np.int64)
    row, col, w = np.asarray(conn.row), np.asarray(conn.col), np.asarray(conn.wnz, np.float32)
    N = row.size - 1
    nz = np.diff(row) > 0
    x = np.array(x0, np.float32)
    hist = np.zeros((steps + 1, N, 6), np.float32)
    hist[0] = x
    names = [str(s) for s in m.state_sym]
    for t in range(steps):
        src = t - d
        env = dict(const)
        for k, (inp, var) in enumerate((('c1', 0), ('c2', 3))):
            xj = np.where(src >= 0, hist[np.maximum(src, 0), col, var], np.float32(0))
            S = np.zeros(N, np.float32)
            S[nz] = np.add.reduceat((w * xj).astype(np.float32), row[:-1][nz])
            env[inp] = (G * S).astype(np.float32)
        for v, n in enumerate(names):
            env[n] = x[:, v]
        f = [np.asarray(eval(e, {}, env), np.float32) for e in m.drift]
        x = np.stack([(x[:, v] + np.float32(dt) * f[v]).astype(np.float32) for v in range(6)], -1)
        hist[t + 1] = x
    return x


def hmje_state0(N, seed=0):
    rng = np.random.default_rng(seed)
    x = np.zeros((N, 6), np.float32)
    for v, (lo, hi) in enumerate([(-1.8, -1.2), (-15, -12), (2.8, 3.2), (-1.2, -0.8), (0, 0.2),
                                  (-0.1, 0.1)]):
        x[:, v] = rng.uniform(lo, hi, N)
    return x


def test_oracle_hmje_pinned_on_tvb_hpc_model(tmp_path):
    """The bundled HMJE file, stepped by the LEMS oracle, against tvb_hpc's
    own HMJE definition with its two coupled inputs."""
    path = tmp_path / 'hmje_CUDA.xml'
    path.write_text(hmje_text())
    conn = _conn(N=30, seed=11)
    x0 = hmje_state0(conn.nnode)
    params = np.array([[3.0, 0.3, -1.6, 3.1, 0.00035], [6.0, 0.8, -2.2, 3.0, 0.001]], np.float32)
    got = lo.run(str(path), 'HMJE', conn.row, conn.col, conn.wnz, conn.lnz, params, 0.1, 300, x0)
    for b in range(params.shape[0]):
        ref = hmje_by_tvb_hpc(conn, x0, params[b], 300)
        err = np.abs(got['state'][b] - ref).max() / np.abs(ref).max()
        assert err < 1e-5, err
    np.testing.assert_allclose(got['expo'][..., 3], got['state'][..., 3] - got['state'][..., 0],
                               rtol=1e-6, atol=1e-6)


def test_generated_library_exports_every_declared_symbol():
    "Every entry point include/tvbg_lems.h declares is exported by a generated library."
    import re
    import subprocess
    text = open(os.path.join(os.path.dirname(lems.INCLUDE), 'include', 'tvbg_lems.h')).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    syms = sorted(set(re.findall(r'\b(tvbg_lems_[a-z0-9_]+)\s*\(', text)))
    assert len(syms) >= 8
    L = lems.LemsLibrary(lems.load_model('Ou'))
    out = subprocess.run(['nm', '-D', '--defined-only', L.path], capture_output=True, text=True,
                         check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if ' T ' in line)
    assert not [s for s in syms if s not in exported]
    assert set(lems.SIGNATURES) == set(syms)
    # nothing else leaks out of the generated library
    assert not [s for s in exported if s.startswith('tvbg') and s not in syms]
