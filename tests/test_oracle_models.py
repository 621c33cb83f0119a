"""
The oracle's restatement of the RWW and Jansen-Rit drifts (oracle/
tvbg_oracle_step.inc) against the model definitions of tvb_hpc/model.py:
209-247 themselves -- the attribute strings (state, auxex, drift, const) are
evaluated symbolically with sympy, so the pin does not go through any code
of this repository's kernels.  One FP64 Euler step of a node without edges
(linear coupling: c = b) must equal x + dt f(x, c, p).
"""

import numpy as np
import pytest
import sympy

import pyoracle as orc
from tvb_hpc import model
from tvb_hpc.utils import parse


def reference_drift(m):
    "sympy drift of a tvb_hpc model with its auxiliary expressions substituted."
    aux = {}
    for name, expr in m.auxex:
        aux[sympy.Symbol(name)] = parse(expr).subs(aux)
    params = {p.name for p in m.param_sym}
    consts = {sympy.Symbol(k): v for k, v in m.const.items() if k not in params}
    f = [parse(d).subs(aux).subs(consts) for d in m.drift]
    args = list(m.state_sym) + list(m.input_sym) + list(m.param_sym)
    return sympy.lambdify(args, f, 'numpy')


@pytest.mark.parametrize('name,kid', [('RWW', 5), ('JansenRit', 6)])
def test_oracle_drift_matches_model_definition(name, kid):
    m = getattr(model, name)()
    f = reference_drift(m)
    rng = np.random.default_rng(kid)
    I, ns, npar = 16, m.nsvar, len(m.param_sym)
    lim = np.array([(min(lo, hi), max(lo, hi)) for lo, hi in m.limit], float)
    x = rng.uniform(lim[:, 0], lim[:, 1], (I, 1, ns)) * 0.5
    p = np.stack([rng.uniform(0.8, 1.2, I) * m.const[s.name] for s in m.param_sym], -1)[:, None, :]
    c = rng.uniform(-0.5, 0.5, I)
    dt = 0.1
    kid2, consts, sigma = m.engine_spec()
    assert kid2 == kid
    got = np.zeros((I, ns))
    for b in range(I):   # one call per instance: the coupling offset b carries the input
        out = orc.run(kid, 0, np.array([0, 0]), np.zeros(0, np.int32), np.zeros(0, np.float32), 8,
                      1, dt, np.zeros((1, 0), np.int32), [1.0], p[b:b + 1], x[b:b + 1],
                      consts=consts, sigma=sigma, cf_b=float(c[b]), real='f64')
        got[b] = out['state'][0, 0]
    for b in range(I):
        fx = np.array(f(*x[b, 0], c[b], *p[b, 0]), float)
        dt32 = float(np.float32(dt))   # the oracle's step size is a float32
        # the kernels take the constants as float32: 1e-6 relative
        np.testing.assert_allclose(got[b], x[b, 0] + dt32 * fx, rtol=1e-6, atol=1e-9)


def test_oracle_rejects_noise_beyond_four_state_variables():
    m = model.JansenRit()
    kid, consts, sigma = m.engine_spec()
    with pytest.raises(RuntimeError):
        orc.run(kid, 0, np.array([0, 0]), np.zeros(0, np.int32), np.zeros(0, np.float32), 8, 1,
                0.1, np.zeros((1, 0), np.int32), [1.0], np.ones((1, 1, 2)), np.zeros((1, 1, 6)),
                consts=consts, sigma=sigma, flags=orc.F_NOISE, real='f64')
