"""
Time-stepping schemes with the schema of tvb_hpc/scheme.py.

``euler``, ``euler_maruyama`` and ``euler_maruyama_logp`` build symbolic
expressions (sympy here, pymbolic in the reference, scheme.py:29-48).  The
scheme classes select the kernel's update: EulerStep is the deterministic
x + dt f (scheme.py:55-85); EulerMaryuyamaStep adds sqrt(dt) dW g
(scheme.py:88-107) where dW comes from the in-kernel Philox generator
instead of an input array (so noise is generated where it is used).
"""

from typing import Union

import numpy as np
import sympy

from .utils import parse


def euler(x, f, dt=None):
    "Construct standard Euler step."
    dt = dt if dt is not None else sympy.Symbol('dt')
    return x + dt * f


def euler_maruyama(x, f, g, dt=None, dWt=None):
    "Construct SDE Euler-Maruyama step."
    dt = dt if dt is not None else sympy.Symbol('dt')
    dWt = dWt if dWt is not None else sympy.Symbol('dWt')
    return x + dt * f + dWt * dt ** sympy.Rational(1, 2) * g


def euler_maruyama_logp(x, f, g, xn=None, dt=None, step=euler):
    "Construct normal log p."
    dt = dt if dt is not None else sympy.Symbol('dt')
    mu = step(x, f, dt)
    sd = dt ** sympy.Rational(1, 2) * g
    if xn is None:
        xn = np.array([sympy.Symbol(str(v) + '_n') for v in x], dtype=object)
    return -(xn - mu) ** 2 / (2 * sd ** 2)


class TimeStepScheme:
    noise = False


class EulerStep(TimeStepScheme):
    "Deterministic Euler step (scheme.py:55-85)."

    def __init__(self, dt: Union[str, float]):
        self.dt = dt

    def dt_value(self, kwargs=None):
        "Numeric dt: a literal, or the kernel argument named by a symbolic dt."
        if isinstance(self.dt, (int, float, np.number)):
            return float(self.dt)
        name = getattr(self.dt, 'name', str(self.dt))
        if kwargs is None or name not in kwargs:
            raise TypeError('symbolic dt %r must be passed as a kernel argument' % name)
        return float(kwargs[name])

    def kernel_isns(self):
        return ['state[i_node, i_svar] = state[i_node, i_svar] + %s * drift[i_node, i_svar]'
                % (self.dt, )]


class EulerMaryuyamaStep(EulerStep):
    "Euler-Maruyama step (scheme.py:88-107)."
    noise = True

    def kernel_isns(self):
        return ['<> sqrt_dt = sqrtf(%s)' % (self.dt, ),
                'state[i_node, i_svar] = state[i_node, i_svar] + %s*drift[i_node, i_svar] '
                '+ sqrt_dt*dWt[i_node, i_svar]*diffs[i_node, i_svar]' % (self.dt, )]


_ = parse
