"""
Neural-mass models with the class-attribute schema of tvb_hpc/model.py.

A model is described by attribute strings (state, input, param, drift,
diffs, obsrv, const, auxex, limit), exactly as in tvb-hpc.  The GB300 engine
does not generate code from them: each supported class maps to a
hand-written device functor (tvb-hpc_gb300/csrc/tvbg_device.cuh).  A model
whose drift/obsrv strings differ from the built-in definition is rejected
by ``engine_spec`` rather than silently run with the wrong equations.
"""

from typing import List

import numpy as np

from . import _native as nat
from .utils import exprs, vars, simplify, parse


class BaseModel:
    """
    BaseModel parses attributes on subclasses, defining a networked SDE
    (tvb_hpc/model.py:31-155).
    """

    dt = 1e-3
    state = ''
    input = ''
    param = ''
    drift = '',
    diffs = '',
    obsrv = '',
    const = {}
    auxex = []
    limit = []

    #: engine description: kernel id, const order, param names
    _kernel = None
    _kernel_consts = ()

    def __init__(self):
        # instance copy so per-instance edits (osc.const['omega'] = ...) do
        # not leak into the class, as the reference's mutation would
        self.const = dict(self.const)
        self.state_sym = vars(self.state)
        self.input_sym = vars(self.input)
        self.param_sym = vars(self.param)
        self.drift_sym = exprs(self.drift)
        self.diffs_sym = exprs(self.diffs)
        self.obsrv_sym = exprs(self.obsrv)

    @property
    def indvars(self):
        return np.r_[self.state_sym, self.input_sym, self.param_sym]

    def partial(self, expr):
        "Partial derivatives of expr w.r.t. indvars (model.py:61-65)."
        e = parse(expr)
        return np.array([simplify(e.diff(v)) for v in self.indvars], dtype=object)

    def prep_arrays(self, nnode: int) -> List[np.ndarray]:
        """
        Prepare state, input, param, drift, diffs, obsrv arrays
        (model.py:67-84): state drawn uniformly inside `limit`, params from
        `const`.
        """
        dtype = np.float32
        arrs: List[np.ndarray] = []
        for key in 'state input param drift diffs obsrv'.split():
            shape = nnode, len(getattr(self, key + '_sym'))
            arrs.append(np.zeros(shape, dtype))
        state = arrs[0]
        for i, (lo, hi) in enumerate(self.limit):
            state[:, i] = np.random.uniform(float(lo), float(hi), size=(nnode, ))
        param = arrs[2]
        for i, psym in enumerate(self.param_sym):
            param[:, i] = self.const[psym.name]
        return arrs

    # ---- engine mapping ----------------------------------------------------
    @property
    def nsvar(self):
        return len(self.state_sym)

    @property
    def nobs(self):
        return len(self.obsrv_sym)

    def engine_spec(self):
        """
        (kernel id, constants vector[16], noise sigma[4]) for the C ABI.
        Raises NotImplementedError for a model without a hand-written kernel
        or whose equations were edited.
        """
        cls = type(self)
        base = next((c for c in cls.__mro__ if _BUILTIN.get(c.__name__) is c), None)
        if base is None or self._kernel is None:
            raise NotImplementedError(
                'model %s has no GB300 kernel (built: %s)' % (
                    cls.__name__, ', '.join(sorted(_BUILTIN))))
        for key in ('state', 'drift', 'obsrv', 'param', 'input'):
            if _norm(getattr(self, key)) != _norm(getattr(base, key)):
                raise NotImplementedError(
                    '%s.%s differs from the built-in definition; the engine '
                    'runs hand-written kernels only' % (cls.__name__, key))
        consts = np.zeros(16, np.float32)
        for i, name in enumerate(self._kernel_consts):
            consts[i] = float(self.const[name])
        sig = np.zeros(max(4, len(self.diffs)), np.float32)
        for i, g in enumerate(self.diffs):
            sig[i] = float(parse(g).subs({k: v for k, v in self.const.items()}))
        if self.nsvar > 4 and np.any(sig != 0):
            raise NotImplementedError('noise on more than 4 state variables is not built')
        return self._kernel, consts, sig[:4].copy()

    def node_params(self, nnode):
        "Per-node parameter array [nnode, npar] from const (prep_arrays)."
        p = np.zeros((nnode, len(self.param_sym)), np.float32)
        for i, psym in enumerate(self.param_sym):
            p[:, i] = self.const[psym.name]
        return p


def _norm(v):
    if isinstance(v, str):
        return ' '.join(v.split())
    return tuple(' '.join(str(x).split()) for x in v)


class _TestModel(BaseModel):
    state = 'y1 y2'
    input = 'i1'
    param = 'a b c'
    auxex = [('y1_3', 'y1 * y1 * y1')]
    drift = '(y1 - y1_3/3 + y2 + e)*b', '(a - y1 + i1 + d)/b'
    diffs = 'c', 'c'
    obsrv = 'y1',
    const = {'d': 3.0, 'e': -12.23904e-2, 'a': 1.05, 'b': 3.0, 'c': 1e-5}
    limit = (-1, 1), (-1, 1)


class Kuramoto(BaseModel):
    "Kuramoto model of phase synchronization (model.py:169-182)."
    state = 'theta'
    limit = (0, 2 * np.pi),
    input = 'I'
    param = 'omega'
    drift = 'omega + I',
    diffs = 0,
    obsrv = 'theta', 'sin(theta)'
    const = {'omega': 1.0}
    _kernel = nat.MODEL_KURAMOTO
    _kernel_consts = ()


class HMJE(BaseModel):
    """Hindmarsh-Rose-Jirsa Epileptor model of seizure dynamics (model.py:185-206).

    Its two coupled inputs (c1 from x1, c2 from x2) run on the engine
    through the bundled LEMS file of this model (`HMJE.lems()`, i.e.
    tvb_hpc.lems.load_model('HMJE'): one ring channel per input on the
    group kernel); engine_spec() has no hand-written kernel for it."""

    @staticmethod
    def lems():
        "The bundled LEMS model of HMJE (two coupled inputs, x0/Iext/r per work item)."
        from . import lems
        return lems.load_model('HMJE')
    state = 'x1 y1 z x2 y2 g'
    limit = (-2, 1), (20, 2), (2, 5), (-2, 0), (0, 2), (-1, 1)
    input = 'c1 c2'
    param = 'x0 Iext r'
    drift = (
        'tt * (y1 - z + Iext + Kvf * c1 + ('
        '  (x1 <  0)*(-a * x1 * x1 + b * x1)'
        '+ (x1 >= 0)*(slope - x2 + 0.6 * (z - 4)**2)'
        ') * x1)',
        'tt * (c - d * x1 * x1 - y1)',
        'tt * (r * (4 * (x1 - x0) - z +  Ks * c1))',
        'tt * (-y2 + x2 - x2*x2*x2 + Iext2 + 2 * g - 0.3 * (z - 3.5) + Kf * c2)',
        'tt * ((-y2 + (x2 >= (-0.25)) * (aa * (x2 + 0.25))) / tau)',
        'tt * (-0.01 * (g - 0.1 * x1))'
    )
    diffs = 0, 0, 0, 0.0003, 0.0003, 0
    obsrv = 'x1', 'x2', 'z', '-x1 + x2'
    const = {'Iext2': 0.45, 'a': 1.0, 'b': 3.0, 'slope': 0.0, 'tt': 1.0, 'c':
             1.0, 'd': 5.0, 'Kvf': 0.0, 'Ks': 0.0, 'Kf': 0.0, 'aa': 6.0, 'tau':
             10.0, 'x0': -1.6, 'Iext': 3.1, 'r': 0.00035}

    def __init__(self):
        # pymbolic comparisons in the drift have no sympy string form; keep
        # the attribute schema but skip parsing of the drift.
        self.const = dict(self.const)
        self.state_sym = vars(self.state)
        self.input_sym = vars(self.input)
        self.param_sym = vars(self.param)
        self.drift_sym = np.array(list(self.drift), dtype=object)
        self.diffs_sym = exprs(self.diffs)
        self.obsrv_sym = exprs(self.obsrv)


class RWW(BaseModel):
    "Reduced Wong-Wang firing rate model (model.py:209-223)."
    state = 'S'
    limit = (0, 1),
    input = 'c'
    param = 'w io'
    const = {'a': 0.270, 'b': 0.108, 'd': 154.0, 'g': 0.641,
             'ts': 100.0, 'J': 0.2609, 'w': 0.6, 'io': 0.33}
    auxex = [
        ('x', 'w * J * S + io + J * c'),
        ('h', '(a * x - b) / (1 - exp(-d*(a*x - b)))')
    ]
    drift = '- (S / ts) + (1 - S) * h * g',
    diffs = 0.01,
    obsrv = 'S',
    _kernel = nat.MODEL_RWW
    _kernel_consts = ('a', 'b', 'd', 'g', 'ts', 'J')


class JansenRit(BaseModel):
    "Jansen-Rit model of visual evoked potentials (model.py:226-247)."
    state = 'y0 y1 y2 y3 y4 y5'
    limit = (-1, 1), (-500, 500), (-50, 50), (-6, 6), (-20, 20), (-500, 500)
    const = {'A': 3.25, 'B': 22.0, 'a': 0.1, 'b': 0.05, 'v0': 5.52,
             'nu_max': 0.0025, 'r': 0.56, 'J': 135.0, 'a_1': 1.0, 'a_2': 0.8,
             'a_3': 0.25, 'a_4': 0.25, 'mu': 0.22}
    input = 'lrc'
    param = 'v0 r'
    auxex = [
        ('sigm_y1_y2', '2 * nu_max / (1 + exp(r * (v0 - (y1 - y2))))'),
        ('sigm_y0_1', '2 * nu_max / (1 + exp(r * (v0 - (a_1 * J * y0))))'),
        ('sigm_y0_3', '2 * nu_max / (1 + exp(r * (v0 - (a_3 * J * y0))))'),
    ]
    drift = (
        'y3', 'y4', 'y5',
        'A * a * sigm_y1_y2 - 2 * a * y3 - a**2 * y0',
        'A * a * (mu + a_2 * J * sigm_y0_1 + lrc) - 2 * a * y4 - a**2 * y1',
        'B * b * (a_4 * J * sigm_y0_3) - 2 * b * y5 - b**2 * y2'
    )
    diffs = 0, 0, 0, 0, 0, 0
    obsrv = 'y0 - y1',
    _kernel = nat.MODEL_JANSENRIT
    _kernel_consts = ('A', 'B', 'a', 'b', 'nu_max', 'J', 'a_1', 'a_2', 'a_3', 'a_4', 'mu')


class Linear(BaseModel):
    "Linear differential equation (model.py:250-259)."
    state = 'x'
    limit = (-10, 10),
    input = 'c'
    param = 'lam'
    const = {'lam': -1}
    drift = 'lam * x + c',
    diffs = 1e-2,
    obsrv = 'x',
    _kernel = nat.MODEL_LINEAR
    _kernel_consts = ()


class G2DO(BaseModel):
    "Generic nonlinear 2-D (phase plane) oscillator (model.py:262-276)."
    state = 'W V'
    limit = (-5, 5), (-5, 5)
    input = 'c_0'
    param = 'a'
    const = {'tau': 1.0, 'I': 0.0, 'a': -2.0, 'b': -10.0, 'c': 0.0, 'd': 0.02,
             'e': 3.0, 'f': 1.0, 'g': 0.0, 'alpha': 1.0, 'beta': 1.0,
             'gamma': 1.0}
    drift = (
        'd * tau * (alpha*W - f*V**3 + e*V**2 + g*V + gamma*I + gamma*c_0)',
        'd * (a + b*V + c*V**2 - beta*W) / tau'
    )
    diffs = 1e-3, 1e-3
    obsrv = 'W', 'V'
    _kernel = nat.MODEL_G2DO
    _kernel_consts = ('tau', 'I', 'b', 'c', 'd', 'e', 'f', 'g', 'alpha', 'beta', 'gamma')


class Generic2dOscillator(BaseModel):
    """
    Generic 2-D oscillator in the form of the CUDA DSL kernel
    (dsl/dsl_cuda/CUDAmodels/oscillator.c:149-150) and of TVB: the cubic and
    the coupling act on V.  tvb_hpc's G2DO (model.py:262-276) attaches that
    equation to W instead; with the default constants its fixed point is a
    saddle and trajectories diverge within ~10^4 steps of 0.1 ms, so the
    benchmark's "2D generic oscillator" uses this form.
    """
    state = 'V W'
    limit = (-2, 4), (-6, 6)
    input = 'c_0'
    param = 'a'
    const = dict(G2DO.const)
    drift = (
        'd * tau * (alpha*W - f*V**3 + e*V**2 + g*V + gamma*I + gamma*c_0)',
        'd * (a + b*V + c*V**2 - beta*W) / tau'
    )
    diffs = 1e-3, 1e-3
    obsrv = 'V', 'W'
    _kernel = nat.MODEL_G2DOSC
    _kernel_consts = G2DO._kernel_consts


class MPR(BaseModel):
    """
    Montbrio-Pazo-Roxin (2015) mean-field model of quadratic integrate-and-
    fire neurons: r' = (Delta/(pi tau) + 2 r V)/tau,
    V' = (V^2 + eta + J tau r + I + c - (pi tau r)^2)/tau, coupling on r.
    tvb-hpc names this model only in dsl/dsl_cuda/example/cuda_setup.py:156;
    it is added here with the attribute schema of model.py.  The rate is
    clamped at zero after each step.
    """
    state = 'r V'
    limit = (0, 3), (-2, 2)
    input = 'c'
    param = 'eta'
    const = {'Delta': 1.0, 'J': 15.0, 'tau': 1.0, 'I': 0.0, 'eta': -5.0}
    drift = (
        '(Delta / (pi * tau) + 2 * r * V) / tau',
        '(V**2 + eta + J * tau * r + I + c - (pi * tau * r)**2) / tau'
    )
    diffs = 1e-2, 1e-2
    obsrv = 'r', 'V'
    _kernel = nat.MODEL_MPR
    _kernel_consts = ('Delta', 'J', 'tau', 'I')


_BUILTIN = {'Kuramoto': Kuramoto, 'G2DO': G2DO, 'MPR': MPR, 'Linear': Linear,
            'Generic2dOscillator': Generic2dOscillator, 'RWW': RWW, 'JansenRit': JansenRit}
