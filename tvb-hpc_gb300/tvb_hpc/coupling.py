"""
Coupling functions with the schema of tvb_hpc/coupling.py.

A coupling is a pre-summation expression of (pre_syn, post_syn) and a
post-summation expression of `sum` or `mean` (mean = sum / nnode,
network.py:130-131), with parameters `param`.  The engine maps the four
reference classes to hand-written device functors; a coupling whose
expressions differ from the built-in ones is rejected by ``engine_spec``.

NB as in tvb-hpc: pre_syn are observables, not state variables, and when a
model has fewer inputs than observables the observables are truncated
(_check_io, coupling.py:68-84), so G2DO couples its first observable W.
"""

import enum
import itertools

import numpy as np

from . import _native as nat
from .model import BaseModel
from .utils import exprs, getLogger, free_names


class PostSumStat(enum.Enum):
    sum = 'sum'
    mean = 'mean'


class BaseCoupling:
    "coupling.py:42-100"

    param = {}
    pre_sum = ''
    post_sum = ''
    _kernel = None

    def __init__(self, model: BaseModel):
        self.model = model
        # per-instance copy: hackathon.py:27 edits cfun.param['a']
        self.param = dict(self.param)
        self.param_sym = np.array(list(self.param.keys()), dtype=object)
        self.pre_sum_sym = exprs(self.pre_sum)
        self.post_sum_sym = exprs(self.post_sum)
        lname = '%s<%s>' % (self.__class__.__name__, model.__class__.__name__)
        self.logger = getLogger(lname)
        self._check_io()

    def _check_io(self):
        obsrv_sym = self.model.obsrv_sym
        if self.model.input_sym.size < obsrv_sym.size:
            self.logger.debug('input shorter than obsrv, truncating obsrv used for cfun.')
            obsrv_sym = obsrv_sym[:self.model.input_sym.size]
        terms = (obsrv_sym, self.pre_sum_sym, self.post_sum_sym, self.model.input_sym)
        n = max(len(t) for t in terms)
        for t in terms:
            if len(t) not in (1, n):
                raise ValueError('shape mismatch: objects cannot be broadcast '
                                 'to a single shape (%r)' % ([len(t) for t in terms], ))
        self.io = [tuple(t[i if len(t) > 1 else 0] for t in terms) for i in range(n)]

    def post_stat(self, i: int) -> PostSumStat:
        "'mean' or 'sum' used by the i'th post-summation expression."
        names = free_names(self.post_sum_sym[i])
        if 'mean' in names:
            return PostSumStat('mean')
        if 'sum' in names:
            return PostSumStat('sum')
        raise ValueError('unknown stat in %r' % (self.post_sum, ))

    # ---- engine mapping ----------------------------------------------------
    def engine_spec(self):
        """
        (kernel id, a, b, (cmax, midpoint, r)) for the C ABI.  `a`/`b` may be
        symbolic (a name or an object with .name): then they are kernel
        arguments supplied per call, as cfun.param['a'] = pm.parse('a') in
        tvb_hpc/examples/hackathon.py:27.
        """
        cls = type(self)
        base = next((c for c in cls.__mro__ if _BUILTIN.get(c.__name__) is c), None)
        if base is None or base._kernel is None:
            raise NotImplementedError('coupling %s has no GB300 kernel' % cls.__name__)
        if (_norm(self.pre_sum) != _norm(base.pre_sum)
                or _norm(self.post_sum) != _norm(base.post_sum)):
            raise NotImplementedError('%s expressions differ from the built-in '
                                      'definition' % cls.__name__)
        if len(self.io) != 1:
            raise NotImplementedError('the engine couples one observable per model')
        p = self.param
        sig = (p.get('cmax', 0.0), p.get('midpoint', 0.0), p.get('r', 0.0))
        return base._kernel, p.get('a', 0.0), p.get('b', 0.0), sig


def _norm(v):
    if isinstance(v, str):
        return ' '.join(v.split())
    return tuple(' '.join(str(x).split()) for x in v)


def symbolic_name(v):
    "Name of a symbolic parameter value, or None for a number."
    if isinstance(v, (int, float, np.number)):
        return None
    if isinstance(v, str):
        return v
    return getattr(v, 'name', str(v))


class Linear(BaseCoupling):
    "coupling.py:103-106"
    param = {'a': 1e-3, 'b': 0}
    pre_sum = 'pre_syn',
    post_sum = 'a * sum + b',
    _kernel = nat.CFUN_LINEAR


class Sigmoidal(BaseCoupling):
    "coupling.py:109-112"
    param = {'cmin': 0, 'cmax': 0.005, 'midpoint': 6, 'r': 1, 'a': 0.56}
    pre_sum = 'cmax / (1 + exp(r * (midpoint - pre_syn)))',
    post_sum = 'a * sum',
    _kernel = nat.CFUN_SIGMOIDAL


class Diff(Linear):
    "coupling.py:115-116"
    pre_sum = 'pre_syn - post_syn',
    _kernel = nat.CFUN_DIFF


class Kuramoto(Diff):
    "coupling.py:119-121"
    pre_sum = 'sin(pre_syn - post_syn)',
    post_sum = 'a * mean',
    _kernel = nat.CFUN_KURAMOTO


_BUILTIN = {'Linear': Linear, 'Sigmoidal': Sigmoidal, 'Diff': Diff, 'Kuramoto': Kuramoto}
_ = itertools
