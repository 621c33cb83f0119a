"""
CPU oracle for LEMS-XML models: a numpy restatement of the step that
dsl/dsl_cuda/tmpl8_CUDA.py:42-263 generates from a model file
(dsl/dsl_cuda/LEMS2CUDA.py:37-86 feeds it), for checking the engine's
generated kernels.

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the engine.

Independent of the engine's front-end: its own reading of the XML and its
own evaluator of the C expressions the files hold, with C's usual
arithmetic conversions (int -> unsigned -> float -> double; unsuffixed
floating literals are double, `f`-suffixed ones float; integer division
truncates) and C++/CUDA overload rules for the math functions (an
`f`-suffixed function computes in float; an unsuffixed one in float when
every argument is float, else in double).

Step (tmpl8_CUDA.py:145-243), per work item, node i, step t:
    S_i  = sum over in-edges e of w_e * post * pre(x_j[dim](t - d_e), x_i[dim](t)),
           one sum per coupling component with dynamics (the front-end takes two)
    c_k  = S_i of its component (0 for a coupling without dynamics), then c_k *= expr
    derived variables, conditional derived variables, in file order
    x_v  = float(x_v + dt * f_v)         all f_v from the state at t
    wrap ("PI": fmod to [0, 2 pi)) or clamp (lo, hi)
    history[t + 1] = x
d_e = (unsigned)(length_e * rec_speed_dt) in float32; no rec_speed_dt or
"0" means zero delays; history before t0 is zero, slot t0 holds x[dim].
Noise is not restated (its statistics are tested instead).

Parity: pinned on the engine's hand-written models (Kuramoto, the 2-D
oscillator, reduced Wong-Wang) written as LEMS files, whose steps the main
oracle (tvbg_oracle.c) restates from tvb_hpc; the reference's own LEMS
files are read and their derived parameters evaluated here for the
front-end checks.  No golden vectors of the reference's generated kernels
exist (they need pycuda and curand noise is always on).
"""

import math
import xml.etree.ElementTree as ET

import numpy as np

F32, F64, I32, U32 = np.float32, np.float64, np.int32, np.uint32
_RANK = {I32: 0, U32: 1, F32: 2, F64: 3}


# ---------------------------------------------------------------------------
# C expression evaluator
# ---------------------------------------------------------------------------
def _lex(s):
    out, i = [], 0
    while i < len(s):
        c = s[i]
        if c.isspace():
            i += 1
            continue
        if c.isdigit() or (c == '.' and i + 1 < len(s) and s[i + 1].isdigit()):
            j = i
            while j < len(s) and (s[j].isdigit() or s[j] == '.'):
                j += 1
            if j < len(s) and s[j] in 'eE':
                j += 1
                if s[j] in '+-':
                    j += 1
                while j < len(s) and s[j].isdigit():
                    j += 1
            body = s[i:j]
            suf = ''
            while j < len(s) and s[j] in 'fFuUlL':
                suf += s[j].lower()
                j += 1
            if 'f' in suf:
                out.append(('num', F32(float(body))))
            elif '.' in body or 'e' in body.lower():
                out.append(('num', F64(float(body))))
            elif 'u' in suf:
                out.append(('num', U32(int(body))))
            else:
                out.append(('num', I32(int(body))))
            i = j
            continue
        if c.isalpha() or c == '_':
            j = i
            while j < len(s) and (s[j].isalnum() or s[j] == '_'):
                j += 1
            out.append(('id', s[i:j]))
            i = j
            continue
        if s[i:i + 2] in ('<=', '>=', '==', '!=', '&&', '||'):
            out.append(('op', s[i:i + 2]))
            i += 2
            continue
        out.append(('op', c))
        i += 1
    out.append(('end', None))
    return out


def _dt(v):
    return np.asarray(v).dtype.type


def _common(a, b):
    ta, tb = _dt(a), _dt(b)
    for t in (ta, tb):
        if t not in _RANK:
            raise TypeError('unexpected type %r' % t)
    return ta if _RANK[ta] >= _RANK[tb] else tb


def _cast(v, t):
    return np.asarray(v).astype(t)


_UNARY = {
    'sin': np.sin, 'cos': np.cos, 'tan': np.tan, 'asin': np.arcsin, 'acos': np.arccos,
    'atan': np.arctan, 'sinh': np.sinh, 'cosh': np.cosh, 'tanh': np.tanh, 'exp': np.exp,
    'exp2': np.exp2, 'expm1': np.expm1, 'log': np.log, 'log2': np.log2, 'log10': np.log10,
    'log1p': np.log1p, 'sqrt': np.sqrt, 'cbrt': np.cbrt, 'fabs': np.abs, 'floor': np.floor,
    'ceil': np.ceil,
}
_BINARY = {'pow': np.power, 'atan2': np.arctan2, 'fmin': np.fmin, 'fmax': np.fmax,
           'fmod': np.fmod}


def _call(name, args):
    base = name[:-1] if (name.endswith('f') and (name[:-1] in _UNARY or name[:-1] in _BINARY)) \
        else name
    fn = _UNARY.get(base) or _BINARY.get(base)
    if fn is None:
        raise ValueError('function %r' % name)
    if base != name:
        t = F32
    else:
        kinds = {_dt(a) for a in args}
        t = F64 if F64 in kinds or kinds <= {I32, U32} else F32
    with np.errstate(all='ignore'):
        return fn(*[_cast(a, t) for a in args]).astype(t)


class _Parser:
    "Precedence climbing over C expression tokens; values are numpy arrays."

    LEVELS = [('||', ), ('&&', ), ('==', '!='), ('<', '<=', '>', '>='), ('+', '-'),
              ('*', '/', '%')]

    def __init__(self, text, env):
        self.tk = _lex(text)
        self.i = 0
        self.env = env
        self.text = text

    def peek(self):
        return self.tk[self.i]

    def take(self, want=None):
        t = self.tk[self.i]
        if want is not None and t != want:
            raise ValueError('expected %r in %r' % (want, self.text))
        self.i += 1
        return t

    def parse(self):
        v = self.binary(0)
        if self.peek()[0] != 'end':
            raise ValueError('trailing tokens in %r' % self.text)
        return v

    def binary(self, lvl):
        if lvl == len(self.LEVELS):
            return self.unary()
        v = self.binary(lvl + 1)
        while self.peek()[0] == 'op' and self.peek()[1] in self.LEVELS[lvl]:
            op = self.take()[1]
            r = self.binary(lvl + 1)
            v = self.apply(op, v, r)
        return v

    @staticmethod
    def apply(op, a, b):
        with np.errstate(all='ignore'):
            if op in ('&&', '||'):
                x, y = np.asarray(a) != 0, np.asarray(b) != 0
                return (x & y if op == '&&' else x | y).astype(I32)
            t = _common(a, b)
            x, y = _cast(a, t), _cast(b, t)
            if op in ('<', '<=', '>', '>=', '==', '!='):
                f = {'<': np.less, '<=': np.less_equal, '>': np.greater,
                     '>=': np.greater_equal, '==': np.equal, '!=': np.not_equal}[op]
                return f(x, y).astype(I32)
            if op == '+':
                return (x + y).astype(t)
            if op == '-':
                return (x - y).astype(t)
            if op == '*':
                return (x * y).astype(t)
            if op == '/':
                if t in (I32, U32):
                    q = np.abs(x.astype(np.int64)) // np.abs(y.astype(np.int64))
                    return (q * np.sign(x.astype(np.int64)) * np.sign(y.astype(np.int64))).astype(t)
                return (x / y).astype(t)
            if op == '%':
                return np.fmod(x, y).astype(t)
        raise ValueError(op)

    def unary(self):
        t = self.peek()
        if t == ('op', '-'):
            self.take()
            v = self.unary()
            return (-np.asarray(v)).astype(_dt(v))
        if t == ('op', '+'):
            self.take()
            return self.unary()
        if t == ('op', '!'):
            self.take()
            return (np.asarray(self.unary()) == 0).astype(I32)
        return self.primary()

    def primary(self):
        kind, val = self.take()
        if kind == 'num':
            return np.asarray(val)
        if kind == 'id':
            if self.peek() == ('op', '('):
                self.take()
                args = [self.binary(0)]
                while self.peek() == ('op', ','):
                    self.take()
                    args.append(self.binary(0))
                self.take(('op', ')'))
                return _call(val, args)
            if val == 'M_PI_F':
                return np.asarray(F32(math.pi))
            if val not in self.env:
                raise ValueError('unknown name %r in %r' % (val, self.text))
            return np.asarray(self.env[val])
        if (kind, val) == ('op', '('):
            nxt = self.peek()
            if nxt[0] == 'id' and nxt[1] in ('float', 'double', 'int', 'unsigned'):
                ty = {'float': F32, 'double': F64, 'int': I32, 'unsigned': U32}[self.take()[1]]
                self.take(('op', ')'))
                return _cast(self.unary(), ty)
            v = self.binary(0)
            self.take(('op', ')'))
            return v
        raise ValueError('unexpected %r in %r' % (val, self.text))


def ceval(text, env):
    "Evaluate a C expression with numpy values under C's conversion rules."
    return _Parser(text, env).parse()


# ---------------------------------------------------------------------------
# the model file
# ---------------------------------------------------------------------------
def _put(d, k, v):
    d[k] = v          # later definitions replace earlier ones, order of first


def read_model(path, name):
    "Own reading of a LEMS model file: dict of the parts the step uses."
    root = ET.parse(path).getroot()
    comps = list(root.iter('ComponentType'))
    mc = next(c for c in comps if c.get('name') == name)
    dyn = mc.find('Dynamics')
    out = {'constants': {}, 'params': [], 'derived': {}, 'couplings': [], 'noise': False}
    for c in mc.findall('Constant'):
        _put(out['constants'], c.get('name'), c.get('default'))
    for p in mc.findall('Parameter'):
        if p.get('name') not in out['params']:
            out['params'].append(p.get('name'))
    for d in mc.findall('DerivedParameter'):
        _put(out['derived'], d.get('name'), d.get('expression'))
    out['states'] = [(s.get('name'), (s.get('boundaries') or '').strip())
                     for s in dyn.findall('StateVariable')]
    out['dvars'] = [(d.get('name'), d.get('expression')) for d in dyn.findall('DerivedVariable')]
    out['cvars'] = [(c.get('name'), c.get('condition'), [x.strip() for x in c.get('cases').split(';')])
                    for c in dyn.findall('ConditionalDerivedVariable')]
    out['tders'] = [t.get('expression') for t in dyn.findall('TimeDerivative')]
    out['expos'] = [x.get('choices') for x in mc.findall('Exposure')]
    for c in comps:
        nm = c.get('name') or ''
        if c is mc:
            continue
        if nm == 'noise':
            out['noise'] = (c.get('description') or '') == 'on'
        elif 'coupling' in nm:
            cp = {'constants': {}, 'param': None, 'pre': None, 'post': None,
                  'derived': [(d.get('name'), d.get('expression'))
                              for d in c.findall('DerivedParameter')]}
            for k in c.findall('Constant'):
                _put(cp['constants'], k.get('name'), k.get('default'))
            ps = c.findall('Parameter')
            if ps:
                cp['param'] = (ps[0].get('name'), int(ps[0].get('dimension') or 0))
            d = c.find('Dynamics')
            if d is not None:
                for dv in d.findall('DerivedVariable'):
                    e = dv.get('expression')
                    if e is not None and e.strip() not in ('None', 'none'):
                        cp[dv.get('name')] = e
            out['couplings'].append(cp)
    return out


def _none(e):
    return e is None or e.strip() in ('None', 'none', '')


def constants_env(m):
    env = {}
    for n, e in m['constants'].items():
        env[n] = ceval(e, env).astype(F32)
    for cp in m['couplings']:
        for n, e in cp['constants'].items():
            env[n] = ceval(e, env).astype(F32)
    return env


def derived_params(m, params, dt, n_node):
    """Per work item: swept then derived parameters as float32 (dict and
    the slot vector), with dt float and n_node unsigned int."""
    env = constants_env(m)
    env['dt'] = F32(dt)
    env['n_node'] = U32(n_node)
    slots = []
    for k, n in enumerate(m['params']):
        env[n] = F32(params[k])
        slots.append(env[n])
    for n, e in m['derived'].items():
        env[n] = ceval(e, env).astype(F32)
        slots.append(env[n])
    return env, np.array(slots, F32)


def delays(m, env, lengths):
    e = m['derived'].get('rec_speed_dt')
    ln = np.asarray(lengths, F32)
    if e is None or e.strip() in ('0', '0.0', '0f', '0.0f'):
        return np.zeros(ln.shape, np.int64)
    rec = F32(env['rec_speed_dt'])
    return (ln * rec).astype(F32).astype(np.int64)


def run(path, name, row, col, w, lengths, params, dt, nsteps, state0=None):
    """Advance every work item (a row of params) nsteps from t0 = 0.
    Returns dict(state (I, N, ns) float32, expo (I, N, nexpo), delays list)."""
    m = read_model(path, name)
    row = np.asarray(row, np.int64)
    col = np.asarray(col, np.int64)
    w = np.asarray(w, F32)
    N = row.size - 1
    ns = len(m['states'])
    names = [s for s, _ in m['states']]
    params = np.atleast_2d(np.asarray(params, F32))
    I = params.shape[0]
    if state0 is None:
        state0 = np.zeros((N, ns), F32)
        state0[:, 0] = F32(0.001)
    st0 = np.broadcast_to(np.asarray(state0, F32), (I, N, ns))
    dyn = [cp for cp in m['couplings'] if cp['pre'] is not None or cp['post'] is not None]
    dst = np.repeat(np.arange(N), np.diff(row))
    out_state = np.zeros((I, N, ns), F32)
    out_expo = np.zeros((I, N, len(m['expos'])), F32)
    dl = []
    for b in range(I):
        env0, _ = derived_params(m, params[b], dt, N)
        d = delays(m, env0, lengths)
        dl.append(d)
        x = st0[b].copy()
        hist = np.zeros((nsteps + 1, N, ns), F32)     # every state variable, t = 0..T
        hist[0] = x
        nz = np.diff(row) > 0
        for t in range(nsteps):
            env = dict(env0)
            for v, n in enumerate(names):
                env[n] = x[:, v]
            sums = []
            src = t - d
            for cp in dyn:                    # one sum per coupling with dynamics
                dim = cp['param'][1]
                xj = np.where(src >= 0, hist[np.maximum(src, 0), col, dim], F32(0))
                ee = dict(env0)
                ee[cp['param'][0]] = xj.astype(F32)
                ee[names[dim]] = x[dst, dim]
                pre = F32(1) if _none(cp['pre']) else ceval(cp['pre'], ee)
                post = F32(1) if _none(cp['post']) else ceval(cp['post'], ee)
                term = np.broadcast_to(w * np.asarray(post) * np.asarray(pre), w.shape).astype(F32)
                S = np.zeros(N, F32)
                if term.size:
                    S[nz] = np.add.reduceat(term, row[:-1][nz]).astype(F32)
                sums.append(S)
            k = 0
            for c in m['couplings']:
                live = c['pre'] is not None or c['post'] is not None
                S = sums[k] if live else np.zeros(N, F32)
                k += 1 if live else 0
                for n, e in c['derived']:
                    v = S.copy()
                    if not _none(e):
                        v = (v * ceval(e, env)).astype(F32)
                    env[n] = v
            for n, e in m['dvars']:
                env[n] = ceval(e, env).astype(F32)
            for n, cond, (ca, cb) in m['cvars']:
                c_ = np.asarray(ceval(cond, env)) != 0
                env[n] = np.where(c_, ceval(ca, env), ceval(cb, env)).astype(F32)
            f = [np.broadcast_to(ceval(e, env), (N, )).astype(F32) for e in m['tders']]
            xn = np.empty_like(x)
            for v in range(ns):
                xn[:, v] = (x[:, v] + F32(dt) * f[v]).astype(F32)
            for v, (n, bnd) in enumerate(m['states']):
                if bnd == 'PI':
                    two_pi = F32(2) * F32(math.pi)
                    xv = xn[:, v]
                    xn[:, v] = np.where(xv < 0, two_pi - np.fmod(-xv, two_pi),
                                        np.fmod(xv, two_pi)).astype(F32)
                elif bnd:
                    lo, hi = [ceval(s, {}).astype(F32) for s in bnd.split(',')]
                    xn[:, v] = np.where(xn[:, v] < lo, lo,
                                        np.where(xn[:, v] > hi, hi, xn[:, v]))
            x = xn
            hist[t + 1] = x
        out_state[b] = x
        env = constants_env(m)
        for v, n in enumerate(names):
            env[n] = x[:, v]
        for k, e in enumerate(m['expos']):
            out_expo[b, :, k] = np.broadcast_to(ceval(e, env), (N, )).astype(F32)
    return {'state': out_state, 'expo': out_expo, 'delays': dl}
