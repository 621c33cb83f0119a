"""
LEMS-XML model front-end: neural-mass models written in the XML dialect of
tvb-hpc's CUDA DSL (dsl/dsl_cuda/XMLmodels/*.xml, read by
dsl/dsl_cuda/LEMS2CUDA.py:37-86) become step kernels of this engine.

The reference renders the XML through a Mako template into a standalone
CUDA kernel (dsl/dsl_cuda/tmpl8_CUDA.py:42-263: one thread per work item,
dense N x N weights scanned with a branch on w == 0, curand noise).  Here the
XML becomes the device functors of the engine's per-step kernel
(tvbg_step.cuh): a model struct (drift, observables, wrap/clamp) and a
coupling functor (pre(x_j, x_i) per edge), compiled by nvcc for sm_103a into
one shared library per model with the C ABI of include/tvbg_lems.h.  The
engine supplies the CSR gather, the history ring (in shared memory when it
fits), chunked resumable runs and Philox noise.

Step semantics (the template's, tmpl8_CUDA.py:145-243), for work item b and
node i at step t:

    S      = sum_e w_e * post * pre          pre reads x_j[dim](t - d_e) and x_i[dim](t)
    c_k    = S, or 0 for a coupling component without dynamics;
             then c_k *= expression           (the coupling's DerivedParameters)
    derived variables, conditional derived variables (in file order)
    x_v   += dt * f_v(x, c, ...)   (+ nsig * z_v when the noise component is "on")
    x_v    = wrap to [0, 2 pi) ("PI" boundaries) or clamp to (lo, hi)
    ring[t + 1] = x[dim]

with d_e = (unsigned) (length_e * rec_speed_dt) in float32 (D1 truncation,
tmpl8_CUDA.py:155-161; a missing or "0" rec_speed_dt means no delay), the
history zero before t0, and the state starting at 0.001 in variable 0
(tmpl8_CUDA.py:124-129).  Departures from the template, each deliberate:
all derivatives are taken from the state at t (the template does this too)
and the Euler update is applied with or without noise (the template's
update without noise is commented out, tmpl8_CUDA.py:225-229); the noise is
the engine's Philox stream (key = seed, work item; counter = node, step)
instead of per-thread curand XORWOW.

Swept parameters (the model's <Parameter> elements, e.g. global_speed,
global_coupling) are per work item, in file order; derived parameters are
evaluated per work item on the host by the generated library (C semantics:
dt is float, n_node unsigned int).  Expressions are C and are emitted
verbatim; `single=True` turns unsuffixed floating literals into float
literals (the whole step in FP32, as the GPU wants) instead of the C rule
that makes them double.

Restrictions (checked, ValueError / NotImplementedError): at most two
coupling components with dynamics (two only when both are separable: a
model with two coupled inputs, on the group kernel); pre/post read only
the coupled variable, constants and parameters; at most 8 state variables;
swept plus derived parameters at most 16; exposures read state and
constants.

Execution: LemsSweep runs the per-step kernel (one CTA per work item, any
coupling); LemsGroupSet the lane-interleaved group kernel (eight work items
per group) for separable couplings (pre(x_j) written into the ring), sine
differences (sin/cos ring channels) and two separable couplings;
make_set picks the group kernel where it applies.  A state variable's
noise="0" attribute (an extension) takes it out of the noise.
"""

import ctypes
import hashlib
import os
import re
import subprocess
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import _native as nat
from . import scheme as sch
from .engine import Sweep
from .groups import GroupSet, L as L_GROUP

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, 'csrc')
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), 'include')
BUILD_DIR = os.path.join(PKG_ROOT, '_build', 'lems')
LIB_DIR = os.path.join(HERE, '_lib', 'lems')
MODELS_DIR = os.path.join(HERE, 'lems_models')

MAX_K = 16       # swept + derived parameters per work item (tvbg_instance.consts)
MAX_NS = 8
LEMS_ABI = 1

INFO_FIELDS = ('ns', 'nparams', 'nderived', 'nexpo', 'cvar', 'noise', 'rec_speed_dt', 'nsig',
               'abi', 'group')

# functions an expression may call (C / CUDA math)
FUNCS = set('''sin cos tan asin acos atan atan2 sinh cosh tanh exp exp2 expm1 log log2 log10 log1p
sqrt cbrt pow fabs floor ceil fmin fmax fmod sinf cosf tanf asinf acosf atanf atan2f sinhf coshf
tanhf expf exp2f expm1f logf log2f log10f log1pf sqrtf cbrtf powf fabsf floorf ceilf fminf fmaxf
fmodf'''.split())
# names the generated code reserves
RESERVED = {'M_PI_F', 'PI_2'}
# C type names an expression may use in casts
CTYPES = {'float', 'double', 'int', 'unsigned'}

_NUM = re.compile(r'(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?[fFlLuU]*')
_ID = re.compile(r'[A-Za-z_][A-Za-z0-9_]*')


def tokens(expr):
    "Split a C expression into ('num' | 'id' | 'op', text) tokens."
    out, i = [], 0
    while i < len(expr):
        ch = expr[i]
        if ch.isspace():
            i += 1
            continue
        m = _NUM.match(expr, i)
        if m and (ch.isdigit() or (ch == '.' and i + 1 < len(expr) and expr[i + 1].isdigit())):
            out.append(('num', m.group()))
            i = m.end()
            continue
        m = _ID.match(expr, i)
        if m:
            out.append(('id', m.group()))
            i = m.end()
            continue
        two = expr[i:i + 2]
        if two in ('<=', '>=', '==', '!=', '&&', '||'):
            out.append(('op', two))
            i += 2
            continue
        out.append(('op', ch))
        i += 1
    return out


def names_in(expr):
    "Identifiers an expression reads (function names excluded)."
    tk = tokens(expr)
    out = []
    for k, (kind, txt) in enumerate(tk):
        if kind != 'id':
            continue
        if k + 1 < len(tk) and tk[k + 1] == ('op', '('):
            if txt not in FUNCS:
                raise ValueError('unknown function %r in %r' % (txt, expr))
            continue
        if txt not in CTYPES:
            out.append(txt)
    return out


def to_single(expr):
    "Rewrite unsuffixed floating literals as float literals (1.0 -> 1.0f)."
    out = []
    for kind, txt in tokens(expr):
        if kind == 'num' and not txt[-1] in 'fFlLuU' and ('.' in txt or 'e' in txt or 'E' in txt):
            txt = txt + 'f'
        out.append(txt)
    return ' '.join(out)


@dataclass
class Coupling:
    name: str
    constants: list = field(default_factory=list)   # (name, expr)
    param: tuple = None                             # (name, state index)
    pre: str = None
    post: str = None
    derived: list = field(default_factory=list)     # (name, expr or None)

    @property
    def dynamic(self):
        return self.pre is not None or self.post is not None


@dataclass
class LemsModel:
    name: str
    constants: list            # (name, expr)
    params: list               # swept per work item
    derived_params: list       # (name, expr)
    states: list               # (name, boundaries)
    derived_vars: list         # (name, expr)
    cond_vars: list            # (name, condition, (if_case, else_case))
    time_derivs: list          # (name, expr)
    exposures: list            # (name, expr)
    couplings: list            # Coupling
    noise: bool
    source: str = ''
    noise_scales: list = None  # per state variable factor on nsig (default 1)

    # -- shape ------------------------------------------------------------------
    @property
    def ns(self):
        return len(self.states)

    @property
    def state_names(self):
        return [s for s, _ in self.states]

    @property
    def dyn_couplings(self):
        "Coupling components with dynamics (pre/post), at most two."
        return [c for c in self.couplings if c.dynamic]

    @property
    def dyn_coupling(self):
        dyn = self.dyn_couplings
        return dyn[0] if dyn else None

    @property
    def cvar(self):
        "Index of the coupled state variable (the ring's observable)."
        c = self.dyn_coupling
        return int(c.param[1]) if c is not None and c.param is not None else 0

    @property
    def cvar2(self):
        "State variable the second coupling reads (= cvar with one coupling)."
        dyn = self.dyn_couplings
        return int(dyn[1].param[1]) if len(dyn) > 1 and dyn[1].param is not None else self.cvar

    @property
    def scales(self):
        return list(self.noise_scales) if self.noise_scales else [1.0] * self.ns

    def _separable(self, c):
        "pre reads only x_j (and constants/parameters), post not x_j."
        pj, own = c.param[0], self.state_names[c.param[1]]
        if c.post is not None and pj in names_in(c.post):
            return False
        return c.pre is None or own not in names_in(c.pre)

    @property
    def k_names(self):
        "Per-work-item slots: swept parameters, then derived parameters."
        return list(self.params) + [n for n, _ in self.derived_params]

    def k_index(self, name):
        ks = self.k_names
        return ks.index(name) if name in ks else -1

    def derived(self, name):
        for n, e in self.derived_params:
            if n == name:
                return e
        return None

    @property
    def coupling_class(self):
        """How the group kernel can take the coupling: 'sep' (pre reads only
        x_j: applied when the ring slot is written), 'sc' (pre is
        sin(x_j - x_i): sin and cos ring channels), 'sep2' (two separable
        couplings, one ring channel each), or 'edge' (per edge only: the
        per-step kernel)."""
        dyn = self.dyn_couplings
        if len(dyn) == 2:
            return 'sep2' if all(self._separable(c) for c in dyn) else 'edge2'
        c = self.dyn_coupling
        if c is None:
            return 'sep'
        pj, own = c.param[0], self.state_names[c.param[1]]
        if c.post is not None and pj in names_in(c.post):
            return 'edge'
        if self._separable(c):
            return 'sep'
        tk = tokens(c.pre)
        if (len(tk) == 6 and tk[0][0] == 'id' and tk[0][1] in ('sin', 'sinf') and tk[1] == ('op', '(')
                and tk[2] == ('id', pj) and tk[3] == ('op', '-') and tk[4] == ('id', own)
                and tk[5] == ('op', ')')):
            return 'sc'
        return 'edge'

    @property
    def has_delays(self):
        e = self.derived('rec_speed_dt')
        return e is not None and e.strip() not in ('0', '0.0', '0.0f', '0f')

    # -- checks -----------------------------------------------------------------
    def validate(self):
        if not 1 <= self.ns <= MAX_NS:
            raise NotImplementedError('%d state variables: the engine takes 1..%d' % (self.ns, MAX_NS))
        if len(self.time_derivs) != self.ns:
            raise ValueError('%d time derivatives for %d state variables' % (
                len(self.time_derivs), self.ns))
        if len(self.k_names) > MAX_K:
            raise NotImplementedError('more than %d swept + derived parameters' % MAX_K)
        dyn = self.dyn_couplings
        if len(dyn) > 2:
            raise NotImplementedError('more than two coupling components with dynamics')
        if self.noise_scales is not None and len(self.noise_scales) != self.ns:
            raise ValueError('one noise factor per state variable')
        if not self.exposures:
            raise ValueError('no Exposure: the model needs an observable')
        if self.noise and self.derived('nsig') is None:
            raise ValueError('noise is on but no nsig derived parameter is given')
        mc = [n for n, _ in self.constants]
        cc = [n for c in self.couplings for n, _ in c.constants]
        consts = set(mc) | set(cc)
        params = set(self.params)
        derived = {n for n, _ in self.derived_params}
        states = set(self.state_names)
        cnames = {n for c in self.couplings for n, _ in c.derived}
        dvars = {n for n, _ in self.derived_vars} | {n for n, _, _ in self.cond_vars}
        every = [n for n, _ in self.constants] + cc + list(params) + list(derived) + list(states) \
            + list(cnames) + list(dvars)
        for n in every:
            if n.endswith('_') or n.startswith('tvbg') or n.startswith('lems_') or n in RESERVED \
                    or n in FUNCS:
                raise ValueError('name %r is reserved by the generated code' % n)
        if len(set(every)) != len(every):
            dup = sorted({n for n in every if every.count(n) > 1})
            raise ValueError('names defined twice: %s' % ', '.join(dup))

        def need(expr, allowed, where):
            for n in names_in(expr):
                if n not in allowed and n != 'M_PI_F':
                    raise ValueError('%s: unknown name %r in %r' % (where, n, expr))

        seen = set()
        for n, e in self.constants:
            need(e, seen, 'constant %s' % n)
            seen.add(n)
        seen_c = set(seen)
        for c in self.couplings:
            for n, e in c.constants:
                need(e, seen_c, 'coupling constant %s' % n)
                seen_c.add(n)
        base = consts | params | {'dt', 'n_node'}
        seen = set()
        for n, e in self.derived_params:
            need(e, base | seen, 'derived parameter %s' % n)
            seen.add(n)
        kvals = consts | params | derived
        for c in dyn:
            if c.param is None:
                raise ValueError('coupling %s has dynamics but no <Parameter> for x_j' % c.name)
            if not 0 <= c.param[1] < self.ns:
                raise ValueError('coupling parameter dimension %r out of range' % (c.param[1], ))
            own = self.state_names[c.param[1]]
            for e in (c.pre, c.post):
                if e is not None and e.strip() not in ('None', 'none'):
                    for n in names_in(e):
                        if n in states and n != own:
                            raise NotImplementedError(
                                'coupling reads state %r of the receiving node; only the coupled '
                                'variable %r is available' % (n, own))
                    need(e, kvals | {c.param[0], own}, 'coupling %s' % c.name)
        if len(dyn) == 2 and self.coupling_class != 'sep2':
            raise NotImplementedError('two couplings: both must be separable (pre reads only x_j)')
        avail = kvals | states | cnames
        for cc_ in self.couplings:
            for n, e in cc_.derived:
                if e is not None and e.strip() not in ('None', 'none'):
                    need(e, avail, 'coupling derived parameter %s' % n)
        for n, e in self.derived_vars:
            need(e, avail, 'derived variable %s' % n)
            avail = avail | {n}
        for n, cond, cases in self.cond_vars:
            need(cond, avail, 'condition of %s' % n)
            for e in cases:
                need(e, avail, 'case of %s' % n)
            avail = avail | {n}
        for n, e in self.time_derivs:
            need(e, avail, 'time derivative %s' % n)
        for n, e in self.exposures:
            need(e, consts | states, 'exposure %s' % n)
        for n, b in self.states:
            if b not in ('', 'PI'):
                lo_hi = [v.strip() for v in b.split(',')]
                if len(lo_hi) != 2:
                    raise ValueError('boundaries of %s: %r' % (n, b))
        return self


def _unique(pairs):
    """Later definitions of a name replace earlier ones in place (the XML
    reader of the reference keeps one entry per name)."""
    out, pos = [], {}
    for item in pairs:
        n = item[0] if isinstance(item, tuple) else item
        if n in pos:
            out[pos[n]] = item
        else:
            pos[n] = len(out)
            out.append(item)
    return out


def _attr(el, name, default=None):
    v = el.get(name)
    return default if v is None else v


def parse(path_or_text, name=None):
    """Read a LEMS model file (or XML text).  `name` picks the model's
    ComponentType (default: the one whose Dynamics has state variables);
    components whose name contains 'coupling' are couplings; a component
    named 'noise' with description 'on' turns noise on."""
    text = path_or_text
    src = '<text>'
    if '<' not in path_or_text and os.path.exists(path_or_text):
        src = path_or_text
        with open(path_or_text) as f:
            text = f.read()
    root = ET.fromstring(text)
    cts = [el for el in root.iter('ComponentType')]
    model_ct = None
    for el in cts:
        if name is not None and el.get('name') == name:
            model_ct = el
            break
        if name is None and el.find('Dynamics') is not None and \
                el.find('Dynamics').find('StateVariable') is not None:
            model_ct = el
            break
    if model_ct is None:
        raise ValueError('no model component %s in %s' % (name or '(with state variables)', src))
    mname = model_ct.get('name')
    dyn = model_ct.find('Dynamics')
    constants = _unique([(c.get('name'), _attr(c, 'default', '0'))
                         for c in model_ct.findall('Constant')])
    params = _unique([p.get('name') for p in model_ct.findall('Parameter')])
    derived = _unique([(d.get('name'), d.get('expression'))
                       for d in model_ct.findall('DerivedParameter')])
    states = [(s.get('name'), _attr(s, 'boundaries', '').strip()) for s in dyn.findall('StateVariable')]
    # extension: <StateVariable noise="0"/> takes a variable out of the noise
    # (the DSL's noise acts on every state variable)
    scales = [float(_attr(s, 'noise', '1')) for s in dyn.findall('StateVariable')]
    dvars = [(d.get('name'), d.get('expression')) for d in dyn.findall('DerivedVariable')]
    cvars = []
    for c in dyn.findall('ConditionalDerivedVariable'):
        cases = [x.strip() for x in c.get('cases').split(';')]
        if len(cases) != 2:
            raise ValueError('conditional %s: two cases expected, got %r' % (c.get('name'), cases))
        cvars.append((c.get('name'), c.get('condition'), tuple(cases)))
    tders = [(t.get('name'), t.get('expression')) for t in dyn.findall('TimeDerivative')]
    expos = [(x.get('name'), x.get('choices') or x.get('default')) for x in model_ct.findall('Exposure')]
    couplings = []
    noise = False
    for el in cts:
        nm = el.get('name') or ''
        if el is model_ct:
            continue
        if nm == 'noise':
            noise = (el.get('description') or '').strip() == 'on'
            continue
        if 'coupling' not in nm:
            continue
        cp = Coupling(nm)
        cp.constants = [(c.get('name'), _attr(c, 'default', '0')) for c in el.findall('Constant')]
        ps = el.findall('Parameter')
        if ps:
            cp.param = (ps[0].get('name'), int(float(_attr(ps[0], 'dimension', '0') or 0)))
        d = el.find('Dynamics')
        if d is not None:
            for dv in d.findall('DerivedVariable'):
                if dv.get('name') == 'pre':
                    cp.pre = dv.get('expression')
                elif dv.get('name') == 'post':
                    cp.post = dv.get('expression')
            if cp.pre is not None and cp.pre.strip() in ('None', 'none'):
                cp.pre = None
            if cp.post is not None and cp.post.strip() in ('None', 'none'):
                cp.post = None
        cp.derived = [(x.get('name'), x.get('expression')) for x in el.findall('DerivedParameter')]
        couplings.append(cp)
    m = LemsModel(mname, constants, params, derived, states, dvars, cvars, tders, expos, couplings,
                  noise, source=src, noise_scales=None if all(v == 1.0 for v in scales) else scales)
    return m.validate()


def lems_file(model_name, folder=None):
    "Path of a model file: <folder>/<model_name lower-case>_CUDA.xml (LEMS2CUDA.py:16-18)."
    return os.path.join(folder or MODELS_DIR, model_name.lower() + '_CUDA.xml')


def load_model(model_name, folder=None):
    "Load model `model_name` from its file (LEMS2CUDA.py:26-34)."
    return parse(lems_file(model_name, folder), name=model_name)


# ---------------------------------------------------------------------------
# code generation
# ---------------------------------------------------------------------------
def _expr(e, single):
    e = e.strip()
    return to_single(e) if single else e


def _none(e):
    return e is None or e.strip() in ('None', 'none', '')


def render_cuda(m, single=False):
    """CUDA source of the model's library: device functors for the engine's
    per-step kernel plus the exported entry points of include/tvbg_lems.h."""
    E = lambda e: _expr(e, single)  # noqa: E731
    L = []
    w = L.append
    kn = m.k_names
    cp = m.dyn_coupling
    w('// Generated by tvb_hpc.lems from the LEMS model "%s" (%s).' % (m.name, os.path.basename(m.source)))
    w('// Step structure of dsl/dsl_cuda/tmpl8_CUDA.py:145-243 on the engine\'s per-step kernel.')
    w('#include <cmath>')
    w('#include <cstdio>')
    w('#include "tvbg_step.cuh"')
    w('#include "tvbg_step_launch.cuh"')
    w('#include "tvbg_group_launch.cuh"')
    w('')
    w('#define M_PI_F 3.14159265358979323846f')
    w('#define PI_2 (2 * M_PI_F)')
    w('#define TVBG_LEMS_EXPORT extern "C" __attribute__((visibility("default")))')
    w('#pragma nv_diag_suppress 177')
    w('#pragma nv_diag_suppress 550')
    w('#pragma GCC diagnostic ignored "-Wunused-variable"')
    w('#pragma GCC diagnostic ignored "-Wunused-but-set-variable"')
    w('')
    w('namespace {')
    w('using namespace tvbg;')
    w('constexpr int kNS = %d;' % m.ns)
    w('constexpr int kNParams = %d;' % len(m.params))
    w('constexpr int kNDerived = %d;' % len(m.derived_params))
    w('constexpr int kNExpo = %d;' % len(m.exposures))
    w('constexpr int kCVar = %d;' % m.cvar)
    w('')

    def consts(indent='    ', coupling=False):
        for n, e in m.constants:
            w('%sconst float %s = %s;' % (indent, n, E(e)))
        if coupling:
            for c in m.couplings:
                for n, e in c.constants:
                    w('%sconst float %s = %s;' % (indent, n, E(e)))

    def kvals(src, indent='    '):
        for k, n in enumerate(kn):
            w('%sconst float %s = %s[%d];' % (indent, n, src, k))

    # model struct
    w('struct LemsModel {')
    w('    static constexpr int ID = TVBG_MODEL_LEMS;')
    w('    static constexpr int NS = kNS;')
    w('    static constexpr int NP = %d;  // per-work-item slots, read per node' % max(1, len(kn)))
    w('    static constexpr int NOBS = 1 + kNExpo;')
    w('    static constexpr bool kWideNoise = true;')
    w('    static constexpr int CVAR2 = %d;  // state variable of the second coupling' % m.cvar2)
    w('    static constexpr bool kTwoInputs = %s;' % ('true' if len(m.dyn_couplings) == 2 else 'false'))
    w('    __device__ static __forceinline__ float noise_scale(int v_) {')
    w('        switch (v_) {')
    for v, f in enumerate(m.scales):
        w('            case %d: return %sf;' % (v, repr(float(f))))
    w('            default: return 1.0f;')
    w('        }')
    w('    }')
    w('    __device__ static __forceinline__ void drift(const float* x_, float S_, const float* p_,')
    w('                                                 const float* K_, float* f_) {')
    w('        drift2(x_, S_, 0.0f, p_, K_, f_);')
    w('    }')
    w('    // S_, S2_: the raw sums of the first and second coupling with dynamics')
    w('    __device__ static __forceinline__ void drift2(const float* x_, float S_, float S2_,')
    w('                                                  const float* p_, const float*, float* f_) {')
    consts('        ', coupling=True)
    kvals('p_', '        ')
    for v, n in enumerate(m.state_names):
        w('        const float %s = x_[%d];' % (n, v))
    dyn_ids = [id(c) for c in m.dyn_couplings]
    for c in m.couplings:
        src = ('S_' if dyn_ids and id(c) == dyn_ids[0] else
               'S2_' if len(dyn_ids) > 1 and id(c) == dyn_ids[1] else '0.0f')
        for n, e in c.derived:
            w('        float %s = %s;' % (n, src))
            if not _none(e):
                w('        %s *= %s;' % (n, E(e)))
    for n, e in m.derived_vars:
        w('        const float %s = %s;' % (n, E(e)))
    for n, cond, (a, b) in m.cond_vars:
        w('        float %s;' % n)
        w('        if (%s)' % E(cond))
        w('            %s = %s;' % (n, E(a)))
        w('        else')
        w('            %s = %s;' % (n, E(b)))
    for v, (n, e) in enumerate(m.time_derivs):
        w('        f_[%d] = %s;' % (v, E(e)))
    w('    }')
    w('    __device__ static __forceinline__ float obs(const float* x_, int k_) {')
    consts('        ')
    for v, n in enumerate(m.state_names):
        w('        const float %s = x_[%d];' % (n, v))
    w('        switch (k_) {')
    for k, (n, e) in enumerate(m.exposures):
        w('            case %d: return %s;  // %s' % (k + 1, E(e), n))
    w('            default: return x_[kCVar];')
    w('        }')
    w('    }')
    # group-kernel hooks: the ring value of a separable coupling, and the
    # coupling input from the gathered sum
    cls = m.coupling_class
    dyn = m.dyn_couplings

    def ring_value_fn(fname, c):
        w('    __host__ __device__ static __forceinline__ float %s(float o_, const float* p_) {' % fname)
        if c is not None and cls in ('sep', 'sep2'):
            consts('        ', coupling=True)
            kvals('p_', '        ')
            w('        const float %s = o_;' % c.param[0])
            w('        return %s;' % ('1.0f' if _none(c.pre) else '(%s)' % E(c.pre)))
        else:
            w('        return o_;')
        w('    }')

    def coupling_fn(fname, c):
        w('    __device__ static __forceinline__ float %s(float S_, const float* x_, const float* p_) {'
          % fname)
        if c is not None and cls in ('sep', 'sc', 'sep2'):
            consts('        ', coupling=True)
            kvals('p_', '        ')
            d = int(c.param[1])
            w('        const float %s = x_[%d];' % (m.state_names[d], d))
            w('        return %s * S_;' % ('1.0f' if _none(c.post) else '(%s)' % E(c.post)))
        else:
            w('        return 0.0f;')
        w('    }')

    ring_value_fn('ring_value', dyn[0] if dyn else None)
    ring_value_fn('ring_value2', dyn[1] if len(dyn) > 1 else None)
    coupling_fn('coupling', dyn[0] if dyn else None)
    coupling_fn('coupling2', dyn[1] if len(dyn) > 1 else None)
    w('    __device__ static __forceinline__ void limit(float* x_, uint32_t) {')
    for v, (n, b) in enumerate(m.states):
        if b == 'PI':
            w('        x_[%d] = x_[%d] < 0.0f ? PI_2 - fmodf(-x_[%d], PI_2) : fmodf(x_[%d], PI_2);'
              % (v, v, v, v))
        elif b:
            lo, hi = [s.strip() for s in b.split(',')]
            w('        {')
            w('            const float lim_[2] = {%s, %s};' % (lo, hi))
            w('            if (x_[%d] < lim_[0]) x_[%d] = lim_[0];' % (v, v))
            w('            else if (x_[%d] > lim_[1]) x_[%d] = lim_[1];' % (v, v))
            w('        }')
    w('    }')
    w('};')
    w('}  // namespace')
    w('')
    # coupling functor
    w('namespace tvbg {')
    w('template <>')
    w('struct Cfun<TVBG_CFUN_LEMS> {')
    w('    static constexpr bool kNeedsPost = %s;' % ('true' if cp is not None else 'false'))
    pname = cp.param[0] if cp is not None else 'xj_'
    own = m.state_names[m.cvar] if cp is not None else 'xi_'
    w('    __device__ static __forceinline__ float pre(float %s, float %s, const tvbg_instance& d_) {'
      % (pname, own))
    if cp is not None:
        consts('        ', coupling=True)
        kvals('d_.consts', '        ')
        pre = '1.0f' if _none(cp.pre) else '(%s)' % E(cp.pre)
        post = '1.0f' if _none(cp.post) else '(%s)' % E(cp.post)
        w('        return %s * %s;' % (post, pre))
    else:
        w('        return 0.0f;')
    w('    }')
    w('    __device__ static __forceinline__ float post(float s_, const tvbg_instance&) { return s_; }')
    w('};')
    w('}  // namespace tvbg')
    w('')
    w('namespace {')
    w('thread_local char g_err[512] = "";')
    w('int lems_error(int code, const char* msg) {')
    w('    std::snprintf(g_err, sizeof(g_err), "%s", msg);')
    w('    return code;')
    w('}')
    w('int lems_cuda_error(cudaError_t e, const char* where) {')
    w('    std::snprintf(g_err, sizeof(g_err), "%s: %s (%s)", where, cudaGetErrorName(e),')
    w('                  cudaGetErrorString(e));')
    w('    return TVBG_ECUDA;')
    w('}')
    w('const ErrSink kSink{lems_error, lems_cuda_error};')
    w('using Kernel = void (*)(const tvbg_instance*, int32_t, const int32_t*, int32_t*, int32_t*, uint32_t);')
    w('Kernel lookup(int tpn) {')
    w('    switch (tpn) {')
    for t in (1, 2, 4, 8):
        w('        case %d: return step_kernel<LemsModel, TVBG_CFUN_LEMS, %d>;' % (t, t))
    w('        default: return nullptr;')
    w('    }')
    w('}')
    w('int run(const tvbg_instance* d_inst, int32_t n_inst, const tvbg_launch* cfg, bool persistent,')
    w('        void* stream) {')
    w('    int rc = check_step_launch(cfg, d_inst, n_inst, kSink);')
    w('    if (rc) return rc;')
    w('    if (cfg->model != TVBG_MODEL_LEMS || cfg->cfun != TVBG_CFUN_LEMS || cfg->block_k > 1)')
    w('        return lems_error(TVBG_EINVAL, "LEMS library: model/cfun must be TVBG_*_LEMS, block_k 0 or 1");')
    w('    if (LemsModel::kTwoInputs)')
    w('        return lems_error(TVBG_EUNSUPPORTED, "LEMS library: two coupled inputs run on the group '
      'kernel only (tvbg_lems_group_run)");')
    w('    if (n_inst == 0) return TVBG_OK;')
    w('    Kernel k = lookup(cfg->tpn);')
    w('    const size_t smem = step_smem_bytes(cfg->threads, cfg->smem_ring);')
    w('    cudaStream_t st = static_cast<cudaStream_t>(stream);')
    w('    int grid = 0;')
    w('    rc = prepare_step_launch(reinterpret_cast<const void*>(k), smem, n_inst, cfg, persistent, st,')
    w('                             kSink, &grid);')
    w('    if (rc || grid == 0) return rc;')
    w('    k<<<grid, cfg->threads, smem, st>>>(d_inst, n_inst, persistent ? cfg->d_order : nullptr,')
    w('                                        persistent ? cfg->d_counter : nullptr, cfg->d_status,')
    w('                                        static_cast<uint32_t>(cfg->smem_ring));')
    w('    const cudaError_t e = cudaGetLastError();')
    w('    return e == cudaSuccess ? TVBG_OK : lems_cuda_error(e, "LEMS step kernel launch");')
    w('}')
    w('__global__ void expose_kernel(const float* __restrict__ s_, long long n_, float* __restrict__ o_) {')
    w('    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;')
    w('    if (i >= n_) return;')
    w('    float x_[kNS];')
    w('#pragma unroll')
    w('    for (int v = 0; v < kNS; ++v) x_[v] = s_[i * kNS + v];')
    w('#pragma unroll')
    w('    for (int k = 0; k < kNExpo; ++k) o_[i * kNExpo + k] = LemsModel::obs(x_, 1 + k);')
    w('}')
    gcf = {'sep': 'TVBG_CFUN_LEMS', 'sc': 'TVBG_CFUN_LEMS_SC', 'sep2': 'TVBG_CFUN_LEMS_2'}.get(cls)
    w('GroupKernelFn lookup_group(int cfun, int k) {')
    if gcf is not None:
        w('    if (cfun != %s) return nullptr;' % gcf)
        w('    switch (k) {')
        for kk in (1, 2, 4, 8):
            w('        case %d: return group_kernel<LemsModel, %s, %d>;' % (kk, gcf, kk))
        w('        default: return nullptr;')
        w('    }')
    else:
        w('    return nullptr;')
    w('}')
    w('}  // namespace')
    w('')
    # exports
    w('TVBG_LEMS_EXPORT const char* tvbg_lems_last_error(void) { return g_err; }')
    w('TVBG_LEMS_EXPORT int tvbg_lems_info(int32_t* info) {')
    w('    if (!info) return lems_error(TVBG_EINVAL, "tvbg_lems_info: null");')
    vals = [m.ns, len(m.params), len(m.derived_params), len(m.exposures), m.cvar, int(m.noise),
            m.k_index('rec_speed_dt') if m.has_delays else -1, m.k_index('nsig'), LEMS_ABI,
            {'sep': 1, 'sc': 2, 'sep2': 3}.get(cls, 0)]
    for k, v in enumerate(vals):
        w('    info[%d] = %d;  // %s' % (k, v, INFO_FIELDS[k]))
    w('    return TVBG_OK;')
    w('}')
    w('TVBG_LEMS_EXPORT int tvbg_lems_derived(const float* params_, int32_t n_work_, int32_t n_params_,')
    w('                                      float dt_, int32_t n_node_, float* out_) {')
    w('    if (n_work_ < 0 || !out_ || (n_work_ > 0 && kNParams > 0 && !params_) || n_params_ != kNParams)')
    w('        return lems_error(TVBG_EINVAL, "tvbg_lems_derived: bad arguments");')
    w('    for (int32_t b_ = 0; b_ < n_work_; ++b_) {')
    w('        const float dt = dt_;')
    w('        const unsigned int n_node = static_cast<unsigned int>(n_node_);')
    consts('        ')
    for k, n in enumerate(m.params):
        w('        const float %s = params_[b_ * kNParams + %d];' % (n, k))
    for n, e in m.derived_params:
        w('        const float %s = %s;' % (n, E(e)))
    w('        float* o_ = out_ + static_cast<long long>(b_) * %d;' % MAX_K)
    w('        for (int k_ = 0; k_ < %d; ++k_) o_[k_] = 0.0f;' % MAX_K)
    for k, n in enumerate(kn):
        w('        o_[%d] = %s;' % (k, n))
    w('    }')
    w('    return TVBG_OK;')
    w('}')
    w('TVBG_LEMS_EXPORT int tvbg_lems_sweep(const tvbg_instance* d_inst, int32_t n_inst,')
    w('                                    const tvbg_launch* cfg, void* stream) {')
    w('    return run(d_inst, n_inst, cfg, false, stream);')
    w('}')
    w('TVBG_LEMS_EXPORT int tvbg_lems_batch_run(const tvbg_instance* d_inst, int32_t n_inst,')
    w('                                        const tvbg_launch* cfg, void* stream) {')
    w('    return run(d_inst, n_inst, cfg, true, stream);')
    w('}')
    w('TVBG_LEMS_EXPORT int tvbg_lems_group_run(const tvbg_group* d_groups, int32_t n_groups,')
    w('                                        const tvbg_launch* cfg, void* stream) {')
    w('    int cluster = 1;')
    w('    int rc = check_group_cfg(cfg, kSink, &cluster, 0x116u);  // K = 1, 2, 4, 8')
    w('    if (rc) return rc;')
    w('    if (cfg->model != TVBG_MODEL_LEMS)')
    w('        return lems_error(TVBG_EINVAL, "tvbg_lems_group_run: model must be TVBG_MODEL_LEMS");')
    w('    GroupKernelFn k = lookup_group(cfg->cfun, cfg->block_k);')
    w('    if (!k)')
    w('        return lems_error(TVBG_EUNSUPPORTED, "tvbg_lems_group_run: this coupling needs the '
      'per-step kernel, or cfun/block_k do not match");')
    w('    const size_t smem = group_smem_bytes(cfg->block_k, cfg->threads, group_channels(cfg->cfun));')
    w('    return launch_group_kernel(k, d_groups, n_groups, cfg, cluster, smem, stream, kSink);')
    w('}')
    w('TVBG_LEMS_EXPORT int tvbg_lems_ring_value(const float* slots, int32_t n, float o, int32_t which,')
    w('                                         float* out) {')
    w('    if (n < 0 || (n > 0 && (!slots || !out)) || which < 0 || which > 1)')
    w('        return lems_error(TVBG_EINVAL, "tvbg_lems_ring_value: bad arguments");')
    w('    for (int32_t b = 0; b < n; ++b)')
    w('        out[b] = which ? LemsModel::ring_value2(o, slots + %d * b) : LemsModel::ring_value(o, slots + %d * b);'
      % (MAX_K, MAX_K))
    w('    return TVBG_OK;')
    w('}')
    w('TVBG_LEMS_EXPORT int tvbg_lems_expose(const float* d_state, int64_t n, float* d_out, void* stream) {')
    w('    if (!d_state || !d_out || n < 0) return lems_error(TVBG_EINVAL, "tvbg_lems_expose: bad arguments");')
    w('    if (n == 0) return TVBG_OK;')
    w('    const long long blocks = (n + 255) / 256;')
    w('    expose_kernel<<<static_cast<unsigned>(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(')
    w('        d_state, n, d_out);')
    w('    const cudaError_t e = cudaGetLastError();')
    w('    return e == cudaSuccess ? TVBG_OK : lems_cuda_error(e, "tvbg_lems_expose launch");')
    w('}')
    return '\n'.join(L) + '\n'


# ---------------------------------------------------------------------------
# build and load
# ---------------------------------------------------------------------------
_HEADERS = ('tvbg_step.cuh', 'tvbg_device.cuh', 'tvbg_step_launch.cuh', 'tvbg_lanes.cuh',
            'tvbg_step_blocked.cuh', 'tvbg_group_launch.cuh')


def _key(src):
    h = hashlib.sha256(src.encode())
    for f in _HEADERS:
        with open(os.path.join(CSRC, f), 'rb') as fh:
            h.update(fh.read())
    for f in ('tvbg.h', 'tvbg_lems.h'):
        with open(os.path.join(INCLUDE, f), 'rb') as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def build_library(m, single=False):
    "Render and compile the model's library (cached by source hash); returns its path."
    from ._build import ARCH, FLAGS, nvcc
    src = render_cuda(m, single)
    key = _key(src)
    tag = re.sub(r'[^A-Za-z0-9]', '_', m.name.lower()) + ('_f32' if single else '')
    so = os.path.join(LIB_DIR, 'libtvbg_lems_%s_%s.so' % (tag, key))
    if os.path.exists(so):
        return so
    if os.path.isdir(LIB_DIR):      # libraries of earlier versions of this model
        for f in os.listdir(LIB_DIR):
            if re.fullmatch(r'libtvbg_lems_%s_[0-9a-f]{16}\.so' % re.escape(tag), f):
                os.remove(os.path.join(LIB_DIR, f))
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    cu = os.path.join(BUILD_DIR, 'lems_%s_%s.cu' % (tag, key))
    with open(cu, 'w') as f:
        f.write(src)
    tmp = so + '.%d.tmp' % os.getpid()
    cmd = ([nvcc()] + ARCH + FLAGS + ['-Xcompiler', '-fvisibility=hidden', '-I', CSRC, '-I', INCLUDE,
                                      '-shared', '-cudart', 'static', cu, '-o', tmp])
    p = subprocess.run(cmd, capture_output=True, text=True)
    with open(cu[:-3] + '.log', 'w') as f:
        f.write(' '.join(cmd) + '\n' + p.stdout + p.stderr)
    if p.returncode != 0:
        raise RuntimeError('nvcc failed for LEMS model %s:\n%s' % (m.name, p.stderr[-4000:]))
    os.replace(tmp, so)
    return so


def bundled_models():
    "Names of the model files shipped in lems_models/."
    out = []
    for f in sorted(os.listdir(MODELS_DIR)):
        if f.endswith('_CUDA.xml'):
            root = ET.parse(os.path.join(MODELS_DIR, f)).getroot()
            for el in root.iter('ComponentType'):
                d = el.find('Dynamics')
                if d is not None and d.find('StateVariable') is not None:
                    out.append(el.get('name'))
                    break
    return out


def prebuild(jobs=None):
    "Compile the libraries of every bundled model in parallel; returns their paths."
    import concurrent.futures as cf
    ms = [load_model(n) for n in bundled_models()]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(ms), os.cpu_count() or 4)) as ex:
        return list(ex.map(build_library, ms))


_vp, _i32, _i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
SIGNATURES = {
    'tvbg_lems_last_error': (ctypes.c_char_p, []),
    'tvbg_lems_info': (ctypes.c_int, [_vp]),
    'tvbg_lems_derived': (ctypes.c_int, [_vp, _i32, _i32, ctypes.c_float, _i32, _vp]),
    'tvbg_lems_sweep': (ctypes.c_int, [_vp, _i32, ctypes.POINTER(nat.tvbg_launch), _vp]),
    'tvbg_lems_batch_run': (ctypes.c_int, [_vp, _i32, ctypes.POINTER(nat.tvbg_launch), _vp]),
    'tvbg_lems_expose': (ctypes.c_int, [_vp, _i64, _vp, _vp]),
    'tvbg_lems_group_run': (ctypes.c_int, [_vp, _i32, ctypes.POINTER(nat.tvbg_launch), _vp]),
    'tvbg_lems_ring_value': (ctypes.c_int, [_vp, _i32, ctypes.c_float, _i32, _vp]),
}

_LIBS = {}


class LemsLibrary:
    "A generated model library, loaded and typed."

    def __init__(self, m, single=False):
        self.model = m
        self.single = bool(single)
        self.path = build_library(m, single)
        if self.path not in _LIBS:
            lib = ctypes.CDLL(self.path)
            for n, (res, args) in SIGNATURES.items():
                fn = getattr(lib, n)
                fn.restype, fn.argtypes = res, args
            _LIBS[self.path] = lib
        self.lib = _LIBS[self.path]
        buf = (ctypes.c_int32 * len(INFO_FIELDS))()
        self.check(self.lib.tvbg_lems_info(ctypes.cast(buf, _vp)))
        self.info = dict(zip(INFO_FIELDS, list(buf)))
        if self.info['abi'] != LEMS_ABI:
            raise RuntimeError('LEMS library ABI mismatch')

    def check(self, rc):
        if rc != nat.TVBG_OK:
            raise nat.TvbgError(rc, self.lib.tvbg_lems_last_error().decode(errors='replace'))

    def derived(self, params, dt, n_node):
        "Per-work-item slots K (n_work, 16): swept then derived parameters."
        p = np.ascontiguousarray(np.asarray(params, np.float32).reshape(-1, len(self.model.params))
                                 if self.model.params else np.zeros((len(params), 0), np.float32))
        out = np.zeros((p.shape[0], MAX_K), np.float32)
        self.check(self.lib.tvbg_lems_derived(p.ctypes.data if p.size else None, p.shape[0],
                                              len(self.model.params), float(np.float32(dt)),
                                              int(n_node), out.ctypes.data))
        return out


class _EngineModel:
    """The engine-facing face of a LEMS model (what InstanceSet and GroupSet
    read): the per-work-item slots are its per-node parameters."""

    def __init__(self, m, noise):
        self.m = m
        self.nsvar = m.ns
        self.nobs = 1 + len(m.exposures)
        self.param_sym = list(m.k_names) or ['lems_unused']
        self._noise = noise

    def engine_spec(self):
        sigma = np.full(4, 1.0 if self._noise else 0.0, np.float32)
        return nat.MODEL_LEMS, np.zeros(MAX_K, np.float32), sigma

    def node_params(self, N):
        return np.zeros((N, len(self.param_sym)), np.float32)


class _EngineCoupling:
    def __init__(self, cfun_id=nat.CFUN_LEMS):
        self.cfun_id = cfun_id

    def engine_spec(self):
        return self.cfun_id, 0.0, 0.0, np.zeros(3, np.float32)


def _setup(lib, m, conn, dt, params):
    """Per-work-item slots K (I, 16), the delay tables (one per distinct
    rec_speed_dt) and each work item's table index."""
    params = np.asarray(params, np.float32)
    if params.ndim == 1:
        params = params.reshape(-1, max(1, len(m.params)))
    I = params.shape[0]
    K = lib.derived(params, dt, int(conn.nnode))
    ki = lib.info['rec_speed_dt']
    if ki >= 0:
        recs = K[:, ki]
        if not np.all(np.isfinite(recs)) or np.any(recs < 0):
            raise ValueError('rec_speed_dt must be finite and non-negative')
        uniq, tab_of = np.unique(recs, return_inverse=True)
        tables = [dsl_delays(conn.lnz, r) for r in uniq]
        if max((int(t.max()) if t.size else 0) for t in tables) >= 1 << 20:
            raise ValueError('delays beyond 2^20 steps')
    else:
        tables, tab_of = [np.zeros(conn.nnz, np.int64)], np.zeros(I, np.int64)
    return params, K, tables, tab_of


def _state0(m, N, state0):
    if state0 is None:
        state0 = np.zeros((N, m.ns), np.float32)
        state0[:, 0] = 0.001
    return state0


def _slots_per_node(m, K, N):
    npar = max(1, len(m.k_names))
    return np.ascontiguousarray(np.broadcast_to(K[:, None, :npar], (K.shape[0], N, npar)))


def _sigma(lib, K, dt, noise):
    """Per work item nsig / sqrt(dt) times each variable's noise factor (up
    to 4 state variables; with more, the kernels take sigma[0] times the
    factor), or zeros without noise."""
    if not noise:
        return np.zeros((K.shape[0], 4), np.float32)
    sq = np.sqrt(np.float32(dt)).astype(np.float32)
    sig = (K[:, lib.info['nsig']] / sq).astype(np.float32)
    out = np.repeat(sig[:, None], 4, axis=1)
    sc = lib.model.scales
    if len(sc) <= 4:
        for v in range(len(sc)):
            out[:, v] = (out[:, v] * np.float32(sc[v])).astype(np.float32)
    return out


def dsl_delays(lengths, rec_speed_dt):
    "d = (unsigned) (length * rec_speed_dt) in float32 (tmpl8_CUDA.py:155-161)."
    ln = np.asarray(lengths, np.float32)
    return (ln * np.float32(rec_speed_dt)).astype(np.int64)


class LemsSweep(Sweep):
    """
    Work items of one LEMS model on one connectome, advanced on the device.

    m : LemsModel (see parse / load_model)
    conn : Connectivity (CSR; weights and lengths)
    dt : step (the model's time unit)
    params : (n_work, n_params) swept parameters in the model's file order
             (e.g. [global_speed, global_coupling]), as in
             dsl/dsl_cuda/example/cuda_run.py:67-90
    state0 : (n_work, N, ns) or (N, ns); default 0.001 in variable 0
             and 0 elsewhere (tmpl8_CUDA.py:124-129)
    noise : None (the file's noise component) or True/False
    single : FP32 literals (see render_cuda)
    Remaining keyword arguments go to engine.Sweep (seed, trace_every, ...).
    """

    def __init__(self, m, conn, dt, params, state0=None, noise=None, single=False, tpn=None,
                 **kwargs):
        if len(m.dyn_couplings) > 1:
            raise ValueError('LEMS model %s: two coupled inputs run on LemsGroupSet only' % m.name)
        self.lems = LemsLibrary(m, single)
        self.lmodel = m
        noise = m.noise if noise is None else bool(noise)
        params, K, tables, tab_of = _setup(self.lems, m, conn, dt, params)
        I, N = params.shape[0], int(conn.nnode)
        em = _EngineModel(m, noise)
        scm = sch.EulerMaryuyamaStep(dt) if noise else sch.EulerStep(dt)
        kwargs.setdefault('blocked', False)
        super().__init__(em, _EngineCoupling(), scm, conn, dt, np.zeros(I, np.float32),
                         state0=_state0(m, N, state0), nparam=_slots_per_node(m, K, N),
                         delay_tables=(tables, tab_of), tpn=tpn, **kwargs)
        self.kernel_key = self.lems.path
        self.consts = K
        self.sigma = _sigma(self.lems, K, dt, noise)
        self.params = params

    def launch(self, launches=None, tpn=None, stream=None):
        "Enqueue the prepared launches on `stream` (no host sync)."
        launches = launches if launches is not None else self._uploaded
        tpn = tpn if tpn is not None else (self.tpn or 2)
        sh = nat.stream_handle(stream)
        for dev, n, smem, bk in launches:
            cfg = self._launch_cfg(smem, tpn, bk)
            self.lems.check(self.lems.lib.tvbg_lems_sweep(dev.data_ptr(), n, ctypes.byref(cfg), sh))

    def exposures(self, stream=None):
        "Exposures of the current state, (n_work, N, nexpo), on the device."
        torch = self.torch
        ne = len(self.lmodel.exposures)
        out = torch.empty((self.n, self.N, ne), dtype=torch.float32, device='cuda')
        self.lems.check(self.lems.lib.tvbg_lems_expose(self.state.data_ptr(), self.n * self.N,
                                                       out.data_ptr(), nat.stream_handle(stream)))
        return out


class LemsGroupSet(GroupSet):
    """
    Work items of one LEMS model on the lane-interleaved group kernel: eight
    work items sharing a delay table per group, time-blocked (K = 4 or 8 <=
    d_min + 1 steps per block).  Takes models whose coupling is separable
    (pre reads only x_j: its value is written into the ring) or a sine
    difference post * sin(x_j - x_i) (sin and cos ring channels); others
    need LemsSweep (ValueError here).  Short delays take short blocks
    (K = 2 for d_min = 1, K = 1 for zero delays).
    Noise needs one nsig for every work item.  Arguments as LemsSweep, plus
    GroupSet's block_k, threads, cluster, trace_*, bold_*.
    """

    block_ks = (8, 4, 2, 1)   # the generated libraries build every block length

    def __init__(self, m, conn, dt, params, state0=None, noise=None, single=False, **kwargs):
        self.lems = LemsLibrary(m, single)
        self.lmodel = m
        cls = self.lems.info['group']
        if cls == 0:
            raise ValueError('LEMS model %s: its coupling needs the per-step kernel' % m.name)
        if kwargs.get('history', 'zero') != 'zero':
            raise ValueError('LEMS groups start from zero history')
        noise = m.noise if noise is None else bool(noise)
        params, K, tables, tab_of = _setup(self.lems, m, conn, dt, params)
        I, N = params.shape[0], int(conn.nnode)
        sig = _sigma(self.lems, K, dt, noise)
        if noise and not np.all(sig == sig[0]):
            raise ValueError('LEMS groups need one nsig for every work item')
        # history before t0: the ring holds pre(0) of each work item (per
        # coupling); the sine coupling's channels hold (sin 0, cos 0)
        self._cls = cls
        self._f = None
        if cls in (1, 3):
            Kc = np.ascontiguousarray(K)
            self._f = []
            for which in range(1 if cls == 1 else 2):
                f = np.zeros(I, np.float32)
                self.lems.check(self.lems.lib.tvbg_lems_ring_value(Kc.ctypes.data, I, 0.0, which,
                                                                   f.ctypes.data))
                self._f.append(f)
        em = _EngineModel(m, noise)
        ec = _EngineCoupling({1: nat.CFUN_LEMS, 2: nat.CFUN_LEMS_SC, 3: nat.CFUN_LEMS_2}[cls])
        scm = sch.EulerMaryuyamaStep(dt) if noise else sch.EulerStep(dt)
        super().__init__(em, ec, scm, conn, dt, np.zeros(I, np.float32),
                         state0=_state0(m, N, state0), nparam=_slots_per_node(m, K, N),
                         delay_tables=(tables, tab_of), **kwargs)
        self.sigma = sig[0] if I else np.zeros(4, np.float32)
        self.consts = np.zeros(MAX_K, np.float32)
        self.params = params
        self.slots = K

    def clear_history(self):
        super().clear_history()
        fs = getattr(self, '_f', None)
        if fs is None or (self._cls == 1 and not np.any(fs[0] != 0)):
            return
        torch = self.torch
        N, C = self.N, self.channels
        for g, mem in enumerate(self.members):
            R = int(self.R[g])
            o = int(self.ring_off[g])
            v = np.zeros((C, L_GROUP), np.float32)
            for c, f in enumerate(fs):
                v[c, :mem.size] = f[mem]
            self.ring[o:o + N * R * C * L_GROUP].view(N, R, C, L_GROUP)[:] = torch.from_numpy(v).cuda()

    def _run_groups(self, dev_ptr, n, cfg, stream):
        self.lems.check(self.lems.lib.tvbg_lems_group_run(dev_ptr, n, ctypes.byref(cfg), stream))

    def exposures(self, stream=None):
        "Exposures of the current state, (n_work, N, nexpo), on the device."
        torch = self.torch
        st = self.state.contiguous()
        ne = len(self.lmodel.exposures)
        out = torch.empty((self.n, self.N, ne), dtype=torch.float32, device='cuda')
        self.lems.check(self.lems.lib.tvbg_lems_expose(st.data_ptr(), self.n * self.N,
                                                       out.data_ptr(), nat.stream_handle(stream)))
        return out


def make_set(m, conn, dt, params, prefer='groups', **kwargs):
    """The fastest set that takes the model: LemsGroupSet where the coupling
    and the delays allow it, else LemsSweep."""
    if prefer == 'groups':
        try:
            return LemsGroupSet(m, conn, dt, params, **{k: v for k, v in kwargs.items()
                                                         if k != 'tpn'})
        except ValueError:
            pass
    return LemsSweep(m, conn, dt, params, **kwargs)


def run_simulation(m, weights, lengths, params_matrix, dt, nstep, n_inner_steps, single=False,
                   noise=None, seed=0, tpn=None):
    """
    The launcher of dsl/dsl_cuda/example/cuda_run.py:67-142 on the engine:
    `nstep` launches of `n_inner_steps` steps for every work item (a row of
    params_matrix), returning the exposures after each launch as
    (nstep, n_nodes * nexpo, n_work) -- the reference's tavg layout -- and
    the set that ran them (LemsGroupSet where the coupling and delays allow,
    else LemsSweep).  weights and lengths are dense N x N.
    """
    from .network import Connectivity
    conn = Connectivity.from_dense(np.asarray(weights, np.float32), np.asarray(lengths, np.float32))
    sw = make_set(m, conn, dt, params_matrix, noise=noise, single=single, seed=seed, tpn=tpn)
    out = []
    for _ in range(int(nstep)):
        sw.run(int(n_inner_steps))
        e = sw.exposures()                     # (n_work, N, nexpo)
        out.append(e.permute(2, 1, 0).reshape(-1, sw.n))
    torch = sw.torch
    tavg = torch.stack(out).cpu().numpy() if out else np.zeros((0, sw.N, sw.n), np.float32)
    return tavg, sw
