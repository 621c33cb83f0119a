"""
Utilities mirroring tvb_hpc/utils.py: logger, timer, symbolic helpers.

tvb-hpc parses expressions with pymbolic; here sympy does the parsing (every
identifier becomes a Symbol, so names such as ``I`` or ``E`` stay plain
variables).  Only what the step path and the reference's tests need is kept.
"""

import logging
import re
import time

import numpy as np
import sympy

_FUNCS = {
    'sin': sympy.sin, 'cos': sympy.cos, 'tan': sympy.tan, 'exp': sympy.exp,
    'log': sympy.log, 'sqrt': sympy.sqrt, 'tanh': sympy.tanh, 'abs': sympy.Abs,
    'sqrtf': sympy.sqrt, 'expf': sympy.exp, 'sinf': sympy.sin, 'cosf': sympy.cos,
}
_IDENT = re.compile(r'[A-Za-z_][A-Za-z_0-9]*')


def getLogger(name):
    "utils.py:39-40"
    return logging.getLogger(name)


def parse(expr):
    "Parse an expression string into sympy; every identifier is a Symbol."
    if isinstance(expr, (int, float, np.number)):
        return sympy.Float(expr) if isinstance(expr, float) else sympy.Integer(int(expr))
    if isinstance(expr, sympy.Basic):
        return expr
    s = str(expr)
    local = {}
    for name in set(_IDENT.findall(s)):
        local[name] = _FUNCS.get(name, sympy.Symbol(name))
    return sympy.parsing.sympy_parser.parse_expr(s, local_dict=local, evaluate=False)


def vars(svars):
    "Array of symbols from space-separated names (utils.py:67-73)."
    return np.array([sympy.Symbol(v) for v in str(svars).split()], dtype=object)


def exprs(sexprs):
    "Array of parsed expressions (utils.py:76-90)."
    out = []
    for e in sexprs:
        try:
            out.append(parse(e))
        except Exception as exc:  # noqa: BLE001 - mirror reference message
            raise Exception(repr(e)) from exc
    return np.array(out, dtype=object)


def free_names(expr):
    "Names of the free symbols of an expression."
    return sorted(s.name for s in parse(expr).free_symbols)


def simplify(expr):
    "Simplify via sympy (utils.py:59-64)."
    return sympy.simplify(parse(expr))


class VarSubst:
    "Substitute variables by name (utils.py:110-120)."

    def __init__(self, verbose=False, **substs):
        self.verbose = verbose
        self.substs = {k: parse(v) for k, v in substs.items()}

    def __call__(self, expr):
        e = parse(expr)
        return e.xreplace({sympy.Symbol(k): v for k, v in self.substs.items()})


def subst_vars(expr, **var_name_to_exprs):
    "utils.py:123-125"
    return VarSubst(**var_name_to_exprs)(expr)


class timer:
    "Wall-clock context manager that logs (utils.py:93-107)."
    logger = getLogger('tvb_hpc.utils.timer')

    def __init__(self, msg=''):
        self.msg = msg

    def __enter__(self, *args):
        self.tic = time.time()
        return self

    def __exit__(self, *args):
        self.elapsed = time.time() - self.tic
        self.logger.info('%s elapsed %.3fs', self.msg, self.elapsed)


def next_pow2(n):
    "Smallest power of two >= n (n >= 1)."
    n = int(n)
    return 1 << max(0, (n - 1).bit_length())
