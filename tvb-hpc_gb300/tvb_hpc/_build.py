"""
In-tree build of the engine library (nvcc, sm_103a) and of the checker.

    python -c "import __graft_entry__ as g; g.build()"

compiles tvb-hpc_gb300/csrc/*.cu in parallel (one nvcc per translation
unit, objects under tvb-hpc_gb300/_build/) and links
tvb_hpc/_lib/libtvbg.so with the CUDA runtime linked statically; then
compiles the libraries of the bundled LEMS models (tvb_hpc/lems_models/,
tvb_hpc/_lib/lems/).
"""

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, 'csrc')
OBJ = os.path.join(PKG_ROOT, '_build')
LIB = os.path.join(HERE, '_lib', 'libtvbg.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '-Xptxas', '-v',
         '--expt-relaxed-constexpr']


def nvcc():
    exe = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(exe):
        raise RuntimeError('nvcc not found')
    return exe


def _deps():
    return (glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(CSRC, '*.h'))
            + [os.path.join(os.path.dirname(PKG_ROOT), 'include', 'tvbg.h')])


def _stale(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(src, obj, extra):
    cmd = [nvcc()] + ARCH + FLAGS + extra + ['-c', src, '-o', obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    log = obj + '.log'
    with open(log, 'w') as f:
        f.write(' '.join(cmd) + '\n' + p.stdout + p.stderr)
    if p.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s' % (os.path.basename(src), p.stderr[-4000:]))
    return obj


def build(force=False, extra=(), jobs=None):
    "Compile every CUDA translation unit and link libtvbg.so; returns its path."
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    deps = _deps()
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + '.o')
        objs.append(o)
        if force or _stale(s, o, deps):
            todo.append((s, o))
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], list(extra)), todo))
    if todo or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ['-shared', '-cudart', 'static', '-o', LIB] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError('link failed:\n' + p.stderr[-4000:])
    from . import lems
    lems.prebuild(jobs)
    return LIB
