"""
Generate the golden fixtures under tests/golden/ (run in a container that
has the reference tree and the oracle/_ref build; outputs are committed).

  philox_triton.npz  Philox4x32-10 words from Triton's public randint4x
                     (interpreter mode on the CPU): counter = (offset, 0, 0, 0),
                     key = (seed_lo, seed_hi) -- a library implementation of
                     the Salmon et al. (2011) generator.
  hcp0.npz           the reference's own 84-node connectome fixture
                     (data/hcp0.npz), used by the hackathon known-answer test.
  ref_kuramoto.npz   the reference CUDA DSL Kuramoto kernel
                     (dsl/dsl_cuda/CUDAmodels/kuramoto.c) compiled for the host
                     by oracle/Makefile with noise stubbed out, run one thread
                     per instance as cuda_run.py launches it.
  ref_balloon.npz    refs/balloon.c bold_update, host-compiled, 300 steps of
                     a constant input per node.
  ref_covar.npz      refs/covar.c update_cov + cov_to_corr, host-compiled.

    python tests/golden/make_golden.py [REFERENCE_ROOT]
"""

import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
sys.path.insert(0, os.path.join(ROOT, 'tvb-hpc_gb300'))


def philox_triton():
    os.environ['TRITON_INTERPRET'] = '1'
    import torch
    import triton
    import triton.language as tl

    @triton.jit
    def k(out_ptr, seed, N: tl.constexpr):
        off = tl.arange(0, N)
        a, b, c, d = tl.randint4x(seed, off)
        tl.store(out_ptr + off * 4 + 0, a)
        tl.store(out_ptr + off * 4 + 1, b)
        tl.store(out_ptr + off * 4 + 2, c)
        tl.store(out_ptr + off * 4 + 3, d)

    seeds = [0, 12345, 0x0BADC0DE, 0x0EADBEEFCAFEBABE]
    n = 256
    words = []
    for s in seeds:
        out = torch.zeros(4 * n, dtype=torch.int32)
        k[(1, )](out, s, N=n)
        words.append(out.numpy().view(np.uint32).reshape(n, 4))
    np.savez_compressed(os.path.join(HERE, 'philox_triton.npz'),
                        seeds=np.array(seeds, np.uint64), words=np.stack(words))


def ref_kuramoto(ref):
    import pyoracle
    from tvb_hpc.network import synthetic_connectome
    lib = pyoracle.load_ref()
    N, n_work, n_step = 24, 4, 300
    w, ln = synthetic_connectome(N, 0.3, seed=7)
    speeds = np.array([2.0, 3.0, 4.0, 5.0], np.float32)
    couplings = np.array([0.5, 1.0, 2.0, 4.0], np.float32)
    dt = np.float32(0.1)
    dmax = int((ln / speeds.min() / dt).max()) + 1
    nh = int(2 ** np.ceil(np.log2(dmax + 2)))
    params = np.stack([speeds, couplings]).astype(np.float32)          # [2][n_work]
    state = np.zeros((nh, N, n_work), np.float32)
    tavg = np.zeros((N, n_work), np.float32)
    chunks = [100, 100, 100]
    t = 0
    for c in chunks:
        lib.ref_kuramoto(t, N, nh, c, dt, w.ctypes.data, ln.ctypes.data, params.ctypes.data,
                         state.ctypes.data, tavg.ctypes.data, n_work)
        t += c
    np.savez_compressed(os.path.join(HERE, 'ref_kuramoto.npz'), weights=w, lengths=ln,
                        speeds=speeds, couplings=couplings, dt=dt, nh=nh, n_step=n_step,
                        chunks=np.array(chunks), state=state, tavg=tavg)


def ref_balloon(ref):
    "balloon.c driven by a constant input per node (ms step 1.0 -> 1e-3 s)."
    import pyoracle
    lib = pyoracle.load_ref()
    N, nt, steps = 5, 1, 300
    x0 = np.linspace(-0.5, 0.5, N).astype(np.float32)
    bold = np.zeros((4, N, nt), np.float32)
    bold[1:] = 1
    out = np.zeros((steps, N), np.float32)
    dt = np.float32(1e-3)
    for k in range(steps):
        o = np.zeros((N, nt), np.float32)
        xx = np.ascontiguousarray(x0[:, None])
        lib.ref_bold_update(N, dt, bold.ctypes.data, xx.ctypes.data, o.ctypes.data, nt)
        out[k] = o[:, 0]
    np.savez_compressed(os.path.join(HERE, 'ref_balloon.npz'), x0=x0, out=out, dt_ms=1.0)


def ref_covar(ref):
    import pyoracle
    lib = pyoracle.load_ref()
    T, N = 40, 12
    rng = np.random.default_rng(5)
    x = rng.normal(0, 1, (T, N)).astype(np.float32) + np.linspace(0, 1, N, dtype=np.float32)
    cov = np.zeros((N, N), np.float32)
    means = np.zeros((2, N), np.float32)
    for s in range(T):
        row = np.ascontiguousarray(x[s])
        lib.ref_update_cov(s, N, cov.ctypes.data, means.ctypes.data, row.ctypes.data)
    corr = np.zeros((N, N), np.float32)
    lib.ref_cov_to_corr(T, N, cov.ctypes.data, corr.ctypes.data)
    np.savez_compressed(os.path.join(HERE, 'ref_covar.npz'), x=x, corr=corr)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('TVB_HPC_REFERENCE', '')
    if not ref:
        sys.exit('usage: make_golden.py <tvb-hpc checkout> (or set TVB_HPC_REFERENCE)')
    import subprocess
    subprocess.run(['make', '-s', '-C', os.path.join(ROOT, 'oracle')], check=True)
    subprocess.run(['make', '-s', '-C', os.path.join(ROOT, 'oracle'), 'ref', 'REF=' + ref],
                   check=True)
    shutil.copyfile(os.path.join(ref, 'data', 'hcp0.npz'), os.path.join(HERE, 'hcp0.npz'))
    ref_kuramoto(ref)
    ref_balloon(ref)
    ref_covar(ref)
    philox_triton()
    print('golden fixtures written to', HERE)


if __name__ == '__main__':
    main()
