"""
The FC-fit Gram's FP32 arithmetic (fcfit_gram_split_kernel in
csrc/tvbg_fcgrad.cu) restated in numpy, no GPU: every FP32 operation is a
numpy float32 operation (IEEE round-to-nearest), TwoProduct's error term and
the kernel's FMAs are formed exactly in float64 and rounded once.  Checks the
documented error bound -- below 4e-12 of ||c_i|| ||c_j|| -- against a float64
two-pass centred Gram, on a stationary series and on a drifting one (a decay
transient, where the mean sits far from most samples).
"""

import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fma32(a, b, c):
    "fmaf: a b + c formed in float64 (exact for the magnitudes here), rounded once."
    return f32(a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64))


def split_gram(x, mean, L=32):
    """The kernel's arithmetic for the upper triangle (i <= j) of G."""
    T, N = x.shape
    mh = mean.astype(f32)
    ml = (mean - mh.astype(np.float64)).astype(f32)
    d, de = two_sum(x, -mh[None, :])
    hi, lo = two_sum(d, f32(de - ml[None, :]))
    iu, ju = np.triu_indices(N)
    ah = np.zeros(iu.size, f32)
    al = np.zeros(iu.size, f32)
    for t0 in range(0, T, L):
        s = np.zeros(iu.size, f32)
        cp = np.zeros(iu.size, f32)
        sm = np.zeros(iu.size, f32)
        for t in range(t0, min(T, t0 + L)):
            xi, yj = hi[t, iu], hi[t, ju]
            li, lj = lo[t, iu], lo[t, ju]
            p = f32(xi * yj)
            e = f32(xi.astype(np.float64) * yj.astype(np.float64) - p.astype(np.float64))
            sm = f32(sm + fma32(xi, lj, fma32(li, yj, e)))
            s, err = two_sum(s, p)
            cp = f32(cp + err)
        h, l_ = two_sum(ah, s)
        l_ = f32(l_ + f32(al + f32(cp + sm)))
        ah, al = two_sum(h, l_)
    G = np.zeros((N, N))
    G[iu, ju] = ah.astype(np.float64) + al.astype(np.float64)
    G[ju, iu] = G[iu, ju]
    return G


def check(x):
    x = x.astype(f32)
    x64 = x.astype(np.float64)
    mean = x64.mean(0)
    c = x64 - mean
    ref = c.T @ c
    got = split_gram(x, mean)
    nrm = np.sqrt(np.diag(ref))
    err = np.abs(got - ref) / np.outer(nrm, nrm)
    return float(err.max())


def test_split_gram_error_bound():
    rng = np.random.default_rng(0)
    T, N = 2000, 24
    # stationary rates around 0.1
    e1 = check(0.1 + 0.02 * rng.standard_normal((T, N)))
    # a decay transient: the mean sits far from the late samples
    t = np.arange(T)[:, None]
    e2 = check(0.3 * np.exp(-t / 150.0) + 0.002 * rng.standard_normal((T, N)))
    # correlated columns (FC near 1 off the diagonal)
    base = rng.standard_normal((T, 1))
    e3 = check(0.5 + base + 1e-3 * rng.standard_normal((T, N)))
    for e in (e1, e2, e3):
        assert e < 4e-12, (e1, e2, e3)
    print('split Gram error / (||c_i|| ||c_j||): %.1e %.1e %.1e' % (e1, e2, e3))
