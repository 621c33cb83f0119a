"""
GPU Philox generator and FC kernel against the oracle.
  - raw Philox4x32-10 words: bit-exact with the oracle (itself pinned to
    Triton's randint4x);
  - normals: Box-Muller in float vs double, |diff| < 2e-5, plus the
    reference's statistical test (tvb_hpc/tests.py:329-342: KS, mean, std);
  - FC: FP64-reduced Pearson vs the oracle (and np.corrcoef) to 1e-6.
"""

import numpy as np
import pytest
from scipy.stats import kstest

import pyoracle as orc
from tvb_hpc import rng as trng, metric

pytestmark = pytest.mark.gpu


def test_philox_words_bit_exact(cuda):
    for k0, k1, c1, c2 in [(0, 0, 0, 0), (12345, 7, 0, 3), (0xdeadbeef, 0xcafebabe, 99, 1)]:
        got = trng.philox_u32(k0, k1, 4096, c1=c1, c2=c2)
        np.testing.assert_array_equal(got, orc.philox_u32(k0, k1, 4096, c1, c2))


def test_philox_normals_match_oracle_and_are_normal(cuda):
    a = np.zeros(1024 * 1024, np.float32)
    trng.RNG().build().fill(a, seed=42)
    ref = orc.philox_normal(42, 0, a.size)
    assert np.abs(a - ref).max() < 2e-5
    d, p = kstest(a, 'norm')
    assert abs(a.mean()) < 1e-2 and abs(a.std() - 1) < 1e-2
    assert d < 0.01


@pytest.mark.parametrize('I,T,N', [(8, 13, 84), (3, 200, 68), (2, 64, 192)])
def test_fc_matches_oracle(cuda, I, T, N):
    torch = cuda
    rng = np.random.default_rng(N)
    x = (rng.normal(size=(I, T, N)) + rng.normal(size=(I, 1, N)) * 3).astype(np.float32)
    target = np.corrcoef(rng.normal(size=(N, 40)))
    fc, err = metric.fc(torch.from_numpy(x).cuda(), target)
    fc = fc.cpu().numpy()
    for b in range(I):
        ref = orc.fc(x[b])
        np.testing.assert_allclose(fc[b], ref, atol=1e-6)
        np.testing.assert_allclose(ref, np.corrcoef(x[b].T.astype(np.float64)), atol=1e-12)
    np.testing.assert_allclose(err.cpu().numpy(), metric.fc_error(
        np.stack([orc.fc(x[b]) for b in range(I)]), target), rtol=1e-9)
