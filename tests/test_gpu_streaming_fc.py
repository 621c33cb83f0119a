"""
Streaming FC (tvbg_cov_update / tvbg_cov_corr) against the two-pass FP64
FC kernel (tvbg_fc) and the oracle: after T folded samples the correlation
agrees to 1e-6 (both reductions are FP64; the outputs are float32).
"""

import numpy as np
import pytest

import pyoracle as orc
from tvb_hpc import metric

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('I,T,N', [(6, 40, 84), (3, 200, 68), (2, 30, 400)])
def test_streaming_fc_matches_two_pass(cuda, I, T, N):
    torch = cuda
    rng = np.random.default_rng(N)
    x = (rng.normal(size=(I, T, N)) + rng.normal(size=(I, 1, N)) * 5).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    s = metric.StreamingFC(I, N)
    s.update_rows(xd, range(T))         # strided rows of [I, T, N]
    got = s.corr().cpu().numpy()
    ref = metric.fc(xd)
    np.testing.assert_allclose(got, ref.cpu().numpy(), atol=1e-6)
    np.testing.assert_allclose(got[0], orc.fc(x[0]), atol=1e-6)
    # means are the sample means
    np.testing.assert_allclose(s.mean.cpu().numpy(), x.astype(np.float64).mean(axis=1), rtol=1e-12)


def test_streaming_fc_restart_needs_no_clearing(cuda):
    torch = cuda
    rng = np.random.default_rng(1)
    a = torch.from_numpy(rng.normal(size=(4, 25, 30)).astype(np.float32)).cuda()
    b = torch.from_numpy(rng.normal(size=(4, 25, 30)).astype(np.float32)).cuda()
    s = metric.StreamingFC(4, 30)
    s.update_rows(a, range(25))
    s.n = 0                             # a new stream reuses the state arrays
    s.update_rows(b, range(25))
    np.testing.assert_allclose(s.corr().cpu().numpy(), metric.fc(b).cpu().numpy(), atol=1e-6)
