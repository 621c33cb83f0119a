"""
The tvb_hpc API mirror (no GPU needed): attribute schema, coupling io and
post-stat rules (tvb_hpc/tests.py:345-365), region maps failing loudly
without a device (their values: tests/test_gpu_rmap.py),
connectivity CSR (network.py:66-78), synthetic connectomes, and the rule
that models or couplings without a hand-written kernel are rejected.
"""

import numpy as np
import pytest
from scipy import sparse

from tvb_hpc import model, coupling, scheme, network, bold, metric, utils
from tvb_hpc.coupling import PostSumStat


def test_post_stat():
    assert coupling.Linear(model.G2DO()).post_stat(0) == PostSumStat.sum
    assert coupling.Diff(model.G2DO()).post_stat(0) == PostSumStat.sum
    assert coupling.Sigmoidal(model.JansenRit()).post_stat(0) == PostSumStat.sum
    assert coupling.Kuramoto(model.Kuramoto()).post_stat(0) == PostSumStat.mean


def test_io_truncates_obsrv_to_inputs():
    "coupling.py:68-84: G2DO has one input, so it couples obsrv[0] = W."
    cf = coupling.Diff(model.G2DO())
    assert len(cf.io) == 1 and str(cf.io[0][0]) == 'W'
    cf = coupling.Kuramoto(model.Kuramoto())
    assert str(cf.io[0][0]) == 'theta'


def test_models_parse_and_prep_arrays():
    for M in (model.Kuramoto, model.G2DO, model.MPR, model.Linear, model.RWW, model.JansenRit,
              model.HMJE, model._TestModel, bold.BalloonWindkessel):
        m = M()
        arrs = m.prep_arrays(7)
        assert [a.shape for a in arrs] == [(7, len(getattr(m, k + '_sym'))) for k in
                                           'state input param drift diffs obsrv'.split()]
        for i, (lo, hi) in enumerate(m.limit):
            lo, hi = min(lo, hi), max(lo, hi)  # HMJE lists y1 as (20, 2)
            assert np.all(arrs[0][:, i] >= lo) and np.all(arrs[0][:, i] <= hi)


def test_engine_spec_rejects_unbuilt_or_edited():
    with pytest.raises(NotImplementedError):
        model.HMJE().engine_spec()
    kid, consts, sigma = model.RWW().engine_spec()
    assert kid == 5 and consts[5] == np.float32(0.2609) and sigma[0] == np.float32(0.01)
    kid, consts, sigma = model.JansenRit().engine_spec()
    assert kid == 6 and consts[0] == np.float32(3.25) and consts[10] == np.float32(0.22)
    assert np.all(sigma == 0)

    class NoisyJR(model.JansenRit):
        diffs = 0, 0, 0, 0, 0, 1e-3
    with pytest.raises(NotImplementedError):
        NoisyJR().engine_spec()

    class Edited(model.Kuramoto):
        drift = 'omega + 2 * I',
    with pytest.raises(NotImplementedError):
        Edited().engine_spec()

    class Sub(model.G2DO):
        pass
    kid, consts, sigma = Sub().engine_spec()
    assert kid == 1 and consts[4] == np.float32(0.02) and sigma[0] == np.float32(1e-3)

    class MyCf(coupling.Linear):
        pre_sum = 'pre_syn * 2',
    with pytest.raises(NotImplementedError):
        MyCf(model.Linear()).engine_spec()


def test_const_edits_are_per_instance():
    a = model.Kuramoto()
    a.const['omega'] = 3.0
    assert model.Kuramoto().const['omega'] == 1.0
    assert a.node_params(4)[0, 0] == 3.0


def test_connectivity_from_dense_matches_scipy():
    rng = np.random.default_rng(0)
    w = (rng.random((20, 20)) < 0.3) * rng.random((20, 20))
    ln = rng.uniform(10, 100, (20, 20))
    c = network.Connectivity.from_dense(w.astype(np.float32), ln.astype(np.float32))
    s = sparse.csr_matrix(w.astype(np.float32))
    assert np.array_equal(c.row, s.indptr) and np.array_equal(c.col, s.indices)
    assert np.array_equal(c.wnz, s.data) and c.nnz == s.nnz
    assert np.array_equal(c.lnz, ln.astype(np.float32)[w != 0])


def test_synthetic_connectome_recipe():
    w, ln = network.synthetic_connectome(68, 0.3, seed=0)
    assert w.shape == (68, 68) and np.allclose(w, w.T) and np.all(np.diag(w) == 0)
    assert w.max() == 1.0
    dens = (w > 0).sum() / (68 * 67)
    assert 0.25 < dens < 0.35
    nz = ln[w > 0]
    assert nz.min() >= 10 and nz.max() <= 200 and np.allclose(ln, ln.T)
    w2, _ = network.synthetic_connectome(68, 0.3, seed=0)
    assert np.array_equal(w, w2)


def test_rmap_needs_the_device():
    "Region mapping runs on the GPU kernels only: without a device it fails loudly."
    import torch
    if torch.cuda.is_available():
        pytest.skip('a CUDA device is present')
    i = np.r_[:16].reshape((-1, 1))
    with pytest.raises(RuntimeError):
        network.RMapToAvg().kernel()(nroi=4, nvar=1, nnode=16, rmap=i // 4, node=i.astype('f'),
                                     roi=np.zeros((4, 1), 'f'))


def test_scheme_symbolics():
    m = model._TestModel()
    logp = scheme.euler_maruyama_logp(m.state_sym, m.drift_sym, m.diffs_sym).sum()
    parts = m.partial(logp)
    assert len(parts) == len(m.indvars)
    assert scheme.EulerStep(0.1).dt_value() == 0.1
    assert scheme.EulerStep('dt').dt_value({'dt': 0.5}) == 0.5
    assert scheme.EulerMaryuyamaStep(0.1).noise and not scheme.EulerStep(0.1).noise


def test_var_subst():
    e = utils.subst_vars('a + b * pre_syn', b='c + 1')
    assert str(e.expand()) == str(utils.parse('a + c*pre_syn + pre_syn').expand())


def test_fc_error_and_host_covariances():
    rng = np.random.default_rng(2)
    x = rng.normal(size=(100, 6))
    oc = metric.OnlineCov(6)
    for row in x:
        oc.update(row)
    np.testing.assert_allclose(oc.cov, metric.BatchCov()(x), rtol=1e-10, atol=1e-10)
    fc = np.corrcoef(x.T)
    assert metric.fc_error(fc, fc) == 0.0
