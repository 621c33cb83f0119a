"""
Region mapping on the device (tvbg_rmap_to_avg / tvbg_rmap_from_avg): the
reference's own cases (tvb_hpc/tests.py:453-473) through the tvb_hpc API
with numpy arrays, and a large random map against a float64 sum.
"""

import numpy as np
import pytest

from tvb_hpc import network

pytestmark = pytest.mark.gpu


def test_rmap_to_avg(cuda):
    i = np.r_[:16].reshape((-1, 1))
    rmap = i // 4
    node = i.astype('f')
    roi = np.zeros((4, 1), 'f')
    network.RMapToAvg().kernel()(nroi=4, nvar=1, nnode=16, rmap=rmap, node=node, roi=roi)
    np.testing.assert_allclose(roi[:, 0], node.reshape((4, 4)).sum(axis=1))


def test_rmap_from_avg(cuda):
    i = np.r_[:16].reshape((-1, 1))
    rmap = i // 4
    node = np.zeros((16, 1), 'f')
    roi = np.r_[:4].reshape((4, 1)).astype('f')
    network.RMapFromAvg().kernel()(nroi=4, nvar=1, nnode=16, rmap=rmap, node=node, roi=roi)
    np.testing.assert_allclose(rmap, node)


def test_rmap_large_and_tensors(cuda):
    torch = cuda
    rng = np.random.default_rng(0)
    nnode, nroi, nvar = 515056, 68, 3
    rmap = rng.integers(0, nroi, nnode).astype(np.int32)
    rmap[:5] = [-1, nroi, nroi + 7, -3, 0]          # out of range: no region
    node = rng.normal(size=(nnode, nvar)).astype(np.float32)
    roi = torch.zeros((nroi, nvar), device='cuda')
    network.RMapToAvg().kernel()(nroi=nroi, nvar=nvar, nnode=nnode, rmap=torch.from_numpy(rmap).cuda(),
                                 node=torch.from_numpy(node).cuda(), roi=roi)
    ref = np.zeros((nroi, nvar))
    ok = (rmap >= 0) & (rmap < nroi)
    np.add.at(ref, rmap[ok], node[ok].astype(np.float64))
    np.testing.assert_allclose(roi.cpu().numpy(), ref, rtol=1e-4, atol=1e-3)
    back = np.full((nnode, nvar), 7.0, np.float32)
    network.RMapFromAvg().kernel()(nroi=nroi, nvar=nvar, nnode=nnode, rmap=rmap, node=back,
                                   roi=roi.cpu().numpy())
    np.testing.assert_array_equal(back[ok], roi.cpu().numpy()[rmap[ok]])
    assert np.all(back[~ok] == 7.0)
