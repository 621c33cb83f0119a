"""Shared test setup: import paths, the `gpu` marker, common fixtures."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, 'tvb-hpc_gb300'), os.path.join(ROOT, 'oracle')):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


@pytest.fixture(scope='session')
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from tvb_hpc import _native
    _native.load()
    return torch


def circ_rel_err(got, ref):
    "max circular distance / max |ref| (Kuramoto phases)."
    d = np.abs(np.angle(np.exp(1j * (np.asarray(got, np.float64) - np.asarray(ref, np.float64)))))
    return d.max() / max(np.abs(ref).max(), 1e-30)


def rel_err(got, ref):
    "max |got - ref| / max |ref| (the relative state error used in every parity test)."
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-30)
