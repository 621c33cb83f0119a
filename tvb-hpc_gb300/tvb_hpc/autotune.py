"""
Project-written autotuner for the step kernel's launch shape.

For a given instance set it times a short trial of every gather width
(lanes per node, tpn in {1, 2, 4, 8}) with CUDA events on the launching
stream and keeps the fastest.  Trials run on snapshots of the device state,
so tuning leaves the simulation untouched.  Results are cached per
(model, coupling, N, nnz, ring sizes) key for the life of the process.
"""

import numpy as np

from .utils import getLogger

LOG = getLogger(__name__)

_CACHE = {}
TPN_CHOICES = (1, 2, 4, 8)


def _key(iset):
    return (iset.model_id, iset.cfun_id, getattr(iset, 'kernel_key', None), iset.N, iset.nnz,
            tuple(sorted(set(int(x) for x in iset.lognh))), bool(iset.bold is not None),
            tuple(sorted(set(int(k) for k in iset.block_k))), iset.warps)


def tune_tpn(iset, trial_steps=None, choices=TPN_CHOICES):
    """Pick the launch shape of a Sweep by timing `trial_steps` steps of each
    choice: the gather width tpn and, for the time-blocked kernel, the CTA
    width in warps (unless the caller fixed it)."""
    import torch
    key = _key(iset)
    if key in _CACHE:
        return _CACHE[key]
    if trial_steps is None:
        trial_steps = int(np.clip(20000 // max(1, iset.n), 50, 400))
    snap = [t.clone() if t is not None else None
            for t in (iset.ring, iset.state, iset.bold, iset.bold_out, iset.trace)]
    blocked = bool(np.any(iset.block_k > 0))
    if np.all(iset.block_k > 0):
        choices = tuple(c for c in choices if c >= 2)
    fixed_warps = iset.warps
    warp_choices = ((fixed_warps, ) if fixed_warps or not blocked else
                    tuple(w for w in (4, 8, 16, 32) if 32 * w >= iset.N and 32 * w <= 1024))
    best, best_ms, best_w = choices[0], None, fixed_warps
    for wv in warp_choices:
        iset.warps = wv
        launches = iset.prepare(trial_steps)
        for tpn in choices:
            iset.launch(launches, tpn)  # warm-up (also loads the module)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            iset.launch(launches, tpn)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            LOG.debug('warps=%s tpn=%d: %.3f ms for %d steps', wv, tpn, ms, trial_steps)
            if best_ms is None or ms < best_ms:
                best, best_ms, best_w = tpn, ms, wv
    iset.warps = best_w
    for dst, src in zip((iset.ring, iset.state, iset.bold, iset.bold_out, iset.trace), snap):
        if dst is not None:
            dst.copy_(src)
    iset.status.reset()
    _CACHE[key] = best
    LOG.info('autotune %r -> tpn=%d (%.3f ms / %d steps)', key, best, best_ms, trial_steps)
    return best
