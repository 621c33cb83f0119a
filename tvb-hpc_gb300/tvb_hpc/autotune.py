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


# -- lane-interleaved group batches ---------------------------------------------

SHAPE_CLUSTERS = (1, 2, 3, 4, 6, 8, 12, 16)
_GROUP_CACHE = {}


def group_shapes(N, min_threads=128, clusters=SHAPE_CLUSTERS, pipelined=False):
    """Candidate launch shapes (threads, cluster, 0, tpn) of a group of N
    nodes: one node per 8-lane slot spread over C CTAs of a cluster, each
    distinct CTA width once (on its smallest cluster), CTAs of
    min_threads..1024 threads (tpn 1); when no shape qualifies, the default
    rule (several nodes per slot).  With `pipelined`, also the pipelined
    kernel's shapes (two teams per CTA, tpn 2)."""
    from .groups import L, group_shape, pipelined_threads, PIPELINED
    out, seen = [], set()
    for c in clusters:
        per = -(-N // c)
        thr = 32 * -(-(L * per) // 32)
        if thr > 1024 or thr in seen or (thr < min_threads and out):
            continue
        seen.add(thr)
        out.append((thr, c, 0, 1))
    if not out:
        out = [group_shape(N) + (0, 1)]
    if pipelined:
        seen = set()
        for c in clusters:
            thr = pipelined_threads(N, c)
            if not thr or thr in seen or thr < 2 * min_threads:
                continue
            seen.add(thr)
            out.append((thr, c, 0, PIPELINED))
    return out


def group_max_clusters(gset, threads, cluster, tpn=1):
    """Clusters of `cluster` CTAs of `threads` threads of gset's group kernel
    (tpn 2: the pipelined one) that can be resident at once (0: the shape
    cannot be launched)."""
    import ctypes
    from . import _native as nat
    cfg = gset.launch_cfg(int(gset.block_k.max()))
    cfg.threads, cfg.cluster, cfg.tpn = int(threads), int(cluster), int(tpn)
    n = ctypes.c_int32(0)
    nat.check(nat.load().tvbg_group_max_clusters(ctypes.byref(cfg), ctypes.byref(n)))
    return int(n.value)


def _snapshot(sets):
    names = ('ring', 'gstate', 'gbold', 'gbold_out', 'gtrace')
    return [[(n, getattr(s, n).clone()) for n in names if getattr(s, n) is not None] for s in sets]


def _restore(sets, snap):
    for s, saved in zip(sets, snap):
        for n, t in saved:
            getattr(s, n).copy_(t)
        s.status.reset()


def _batch_key(sets, nsteps):
    import torch
    dev = torch.cuda.get_device_name(torch.cuda.current_device())
    parts = []
    for s, n in zip(sets, nsteps):
        gmax = [int(np.max(n[m])) for m in s.members]
        parts.append((s.model_id, s.cfun_id, s.N, s.nnz, s.flags, s.channels,
                      tuple(sorted(set(int(x) for x in s.lognh))),
                      tuple(sorted(set(int(k) for k in s.block_k))), tuple(gmax)))
    return (dev, tuple(parts))


def _time_batch(sets, nsteps, shapes, reps=2, step_ms=None):
    "Best of `reps` event-timed launches of the batch with the given shapes (ms)."
    import torch
    from .groups import GroupBatch
    b = GroupBatch(sets, nsteps, shapes=shapes, step_ms=step_ms)
    main = torch.cuda.current_stream()
    b.launch(main)  # warm-up (module load, first dispatch)
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(main)
        b.launch(main)
        e1.record(main)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    b.status.check()
    return best


def _scaled(nsteps, trial_max_steps):
    longest = max(int(n.max(initial=0)) for n in nsteps)
    scale = max(1.0, longest / float(trial_max_steps))
    return [np.maximum(1, np.ceil(n / scale)).astype(np.int64) for n in nsteps], scale


def _alone_times(gset, small, reps):
    times = {}
    for shape in group_shapes(gset.N, pipelined=gset.can_pipeline):
        if group_max_clusters(gset, shape[0], shape[1], shape[3]) > 0:
            times[shape] = _time_batch([gset], [small], [shape], reps)
    return times


def tune_group_batch(sets, nsteps, trial_max_steps=4096, passes=2, reps=2, verify=True):
    """
    Launch shapes and dispatch priorities of a batch of GroupSets
    (tvbg_group_run launches on forked streams) that minimise the batch's
    makespan, found by measurement.

    A group's steps run in sequence on its cluster, and the launches of all
    sets share the SMs, so the batch ends when its last group does: a
    makespan over many jobs of different lengths that also contend for the
    L2 and the SMs.  The tuner
      1. times every set alone on each candidate shape (group_shapes: CTA
         width, cluster size up to 16 CTAs, plain or pipelined kernel), at
         step counts scaled down by one factor (the longest to about
         trial_max_steps): each shape's step time, hence each group's run
         time;
      2. starting from the better of the default shapes and each set's
         fastest shape alone, tries every candidate shape of one set at a
         time (sets with the longest chains first) on whole-batch trials at
         the scaled step counts, and keeps a change that shortens the batch;
      3. bands the groups of every set by run time into launch priorities
         (GroupBatch.group_priorities: the CTAs of the longest groups of the
         whole batch dispatched first) and keeps the banding if it measures
         faster.
    With `verify` the chosen plan and the default are timed once more at
    full length and the faster is kept.  Device state is restored
    afterwards; results are cached per device and batch signature for the
    life of the process.

    Returns dict(shapes=[(threads, cluster, 0, tpn) per set], step_ms (per
    set, or None without banding), ms (scaled trial of the plan), default_ms,
    scale, trials=[(plan, banded, ms)], alone=[{shape: ms} per set], and with
    `verify` full_ms / full_default_ms).
    The reference exposes the CUDA launch shape as a command-line tunable
    (dsl/dsl_cuda/example/cuda_setup.py:53-86, used by cuda_run.py:109-136);
    this picks it per connectome and orders the dispatch.
    """
    import torch
    nsteps = [np.broadcast_to(np.asarray(n, np.int64), (s.n, )).astype(np.int64)
              for s, n in zip(sets, nsteps)]
    key = _batch_key(sets, nsteps)
    if key in _GROUP_CACHE:
        return _GROUP_CACHE[key]
    small, scale = _scaled(nsteps, trial_max_steps)
    default = [(s.threads, s.cluster, 0, 1) for s in sets]
    snap = _snapshot(sets)
    trials = []
    try:
        alone = []
        for s, n, d in zip(sets, small, default):
            times = _alone_times(s, n, reps)
            if d not in times:
                times[d] = _time_batch([s], [n], [d], reps)
            alone.append(times)

        def step_ms(plan):
            return [alone[i][tuple(plan[i])] / float(small[i].max(initial=1))
                    for i in range(len(sets))]

        def measure(plan, banded=False):
            ms = _time_batch(sets, small, plan, reps, step_ms(plan) if banded else None)
            trials.append((tuple(plan), banded, round(ms, 4)))
            return ms

        default_ms = measure(default)
        fastest = [min(a, key=a.get) for a in alone]
        best, plan = default_ms, list(default)
        ms = measure(fastest)
        if ms < best:
            best, plan = ms, list(fastest)
        order = sorted(range(len(sets)), key=lambda i: -float(nsteps[i].max(initial=0)) * sets[i].N)
        for _ in range(passes):
            changed = False
            for i in order:
                for shape in alone[i]:
                    if shape == tuple(plan[i]):
                        continue
                    cand = list(plan)
                    cand[i] = shape
                    ms = measure(cand)
                    if ms < best * 0.99:
                        plan, best, changed = cand, ms, True
            if not changed:
                break
        banded_ms = measure(plan, banded=True)
        banded = banded_ms < best * 0.99
        if banded:
            best = banded_ms
        result = dict(shapes=[tuple(int(x) for x in p) for p in plan],
                      step_ms=step_ms(plan) if banded else None, ms=best, default_ms=default_ms,
                      scale=scale, trials=trials,
                      alone=[{k: round(v, 4) for k, v in a.items()} for a in alone])
        if verify and (plan != default or banded):
            full_default = _time_batch(sets, nsteps, default, 1)
            full_plan = _time_batch(sets, nsteps, plan, 1, result['step_ms'])
            result.update(full_default_ms=full_default, full_ms=full_plan)
            if full_plan >= full_default:
                result.update(shapes=list(default), step_ms=None, ms=default_ms,
                              kept_default=True)
    finally:
        _restore(sets, snap)
        torch.cuda.synchronize()
    for s, sh in zip(sets, default):
        s.set_shape(*sh)
    _GROUP_CACHE[key] = result
    LOG.info('group batch tuned: %s banded=%s (%.3f ms scaled, default %.3f ms, %d trials)',
             result['shapes'], result['step_ms'] is not None, result['ms'], result['default_ms'],
             len(trials))
    return result


def tune_group_alone(gset, nsteps, trial_max_steps=4096, reps=2):
    """Fastest launch shape of one GroupSet run alone (its own launches only):
    every candidate of group_shapes timed on the set's step counts scaled to
    about trial_max_steps.  Returns ((threads, cluster, 0, tpn), {shape: ms})."""
    import torch
    n = np.broadcast_to(np.asarray(nsteps, np.int64), (gset.n, )).astype(np.int64)
    small, _ = _scaled([n], trial_max_steps)
    snap = _snapshot([gset])
    old = gset.shape
    try:
        times = _alone_times(gset, small[0], reps)
    finally:
        _restore([gset], snap)
        gset.set_shape(*old)
        torch.cuda.synchronize()
    best = min(times, key=times.get)
    return best, times
