"""
Benchmark of the GB300 brain-network step engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
    python bench.py --impl reference ...      (the CPU arm, host cores)

One bench "step" is one full pass of the workload: every instance of the
sweep is reset to its seeded initial state (device-resident copy) and run
for all of its time steps (then, for the grid, the per-instance FC is
computed).  The workload sizes are those of the benchmark configurations
(seeded synthetic connectomes; there is no dataset):

  mixed  (default) uneven batch: connectomes of N in {68, 84, 192, 400, 998}
         (30/30/15/8/3% density), 1024/1024/256/64/16 instances, step counts
         uniform in [5k, 50k], Montbrio-Pazo-Roxin with linear coupling and
         Euler-Maruyama noise (sigma 1e-2), max delay 500 steps; run as one
         CUDA graph of lane-interleaved group launches (one per connectome,
         forked streams).  The plain path (per-step kernel, one sweep per
         connectome in 1000-step launches, connectomes in sequence) is timed
         on the same work and reported beside it.
  grid   dense parameter grid: generic 2-D oscillator (the CUDA DSL / TVB
         form, cubic and coupling on V) with linear difference coupling and
         Euler-Maruyama noise (sigma 1e-3, Philox keyed by
         seed/instance/node/step), N = 84, 30% density, 64 x 64 grid of G in
         logspace(-3, 0) x speed in linspace(1, 20) mm/ms = 4096 instances,
         dt 0.1 ms, 100k steps, Balloon-Windkessel BOLD sampled every 720 ms,
         84 x 84 Pearson FC per instance against a seeded target FC.
  kuramoto  plain Kuramoto sweep, N = 68, 32 instances, 1000 steps (the
         CPU-runnable parity case).
  net515k   one network of 515 056 nodes (sparse synthetic connectivity),
         node-parallel, 1000 steps.
  adjoint  the FC fit: MPR, N = 84, 256 instances, 2000 steps, forward +
         hand-written adjoint with checkpoints every 100 steps; the line
         carries the gradient error vs the FP64 oracle.
  lems_epileptor  the CUDA DSL's default 32 x 32 speed x coupling sweep on
         the Epileptor generated from its LEMS XML file (N = 68, 4000 steps,
         noise on).
  serve  the serving loop: Poisson arrivals of sweep requests, p50/p99
         latency, served vs plain.
  grid_1k, mixed_small, grid_small, net_small: profiling cases.

Metric: node-steps/s (one node x one instance x one time step).  `value`
is device-resident throughput (CUDA events on the launching stream, max
over ranks); `e2e` repeats the step through the public API with the
initial state uploaded from pinned host memory and the FC matrices read
back every step.  Multi-GPU runs (torchrun) are replicas: every rank runs
the whole workload on its GPU (weak scaling, no collective on the data
path).
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, 'tvb-hpc_gb300'))

METRIC = 'node-steps/s on 1 GB300: batched/served vs plain, same tol; p50/p99 sweep latency'
UNIT = 'node-steps/s'


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def grid_workload(n_g=64, n_s=64, nsteps=100_000, N=84, seed=0):
    from tvb_hpc import network
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    G = np.logspace(-3, 0, n_g).astype(np.float32)
    S = np.linspace(1, 20, n_s).astype(np.float32)
    gg, ss = np.meshgrid(G, S, indexing='ij')
    rng = np.random.default_rng(seed + 1)
    I = gg.size
    x0 = rng.uniform(-0.5, 0.5, (I, N, 2)).astype(np.float32)
    target = np.corrcoef(rng.normal(size=(N, 200))).astype(np.float32)
    bold_period = 7200  # 720 ms at dt 0.1 ms
    return dict(name='grid', conn=conn, couplings=gg.ravel(), speeds=ss.ravel(), x0=x0,
                nsteps=nsteps, dt=0.1, bold_period=bold_period,
                bold_len=nsteps // bold_period, target=target, model='Generic2dOscillator',
                cfun='Diff',
                noise=True, seed=12345)


def grid_small_workload():
    """Profiling case of the grid kernel: the 64 G values x 24 speeds in
    [8, 20] mm/ms (every ring in shared memory), 2000 steps; 1536 instances,
    ring backing store + state > L2 is not needed for the smem-ring kernel."""
    wl = grid_workload(n_g=64, n_s=24, nsteps=2000)
    S = np.linspace(8, 20, 24).astype(np.float32)
    G = np.logspace(-3, 0, 64).astype(np.float32)
    gg, ss = np.meshgrid(G, S, indexing='ij')
    wl.update(name='grid_small', couplings=gg.ravel(), speeds=ss.ravel(), bold_period=200,
              bold_len=10)
    return wl


def kuramoto_workload(I=32, N=68, nsteps=1000, seed=0):
    from tvb_hpc import network
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(seed + 1)
    x0 = rng.uniform(0, 2 * np.pi, (I, N, 1)).astype(np.float32)
    omega = rng.normal(2 * np.pi * 0.01, 0.001, (I, N, 1)).astype(np.float32)
    return dict(name='kuramoto', conn=conn, couplings=np.logspace(-2, 1, I).astype(np.float32),
                speeds=np.full(I, 4.0, np.float32), x0=x0, nparam=omega, nsteps=nsteps, dt=0.1,
                bold_period=0, bold_len=0, target=None, model='Kuramoto', cfun='Kuramoto',
                noise=False, seed=0)


PLAIN_CHUNK = 1000
MIXED_SPEC = [(68, 0.30, 1024), (84, 0.30, 1024), (192, 0.15, 256), (400, 0.08, 64),
              (998, 0.03, 16)]


def mixed_workload(seed=0, scale=1.0, steps_lo=5000, steps_hi=50000):
    """Uneven batch: connectomes of N in {68, 84, 192, 400, 998} at densities
    30/30/15/8/3%, 1024/1024/256/64/16 instances, step counts uniform in
    [5k, 50k], Montbrio-Pazo-Roxin (Delta 1, J 15, eta ~ U(-6, -4), noise
    sigma 1e-2) with linear coupling, speed 4 mm/ms so the longest delay is
    500 steps at dt 0.1 ms."""
    from tvb_hpc import network
    parts = []
    for k, (N, dens, I) in enumerate(MIXED_SPEC):
        I = max(1, int(round(I * scale)))
        w, ln = network.synthetic_connectome(N, dens, seed=seed + k)
        conn = network.Connectivity.from_dense(w, ln)
        rng = np.random.default_rng(seed + 100 + k)
        x0 = np.stack([rng.uniform(0.05, 0.3, (I, N)), rng.uniform(-1.5, -0.5, (I, N))], -1)
        eta = rng.uniform(-6, -4, (I, N, 1)).astype(np.float32)
        steps = rng.integers(steps_lo, steps_hi + 1, I)
        parts.append(dict(conn=conn, couplings=np.logspace(-2, -0.5, I).astype(np.float32),
                          speeds=np.full(I, 4.0, np.float32), x0=x0.astype(np.float32),
                          nparam=eta, steps=steps, seed=seed + 1000 + k))
    return dict(name='mixed', parts=parts, model='MPR', cfun='Linear', noise=True, dt=0.1,
                bold_period=0, bold_len=0, target=None, seed=seed)


def mixed_prof_workload():
    """Profiling case of the uneven batch's kernels: every connectome of the
    mixed workload with 1/8 of its instances (128/128/32/8/2) and 500-2000
    steps, so one launch takes milliseconds under ncu's replays."""
    wl = mixed_workload(scale=0.125, steps_lo=500, steps_hi=2000)
    wl['name'] = 'mixed_prof'
    return wl


def grid_1k_workload():
    """Profiling case of the group kernel: the full 64 x 64 grid (same
    instances, rings and BOLD schedule) for 1000 steps; BOLD sampled every
    200 steps so the FC has five rows."""
    wl = grid_workload(nsteps=1000)
    wl.update(name='grid_1k', bold_period=200, bold_len=5)
    return wl


def mixed_small_workload():
    """Traffic-capture case of the uneven batch: every connectome of the
    mixed workload with 1/8 of its instances (128/128/32/8/2), same step
    distribution."""
    wl = mixed_workload(scale=0.125)
    wl['name'] = 'mixed_small'
    return wl


def net515k_workload(N=515056, degree=64, nsteps=1000, seed=0):
    """One very large network, the single simulation of
    tvb_hpc/examples/sim515k.py (515 056 nodes, linear coupling, Euler): its
    connectivity file is not available, so a seeded sparse synthetic one
    stands in (Poisson(64) in-edges per node, log-normal weights, lengths
    U(10, 200) mm at 4 mm/ms, dt 0.1 ms: delays 25-500 steps); the 2-D
    oscillator in its CUDA-DSL form (tvb_hpc's G2DO diverges within 10^4
    steps); 1000 steps per bench step."""
    from tvb_hpc import network
    conn = network.synthetic_sparse_connectome(N, degree, seed=seed)
    rng = np.random.default_rng(seed + 1)
    x0 = rng.uniform(-0.5, 0.5, (1, N, 2)).astype(np.float32)
    return dict(name='net515k', conn=conn, couplings=np.array([0.05], np.float32),
                speeds=np.array([4.0], np.float32), x0=x0, nsteps=nsteps, dt=0.1, bold_period=0,
                bold_len=0, target=None, model='Generic2dOscillator', cfun='Linear', noise=False,
                seed=seed)


def net_small_workload():
    "Profiling case of net515k: 100 000 nodes, same degree and delays, 200 steps."
    wl = net515k_workload(N=100000, nsteps=200)
    wl['name'] = 'net_small'
    return wl


def lems_workload(n_s=32, n_c=32, N=68, nsteps=4000, seed=0):
    """The CUDA DSL's default sweep (dsl/dsl_cuda/example/cuda_setup.py:55-58,
    97-101: a 32 x 32 grid of speed x coupling, one work item per point) on a
    model generated from LEMS XML: the bundled six-variable Epileptor
    (conditional terms, sine coupling), FP32 literals, noise on (two Philox
    calls per step); speeds logspace(0, 2) mm/ms, couplings logspace(-2, 0),
    dt 0.1, 4000 steps; a seeded 68-node synthetic connectome (the config
    recipe) stands in for the DSL's connectivity_68."""
    import itertools
    from tvb_hpc import network
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    speeds = np.logspace(0.0, 2.0, n_s)
    couplings = np.logspace(-2.0, 0.0, n_c)
    params = np.array(list(itertools.product(speeds, couplings)), np.float32)
    I = params.shape[0]
    rng = np.random.default_rng(seed + 1)
    x0 = np.zeros((I, N, 6), np.float32)
    for v, (lo, hi) in enumerate([(-1.8, -1.2), (-15, -12), (2.8, 3.2), (-1.2, -0.8), (0, 0.2),
                                  (-0.1, 0.1)]):
        x0[:, :, v] = rng.uniform(lo, hi, (I, N))
    return dict(name='lems_epileptor', conn=conn, couplings=params[:, 1], speeds=params[:, 0],
                params=params, x0=x0, nsteps=nsteps, dt=0.1, bold_period=0, bold_len=0,
                target=None, model='Epileptor (generated from LEMS XML, FP32 literals)',
                cfun='LEMS: c_a sin(x1_j - x1), scaled by global_coupling', noise=True,
                seed=seed, lems='Epileptor')


def adjoint_workload(N=84, I=256, T=2000, C=100, seed=0):
    """The adjoint fit: Montbrio-Pazo-Roxin + linear coupling, deterministic,
    N = 84 (the seeded synthetic connectome recipe), 256 instances, 2000 steps of 0.1 ms
    at 4 mm/ms, FC of the rate series vs a seeded target, gradients w.r.t. G
    and the 84 per-node eta by the hand-written adjoint with checkpoints every
    100 steps.  One bench step = forward (loss) + backward (gradients)."""
    from tvb_hpc import network
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(seed + 1)
    x0 = np.stack([rng.uniform(0.05, 0.3, (I, N)), rng.uniform(-1.5, -0.5, (I, N))], -1)
    eta = rng.uniform(-6, -4, (I, N)).astype(np.float32)
    G = np.logspace(-2, -0.5, I).astype(np.float32)
    target = np.corrcoef(rng.normal(size=(N, 60))).astype(np.float32)
    return dict(name='adjoint', conn=conn, couplings=G, speeds=np.full(I, 4.0, np.float32),
                x0=x0.astype(np.float32), eta=eta, target_fc=target, nsteps=T, ckpt=C, dt=0.1,
                bold_period=0, bold_len=0, target=None, model='MPR', cfun='Linear', noise=False,
                seed=seed)


WORKLOADS = {'grid': grid_workload, 'grid_small': grid_small_workload, 'grid_1k': grid_1k_workload,
             'kuramoto': kuramoto_workload, 'mixed': mixed_workload,
             'mixed_small': mixed_small_workload, 'mixed_prof': mixed_prof_workload,
             'net515k': net515k_workload,
             'lems_epileptor': lems_workload, 'adjoint': adjoint_workload,
             'net_small': net_small_workload}


def workload_config(wl):
    if wl['name'].startswith('mixed'):
        return {'workload': wl['name'], 'model': wl['model'], 'coupling': wl['cfun'],
                'nodes': [int(p['conn'].nnode) for p in wl['parts']],
                'edges': [int(p['conn'].nnz) for p in wl['parts']],
                'instances': [int(p['couplings'].size) for p in wl['parts']],
                'time_steps': 'uniform 5k-50k per instance', 'dt_ms': wl['dt'],
                'noise': 'philox-em', 'max_delay_steps': 500,
                'l2': wl.get('l2_note'), 'parallelism': 'replicas'}
    c = wl['conn']
    return {'workload': wl['name'], 'model': wl['model'], 'coupling': wl['cfun'],
            'nodes': int(c.nnode), 'edges': int(c.nnz), 'instances': int(wl['couplings'].size),
            'time_steps': int(wl['nsteps']), 'dt_ms': wl['dt'],
            'noise': 'philox-em' if wl['noise'] else 'off',
            'bold_period_steps': int(wl['bold_period']), 'fc': wl['target'] is not None,
            'l2': wl.get('l2_note'), 'parallelism': 'replicas'}


def l2_policy(torch):
    """The L2 rule of the timed region: with more than twice L2 resident on
    the device (rings, state, monitors) the inputs are larger than L2;
    otherwise a buffer of twice L2 is written between timed steps, outside
    the steps' event pairs.  Returns (flush buffer or None, config note)."""
    l2 = int(getattr(torch.cuda.get_device_properties(torch.cuda.current_device()),
                     'L2_cache_size', 0) or 126 * 2**20)
    res = torch.cuda.memory_allocated()
    if res > 2 * l2:
        return None, 'inputs larger than L2 (%.0f MB resident on the device, L2 %.0f MB)' % (
            res / 2**20, l2 / 2**20)
    buf = torch.empty(2 * l2 // 4, dtype=torch.float32, device='cuda')
    return buf, ('L2 flushed between timed steps: a %.0f MB write outside the steps\' event '
                 'pairs (%.0f MB resident on the device, L2 %.0f MB)' % (
                     2 * l2 / 2**20, res / 2**20, l2 / 2**20))


class StepTimer:
    """Times K steps: one event pair around the whole region, or with an L2
    flush buffer, one pair per step with the flush between them."""

    def __init__(self, torch, flush):
        self.torch, self.flush, self.pairs = torch, flush, []
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)

    def start(self):
        self.e0.record()

    def before_step(self):
        if self.flush is not None:
            self.flush.zero_()
            a = self.torch.cuda.Event(enable_timing=True)
            a.record()
            self.pairs.append([a, None])

    def after_step(self):
        if self.flush is not None:
            b = self.torch.cuda.Event(enable_timing=True)
            b.record()
            self.pairs[-1][1] = b

    def stop(self):
        self.e1.record()

    def ms(self):
        if self.flush is None:
            return self.e0.elapsed_time(self.e1)
        return sum(a.elapsed_time(b) for a, b in self.pairs)


def node_steps(wl):
    if wl['name'].startswith('mixed'):
        return float(sum(p['conn'].nnode * p['steps'].sum() for p in wl['parts']))
    return float(wl['couplings'].size) * wl['conn'].nnode * wl['nsteps']


def algorithmic_bytes_per_node_step(wl, nsvar):
    """Algorithmic bytes per node-step: 4 B per delayed read of the coupled
    variable, 8 B per state variable (read + write), 32 B for the balloon
    state when BOLD is on."""
    if wl['name'].startswith('mixed'):
        tot = sum(p['conn'].nnode * p['steps'].sum() for p in wl['parts'])
        E = sum(p['conn'].nnz * p['steps'].sum() for p in wl['parts']) / tot
        return 4.0 * E + 8.0 * nsvar
    E = wl['conn'].nnz / wl['conn'].nnode
    return 4.0 * E + 8.0 * nsvar + (32.0 if wl['bold_period'] else 0.0)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.mark = 0
        self.proc = None
        self.held = 0

    def start(self):
        """Start nvidia-smi and wait (at most 3 s) for its first line, which
        is taken before the timed region and dropped."""
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.QUERY,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while not self.samples and time.time() - t0 < 3.0 and self.proc.poll() is None:
            time.sleep(0.01)
        self.mark = len(self.samples)

    def hold(self, step, min_samples=3, max_s=3.0):
        """A timed region shorter than the sample period leaves too few
        samples: keep running the same step, untimed, until min_samples
        samples were taken since start() (at most max_s seconds).  The line
        reports how many steps were added."""
        import torch
        if self.proc is None:
            return
        t0 = time.time()
        while len(self.samples) - self.mark < min_samples and time.time() - t0 < max_s:
            step()
            torch.cuda.synchronize()
            self.held += 1

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(',')])

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for s in self.samples[self.mark:]:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, s[3:7]):
                if v.lower() == 'active':
                    reasons.add(name)
        out = {'sm_mhz': float(np.median(sm)) if sm else None,
               'sm_max_mhz': float(max(mx)) if mx else None,
               'reasons': sorted(reasons), 'samples': len(sm)}
        if self.held:
            out['window'] = ('timed region + %d untimed steps of the same work after it (fewer '
                             'than 3 samples of the 200 ms period fell in the timed region)'
                             % self.held)
        return out


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def build_sweep(wl, tpn=None, warps=None):
    from tvb_hpc import model, coupling, scheme, engine
    m = getattr(model, wl['model'])()
    cf = getattr(coupling, wl['cfun'])(m)
    scm = scheme.EulerMaryuyamaStep(wl['dt']) if wl['noise'] else scheme.EulerStep(wl['dt'])
    return engine.Sweep(m, cf, scm, wl['conn'], dt=wl['dt'], couplings=wl['couplings'],
                        speeds=wl['speeds'], state0=wl['x0'], nparam=wl.get('nparam'),
                        seed=wl['seed'], bold_period=wl['bold_period'], bold_len=wl['bold_len'],
                        tpn=tpn, warps=warps)


class MixedStep:
    """One bench step of the uneven batch: reset every instance from resident
    copies and run the whole batch as one CUDA-graph launch.  The batch runs
    either as lane-interleaved groups (tvbg_group_run: eight instances per
    lane slice, clusters for large N; default) or as per-instance persistent
    kernels (tvbg_batch_run).  `run_plain` runs the same work as one
    tvbg_sweep per connectome, sequentially (the plain path)."""

    def __init__(self, wl, torch, path='groups', graph=True, tune=True):
        from tvb_hpc import model, coupling, scheme, engine, groups
        self.torch = torch
        self.wl = wl
        self.path = path
        m = getattr(model, wl['model'])()
        cf = getattr(coupling, wl['cfun'])(m)
        scm = scheme.EulerMaryuyamaStep(wl['dt'])
        self.sets = []
        for p in wl['parts']:
            kw = dict(dt=wl['dt'], couplings=p['couplings'], speeds=p['speeds'], state0=p['x0'],
                      nparam=p['nparam'], seed=p['seed'])
            if path == 'groups':
                self.sets.append(groups.GroupSet(m, cf, scm, p['conn'], nsteps=p['steps'], **kw))
            else:
                self.sets.append(engine.InstanceSet(m, cf, scm, p['conn'], **kw))
        self.x0 = [s.state.clone() for s in self.sets]
        steps = [p['steps'] for p in wl['parts']]
        self.steps = steps
        if path == 'groups':
            # launch shapes per connectome (plain or pipelined kernel, CTA
            # width, cluster) and dispatch priorities from the makespan-aware
            # tuner: whole-batch trials at scaled-down step counts
            if tune == 'pipelined':
                shapes = [groups.pipelined_shape(s) for s in self.sets]
            else:
                shapes = 'tune' if tune else None
            self.batch = groups.GroupBatch(self.sets, steps, shapes=shapes)
            self.n_launch = self.batch.n_launches
        else:
            self.batch = engine.Batch(self.sets, steps)
            self.n_launch = len(self.batch.launches)
        if graph:
            self.batch.capture()
        self.ns = m.nsvar
        self.status = self.batch.status
        # plain path: per connectome, the per-step kernel (no time blocking),
        # one sweep launched in chunks of PLAIN_CHUNK steps (as the
        # reference's launcher chunks, dsl/dsl_cuda/example/cuda_run.py:124-142),
        # connectomes one after the other; chunk tables are built up front
        self.plain = []
        for p in wl['parts']:
            sw = engine.Sweep(m, cf, scm, p['conn'], dt=wl['dt'], couplings=p['couplings'],
                              speeds=p['speeds'], state0=p['x0'], nparam=p['nparam'],
                              seed=p['seed'], blocked=False, tpn=2)
            chunks = []
            steps = np.asarray(p['steps'])
            for c in range(int(np.ceil(steps.max() / PLAIN_CHUNK))):
                sw.t[:] = c * PLAIN_CHUNK
                chunks.append(sw.prepare(np.clip(steps - c * PLAIN_CHUNK, 0, PLAIN_CHUNK)))
            sw.t[:] = 0
            self.plain.append((sw, chunks, sw.state.clone()))

    def reset(self, x0=None):
        for s, x in zip(self.sets, self.x0 if x0 is None else x0):
            if self.path == 'groups':
                s.set_state(x)
                s.clear_history()
            else:
                s.state.copy_(x)
                s.ring.zero_()

    def run(self, time_kernels=False):
        evs = []
        torch = self.torch
        go = self.batch.replay if self.batch.graph is not None else self.batch.launch
        # NVTX range of one bench step: ncu --nvtx --nvtx-include "mixed_step/"
        # (with --graph-profiling graph, the concurrent graph as one workload)
        torch.cuda.nvtx.range_push('mixed_step')
        if time_kernels:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            go()
            e1.record()
            evs.append((e0, e1))
        else:
            go()
        torch.cuda.nvtx.range_pop()
        return evs, None

    def run_plain(self):
        for sw, chunks, _ in self.plain:
            for launches in chunks:
                sw.launch(launches, 2)

    def plain_groups(self):
        """The same group kernels with one connectome per launch set, the
        connectomes in sequence, each on its fastest shape when run alone
        (autotune.tune_group_alone).  Returns (ms, shapes)."""
        from tvb_hpc import autotune, groups
        torch = self.torch
        shapes = [autotune.tune_group_alone(s, n)[0] for s, n in zip(self.sets, self.steps)]
        solo = [groups.GroupBatch([s], [n], shapes=[sh])
                for s, n, sh in zip(self.sets, self.steps, shapes)]
        for s, sh in zip(self.sets, self.batch.shapes):
            s.set_shape(*sh)

        def once():
            self.reset()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for b in solo:
                b.launch()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)

        once()  # warm-up
        ms = once()
        for b in solo:
            b.status.check()
        self.reset()
        return ms, shapes

    def accuracy_run(self, nsteps=1000, per_set=2):
        """Every instance of the benchmarked batch run for its first `nsteps`
        steps -- same sets, launch shapes and priorities, one launch set --
        and the final states of `per_set` sampled instances per connectome
        (the longest and a middle one), for the comparison with the oracle."""
        from tvb_hpc import groups
        torch = self.torch
        self.reset()
        short = [np.minimum(np.asarray(n), nsteps) for n in self.steps]
        b = groups.GroupBatch(self.sets, short, shapes=self.batch.shapes,
                              step_ms=self.batch.step_ms)
        b.run()
        out = []
        for s, n in zip(self.sets, self.steps):
            order = np.argsort(-np.asarray(n), kind='stable')
            idx = np.unique(order[np.linspace(0, len(order) - 1, per_set).astype(int)])
            out.append(dict(idx=idx, state=s.state[torch.from_numpy(idx).cuda()].cpu().numpy(),
                            nsteps=nsteps))
        self.reset()
        return out

    def reset_plain(self):
        for sw, _, x0 in self.plain:
            sw.state.copy_(x0)
            sw.ring.zero_()

    def launches_per_step(self):
        return self.n_launch


def build_groups(wl):
    from tvb_hpc import model, coupling, scheme, groups
    m = getattr(model, wl['model'])()
    cf = getattr(coupling, wl['cfun'])(m)
    scm = scheme.EulerMaryuyamaStep(wl['dt']) if wl['noise'] else scheme.EulerStep(wl['dt'])
    return groups.GroupSet(m, cf, scm, wl['conn'], dt=wl['dt'], couplings=wl['couplings'],
                           speeds=wl['speeds'], state0=wl['x0'], nparam=wl.get('nparam'),
                           seed=wl['seed'], bold_period=wl['bold_period'],
                           bold_len=wl['bold_len'])


def groups_supported(wl):
    return ((wl['cfun'] in ('Linear', 'Diff', 'Sigmoidal') and wl['model'] != 'Kuramoto')
            or (wl['model'], wl['cfun']) == ('Kuramoto', 'Kuramoto'))


class GpuStep:
    """One bench step on the device: reset state/ring/balloon from resident
    copies, run every instance for all steps, compute FC.  Separable
    couplings run as lane-interleaved groups (tvbg_group_run), the others on
    the per-instance kernels (tvbg_sweep)."""

    def __init__(self, wl, torch, tpn=None, warps=None, path='groups'):
        self.torch = torch
        self.wl = wl
        self.groups = path == 'groups' and groups_supported(wl)
        if self.groups:
            from tvb_hpc import autotune
            self.sw = build_groups(wl)
            # the set's fastest launch shape alone (plain or pipelined, CTA
            # width, cluster), by short trials
            self.shape = autotune.tune_group_alone(self.sw, wl['nsteps'])[0]
            self.sw.set_shape(*self.shape)
            self.launches = self.sw.prepare(wl['nsteps'])[0]
            self.tpn = None
        else:
            self.sw = build_sweep(wl, tpn, warps)
            self.sw.pick_tpn()
            self.launches = self.sw.prepare(wl['nsteps'])
            self.tpn = self.sw.tpn
        self.path = (('lane-interleaved groups, %s kernel where the delays allow, %d threads x %d '
                      'CTAs' % ('pipelined' if self.shape[3] == 2 else 'plain', self.shape[0],
                                self.shape[1])) if self.groups else 'per-instance kernels')
        self.x0 = self.sw.state.clone()
        self.ns = self.sw.ns
        self.status = self.sw.status
        self.target = (torch.from_numpy(wl['target']).cuda() if wl['target'] is not None
                       else None)
        self.n_launch = len(self.launches)

    def reset(self, x0=None):
        sw = self.sw
        x = self.x0 if x0 is None else x0
        if self.groups:
            sw.clear_history()
            sw.set_state(x)
            if sw.gbold is not None:
                sw.gbold.zero_()
        else:
            sw.ring.zero_()
            sw.state.copy_(x)
            if sw.bold is not None:
                sw.bold.zero_()

    def _launch(self, launches):
        if self.groups:
            self.sw.launch(launches)
        else:
            self.sw.launch(launches, self.sw.tpn)

    def run(self, time_kernels=False):
        from tvb_hpc import metric  # noqa: F401
        torch = self.torch
        sw = self.sw
        evs = []
        if time_kernels:
            for launch in self.launches:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                self._launch([launch])
                e1.record()
                evs.append((e0, e1))
        else:
            self._launch(self.launches)
        fc = None
        if sw.bold_out is not None and self.target is not None:
            fc = metric.fc(sw.bold_out, self.target)
        return evs, fc

    def launches_per_step(self):
        fc_launches = 1 if (self.wl['bold_period'] > 0 and self.target is not None) else 0
        return self.n_launch + fc_launches


class NetStep:
    """One bench step of the single large network: reset state and ring
    from resident copies, advance nsteps (one seed launch and one launch per
    block of K steps, node-parallel)."""

    def __init__(self, wl, torch):
        from tvb_hpc import model, coupling, scheme, bignet
        self.torch = torch
        self.wl = wl
        m = getattr(model, wl['model'])()
        cf = getattr(coupling, wl['cfun'])(m)
        scm = scheme.EulerMaryuyamaStep(wl['dt']) if wl['noise'] else scheme.EulerStep(wl['dt'])
        self.sw = bignet.SingleNetwork(m, cf, scm, wl['conn'], wl['dt'],
                                       coupling=float(wl['couplings'][0]),
                                       speed=float(wl['speeds'][0]), state0=wl['x0'][0],
                                       seed=wl['seed'])
        self.x0 = self.sw.state.clone()
        self.ns = self.sw.ns
        self.status = self.sw.status
        self.tpn = None
        self.path = 'node-parallel single network, one launch per block of %d steps' % self.sw.block_k

    def reset(self, x0=None):
        self.sw.state.copy_(self.x0 if x0 is None else x0)
        self.sw.ring.zero_()
        self.sw.t = 0

    def run(self, time_kernels=False):
        torch = self.torch
        evs = []
        if time_kernels:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            self.sw.launch(self.wl['nsteps'])
            e1.record()
            evs.append((e0, e1))
        else:
            self.sw.launch(self.wl['nsteps'])
        return evs, None

    def launches_per_step(self):
        return 1 + -(-self.wl['nsteps'] // self.sw.block_k)


class LemsStep:
    """One bench step of a LEMS-generated model: reset state and ring from
    resident copies and advance every work item nsteps -- on the
    lane-interleaved group kernel where the model's coupling and delays allow
    (LemsGroupSet), else with one per-step launch per ring group (LemsSweep);
    tables are built once."""

    def __init__(self, wl, torch, tpn=None, path='groups'):
        from tvb_hpc import lems
        self.torch = torch
        self.wl = wl
        m = lems.load_model(wl['lems'])
        self.sw = lems.make_set(m, wl['conn'], wl['dt'], wl['params'], state0=wl['x0'],
                                noise=wl['noise'], single=True, seed=wl['seed'], tpn=tpn,
                                prefer=path)
        self.groups = isinstance(self.sw, lems.LemsGroupSet)
        self.x0 = self.sw.state.clone()
        self.ring0 = self.sw.ring.clone()
        if self.groups:
            self.tpn = None
            self.sw.t[:] = 0
            self.launches, _ = self.sw.prepare(wl['nsteps'])
            self.path = ('generated group kernel (8 work items per group, K = %s steps per '
                         'block), %d groups' % (sorted(set(self.sw.block_k.tolist())),
                                                 self.sw.n_groups))
        else:
            self.tpn = self.sw.pick_tpn()
            self.sw.t[:] = 0
            self.launches = self.sw.prepare(wl['nsteps'])
            self.path = 'generated per-step kernel (one CTA per work item), tpn %d' % self.tpn
        self.ns = m.ns
        self.status = self.sw.status

    def reset(self, x0=None):
        if self.groups:
            self.sw.set_state(self.x0 if x0 is None else x0)
        else:
            self.sw.state.copy_(self.x0 if x0 is None else x0)
        self.sw.ring.copy_(self.ring0)

    def _launch(self):
        if self.groups:
            self.sw.launch(self.launches)
        else:
            self.sw.launch(self.launches, self.tpn)

    def run(self, time_kernels=False):
        torch = self.torch
        evs = []
        if time_kernels:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            self._launch()
            e1.record()
            evs.append((e0, e1))
        else:
            self._launch()
        return evs, None

    def launches_per_step(self):
        return len(self.launches)


class AdjointStep:
    """One bench step of the adjoint fit: FCFit.forward (checkpointed forward
    sweep, FP64 FC loss) and FCFit.backward (recomputation + reverse-time
    kernel per segment, FP64 gradient accumulation)."""

    def __init__(self, wl, torch):
        from tvb_hpc import adjoint
        self.torch = torch
        self.wl = wl
        self.prob = adjoint.FCFit(wl['conn'], wl['dt'], 4.0, wl['x0'], wl['target_fc'],
                                  wl['nsteps'], checkpoint_every=wl['ckpt'])
        self.ns = 2
        self.tpn = 2
        self.status = None
        self.grads = None
        self.path = ('%s forward with checkpoints every %d steps; FC-fit loss '
                     'path on the device (tvbg_fcfit_loss: FP64 FC and loss, no library GEMM); '
                     'per segment: recomputation + reverse-time kernel (%s); FP64 gradients'
                     % ('pipelined group kernel' if self.prob.layout == 'groups'
                        else 'per-step kernel', wl['ckpt'],
                        'lane-interleaved groups, time-blocked%s, %d threads x %d CTAs'
                        % ((', two thread teams' if self.prob.adjoint_shape[2] else '',)
                           + tuple(self.prob.adjoint_shape[:2]))
                        if self.prob.adjoint_kernel == 'groups' else 'per instance'))
        self.x0 = None

    def reset(self, x0=None):
        pass

    def run(self, time_kernels=False):
        torch = self.torch
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        loss = self.prob.forward(self.wl['couplings'], self.wl['eta'])
        self.grads = self.prob.backward()
        e1.record()
        self.loss = loss
        return ([(e0, e1)] if time_kernels else []), None

    def launches_per_step(self):
        segs = -(-self.wl['nsteps'] // self.wl['ckpt'])
        return 3 * segs        # forward segment, recomputation, reverse-time kernel

    def grad_error(self, n_check=4):
        "Max-norm relative error of dL/dG and dL/deta vs the FP64 oracle on a sample."
        sys.path.insert(0, os.path.join(ROOT, 'oracle'))
        import pyoracle as orc
        from tvb_hpc import model as mdl
        wl = self.wl
        c = wl['conn']
        idx = np.linspace(0, wl['couplings'].size - 1, n_check).astype(int)
        d = c.delays(4.0, wl['dt'], 'ceil')
        _, consts, _ = mdl.MPR().engine_spec()
        _, dG_o, deta_o = orc.mpr_adjoint(c.row, c.col, c.wnz, d,
                                          wl['couplings'][idx].astype(np.float64),
                                          wl['eta'][idx].astype(np.float64),
                                          wl['x0'][idx].astype(np.float64), wl['nsteps'], wl['dt'],
                                          consts, wl['target_fc'])
        dG = self.grads[0].cpu().numpy()[idx]
        deta = self.grads[1].cpu().numpy()[idx]
        e = lambda a, b: float(np.abs(a - b).max() / np.abs(b).max())  # noqa: E731
        return {'dG': e(dG, dG_o), 'deta': e(deta, deta_o), 'instances_checked': int(n_check),
                'against': 'FP64 oracle adjoint (C)'}


def cpu_baseline_adjoint(wl, budget_s=12.0):
    "The FP64 oracle's forward + adjoint (C, OpenMP over instances) on a sample."
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import pyoracle as orc
    from tvb_hpc import model as mdl
    c = wl['conn']
    cores = os.cpu_count() or 1
    d = c.delays(4.0, wl['dt'], 'ceil')
    _, consts, _ = mdl.MPR().engine_spec()
    I = wl['couplings'].size

    def run(n):
        idx = np.linspace(0, I - 1, n).astype(int)
        t = time.perf_counter()
        orc.mpr_adjoint(c.row, c.col, c.wnz, d, wl['couplings'][idx].astype(np.float64),
                        wl['eta'][idx].astype(np.float64), wl['x0'][idx].astype(np.float64),
                        wl['nsteps'], wl['dt'], consts, wl['target_fc'], nthreads=cores)
        return time.perf_counter() - t

    n = min(I, max(cores, 4))
    el = run(n)
    n = int(np.clip(n * budget_s / max(el, 1e-6), n, I))
    el = run(n)
    v = n * c.nnode * wl['nsteps'] / el
    return {'value': round(v, 1), 'unit': UNIT, 'cores': cores, 'kind': 'port',
            'sample': '%d of %d instances x %d steps, forward + adjoint (%.1f s), FP64 oracle C + '
                      'OpenMP' % (n, wl['couplings'].size, wl['nsteps'], el)}


def cpu_baseline_lems(wl, budget_s=12.0):
    "The LEMS oracle (numpy, one work item at a time) on a bounded sample."
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import lems_oracle as lo
    from tvb_hpc import lems
    c = wl['conn']
    path = lems.lems_file(wl['lems'])
    idx = np.linspace(0, wl['params'].shape[0] - 1, 4).astype(int)

    def run(nsteps, k):
        t = time.perf_counter()
        lo.run(path, wl['lems'], c.row, c.col, c.wnz, c.lnz, wl['params'][idx[k]:idx[k] + 1],
               wl['dt'], nsteps, wl['x0'][idx[k]])
        return time.perf_counter() - t

    probe = 20
    dt_probe = run(probe, 0)
    nsteps = int(np.clip(probe * budget_s / 4 / max(dt_probe, 1e-6), probe, wl['nsteps']))
    el = sum(run(nsteps, k) for k in range(4))
    v = 4 * c.nnode * nsteps / el
    return {'value': round(v, 1), 'unit': UNIT, 'cores': 1, 'kind': 'port',
            'sample': '4 of %d work items x %d steps (%.1f s), LEMS oracle (numpy), noise off' % (
                wl['params'].shape[0], nsteps, el)}


def roofline_entry(wl, nsvar, kernel_ms_total, steps):
    """Roofline of the step kernel: algorithmic bytes of the timed steps over
    the step kernels' event-timed duration (for the uneven batch, the graph
    of concurrent persistent kernels), against the measured HBM copy rate."""
    peaks = {}
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        peaks = json.load(open(p))
    hbm = peaks.get('hbm_gbs')
    src = 'measured' if hbm else 'fallback'
    hbm = hbm or 6800.0
    bpn = algorithmic_bytes_per_node_step(wl, nsvar)
    achieved = bpn * node_steps(wl) * steps / (kernel_ms_total / 1e3) / 1e9
    # DRAM traffic of the step kernel from an ncu capture (profiles/traffic.json:
    # bytes per node-step measured on a capture case of this workload), per
    # bench step
    traffic, tsrc, compute = None, None, None
    tp = os.path.join(ROOT, 'profiles', 'traffic.json')
    if os.path.exists(tp):
        key = 'mixed' if wl['name'].startswith('mixed') else wl['name'].split('_')[0]
        t = json.load(open(tp)).get(key)
        if t:
            if t.get('dram_bytes_per_node_step'):
                traffic = round(t['dram_bytes_per_node_step'] * node_steps(wl))
            tsrc = t.get('source')
            if 'issue_active_pct' in t:
                # the second roof: the SM's issue slots and FP32 FMA pipe, from the same capture
                compute = {'issue_active_pct': t['issue_active_pct'],
                           'fma_pipe_pct': t['fma_pipe_pct'], 'binding': t['binding']}
    return {'bound': 'hbm', 'achieved': round(achieved, 1), 'peak': hbm, 'unit': 'GB/s',
            'frac': round(achieved / hbm, 4), 'traffic': traffic, 'traffic_source': tsrc,
            'compute': compute,
            'peak_source': src, 'algorithmic_bytes_per_node_step': round(bpn, 2),
            'note': 'achieved = algorithmic bytes / event-timed kernel time; traffic = DRAM '
                    'bytes per bench step (part of the ring reads hit L2)'}


def cpu_baseline(wl, budget_s=12.0):
    "The oracle (C restatement, OpenMP over instances) on a bounded sample."
    if wl['conn'].nnode > 1024:
        return {'value': None, 'unit': UNIT, 'cores': 0, 'kind': 'port',
                'sample': 'not run: the oracle steps networks of up to 1024 nodes'}
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import pyoracle as orc
    from tvb_hpc import network, model as mdl
    m = getattr(mdl, wl['model'])()
    kid, consts, sigma = m.engine_spec()
    cf_id = {'Diff': 1, 'Kuramoto': 2, 'Linear': 0}[wl['cfun']]
    cores = os.cpu_count() or 1
    c = wl['conn']
    I_all = wl['couplings'].size
    # sample: instances spread over the grid (all speeds present)
    n_inst = min(I_all, max(cores * 2, 16))
    idx = np.linspace(0, I_all - 1, n_inst).astype(int)

    def run(nsteps):
        speeds = wl['speeds'][idx]
        delays = np.stack([c.delays(s, wl['dt'], 'ceil') for s in speeds])
        nh = int(2 ** np.ceil(np.log2(delays.max() + 2)))
        nparam = (np.asarray(wl['nparam'])[idx, :, 0] if wl.get('nparam') is not None
                  else np.broadcast_to(m.node_params(c.nnode)[:, 0], (n_inst, c.nnode)))
        t = time.perf_counter()
        orc.run(kid, cf_id, c.row, c.col, c.wnz, nh, nsteps, wl['dt'], delays,
                wl['couplings'][idx], nparam, wl['x0'][idx],
                flags=(orc.F_NOISE if wl['noise'] else 0) | orc.F_BOLD_DEV, sigma=sigma,
                consts=consts, seed=wl['seed'], bold_period=wl['bold_period'] or 0,
                bold_len=max(1, nsteps // max(1, wl['bold_period'] or 1)), bold_obs=1,
                nthreads=cores)
        return time.perf_counter() - t

    probe = 50
    dt_probe = run(probe)
    nsteps = int(np.clip(probe * budget_s / max(dt_probe, 1e-6), probe, wl['nsteps']))
    el = run(nsteps)
    v = n_inst * c.nnode * nsteps / el
    return {'value': round(v, 1), 'unit': UNIT, 'cores': cores, 'kind': 'port',
            'sample': '%d of %d instances x %d steps (%.1f s), oracle C + OpenMP, -O3' % (
                n_inst, I_all, nsteps, el)}


def reference_gpu_kuramoto(wl, n_items, inner=100, reps=3):
    """The reference's own CUDA DSL Kuramoto kernel (dsl/dsl_cuda/CUDAmodels/
    kuramoto.c, compiled unchanged for sm_103a by baseline/Makefile) on the
    workload's connectome: one thread per work item scanning the dense N x N
    weights, curand noise always on, launched as the reference launcher does
    (dsl/dsl_cuda/example/cuda_run.py:109-142): `inner` steps per launch,
    the tavg buffer copied to the host after every launch; blocks of 32 x 1
    threads (blockDim.y = 1: the kernel's __syncthreads() sits in a node loop
    whose trip count depends on threadIdx.y).  Returns node-steps/s."""
    import ctypes
    import torch
    path = os.path.join(ROOT, 'baseline', '_ref', 'kuramoto_sm103a.cubin')
    if not os.path.exists(path):
        return {'unavailable': 'baseline/_ref/kuramoto_sm103a.cubin not built '
                               '(make -C baseline gpu REF=<tvb-hpc checkout>)'}
    cu = ctypes.CDLL('libcuda.so.1')

    def ck(rc, what):
        if rc != 0:
            raise RuntimeError('%s failed (CUresult %d)' % (what, rc))

    torch.cuda.synchronize()                   # the primary context is current
    mod, fn = ctypes.c_void_p(), ctypes.c_void_p()
    ck(cu.cuModuleLoad(ctypes.byref(mod), path.encode()), 'cuModuleLoad')
    try:
        ck(cu.cuModuleGetFunction(ctypes.byref(fn), mod, b'_Z8KuramotojjjjjffPfS_S_S_S_'),
           'cuModuleGetFunction')
        conn = wl['conn']
        N = conn.nnode
        w = np.zeros((N, N), np.float32)
        ln = np.zeros((N, N), np.float32)
        rows = np.repeat(np.arange(N), np.diff(conn.row))
        w[rows, conn.col] = conn.wnz
        ln[rows, conn.col] = conn.lnz
        speed = float(wl['speeds'][0])
        G = np.resize(np.asarray(wl['couplings'], np.float32), n_items)
        bx = 32
        n_items = bx * -(-n_items // bx)
        G = np.resize(G, n_items)
        dmax = int(np.max(ln * np.float32(np.float32(1.0) / np.float32(speed) / np.float32(wl['dt']))))
        nh = 1 << int(np.ceil(np.log2(dmax + 2)))
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()  # noqa: E731
        d_w, d_l = dev(w), dev(ln)
        d_p = dev(np.stack([np.full(n_items, speed, np.float32), G]))    # params [2][items]
        d_s = torch.zeros(nh * N * n_items, dtype=torch.float32, device='cuda')
        d_t = torch.zeros(N * n_items, dtype=torch.float32, device='cuda')
        host_t = torch.empty(N * n_items, dtype=torch.float32).pin_memory()
        nsteps = int(wl['nsteps'])

        def launch(i_step, n_step):
            vals = [ctypes.c_uint(i_step), ctypes.c_uint(N), ctypes.c_uint(nh), ctypes.c_uint(n_step),
                    ctypes.c_uint(2), ctypes.c_float(wl['dt']), ctypes.c_float(speed)] + [
                ctypes.c_void_p(t.data_ptr()) for t in (d_w, d_l, d_p, d_s, d_t)]
            ptrs = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.byref(v), ctypes.c_void_p)
                                                   for v in vals])
            ck(cu.cuLaunchKernel(fn, n_items // bx, 1, 1, bx, 1, 1, 0, None, ptrs, None),
               'cuLaunchKernel')

        def run():
            for i in range(-(-nsteps // inner)):
                launch(i * inner, min(inner, nsteps - i * inner))
                host_t.copy_(d_t)              # the launcher's per-launch tavg download
            torch.cuda.synchronize()

        run()                                  # warm-up (module load, first launch)
        best = None
        for _ in range(reps):
            d_s.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            run()
            el = time.perf_counter() - t0
            best = el if best is None else min(best, el)
        return {'value': round(N * n_items * nsteps / best, 1), 'unit': UNIT,
                'work_items': n_items, 'nodes': N, 'steps': nsteps, 'ms': round(best * 1e3, 3),
                'path': 'reference CUDA DSL kernel kuramoto.c for sm_103a, %d-step launches, '
                        'blocks of 32 x 1, noise on (curand, hard-wired)' % inner}
    finally:
        cu.cuModuleUnload(mod)


def engine_kuramoto_items(wl, n_items, reps=3):
    """The engine on the same sweep as reference_gpu_kuramoto's: the
    workload's Kuramoto network with n_items instances (couplings tiled),
    lane-interleaved groups (sin/cos ring), noise off; node-steps/s."""
    import torch
    from tvb_hpc import model, coupling, scheme, groups
    m = model.Kuramoto()
    cf = coupling.Kuramoto(m)
    I = int(n_items)
    x0 = np.resize(wl['x0'], (I, ) + wl['x0'].shape[1:])
    om = np.resize(wl['nparam'], (I, ) + wl['nparam'].shape[1:])
    gs = groups.GroupSet(m, cf, scheme.EulerStep(wl['dt']), wl['conn'], dt=wl['dt'],
                         couplings=np.resize(wl['couplings'], I), speeds=np.resize(wl['speeds'], I),
                         state0=x0, nparam=om)
    gs.set_shape(*groups.pipelined_shape(gs))
    n = int(wl['nsteps'])
    gs.run(n)
    best = None
    for _ in range(reps):
        gs.t[:] = 0
        gs.clear_history()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        gs.run(n, check=False)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    gs.status.check()
    return {'value': round(wl['conn'].nnode * I * n / (best / 1e3), 1), 'unit': UNIT,
            'instances': I, 'ms': round(best, 3),
            'path': 'lane-interleaved groups, Kuramoto sin/cos ring, %s kernel, noise off'
                    % ('pipelined' if gs.tpn == 2 else 'plain')}


def gpu_arm(args):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        dist.init_process_group('nccl')
    torch.cuda.set_device(local)
    from tvb_hpc import _native
    _native.load()
    wl = WORKLOADS[args.workload]()
    if wl['name'].startswith('mixed'):
        gs = MixedStep(wl, torch, args.path, not args.no_graph,
                       'pipelined' if args.no_tune and args.pipelined else not args.no_tune)
    elif wl['name'].startswith('net'):
        gs = NetStep(wl, torch)
    elif wl['name'].startswith('lems'):
        gs = LemsStep(wl, torch, args.tpn, 'groups' if args.path == 'groups' else 'sweep')
    elif wl['name'] == 'adjoint':
        return adjoint_finish(args, wl, AdjointStep(wl, torch), torch, world, rank, barrier_fn=None)
    else:
        gs = GpuStep(wl, torch, args.tpn, args.warps, args.path)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up
    for _ in range(args.warmup):
        gs.reset()
        gs.run()
    torch.cuda.synchronize()
    # device-resident timed region
    flush, wl['l2_note'] = l2_policy(torch)
    timer = StepTimer(torch, flush)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    kern_ms, n_kern = 0.0, 0
    all_evs = []
    timer.start()
    for _ in range(args.steps):
        timer.before_step()
        gs.reset()
        evs, fc = gs.run(time_kernels=True)
        timer.after_step()
        all_evs.extend(evs)
    timer.stop()
    barrier()

    def again():
        gs.reset()
        gs.run()
    clocks.hold(again)
    clk = clocks.stop()
    total_ms = timer.ms()
    for a, b in all_evs:
        kern_ms += a.elapsed_time(b)
        n_kern += 1
    t = torch.tensor([total_ms], device='cuda')
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * node_steps(wl) * args.steps / (total_ms / 1e3)
    gs.status.check()

    plain = None
    if wl['name'].startswith('mixed'):
        # the plain path on the same work: one sweep launch per connectome
        gs.reset_plain()
        gs.run_plain()
        torch.cuda.synchronize()
        gs.reset_plain()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record()
        gs.run_plain()
        p1.record()
        torch.cuda.synchronize()
        pms = p0.elapsed_time(p1)
        plain = {'value': round(node_steps(wl) / (pms / 1e3), 1), 'unit': UNIT,
                 'ms_per_step': round(pms, 3),
                 'path': 'per-step kernel, one sweep per connectome in %d-step launches, '
                         'connectomes in sequence' % PLAIN_CHUNK}
        if gs.path == 'groups':
            gms, gshapes = gs.plain_groups()
            plain['groups'] = {
                'value': round(node_steps(wl) / (gms / 1e3), 1), 'unit': UNIT,
                'ms_per_step': round(gms, 3),
                'shapes': [[x[0], x[1], 'pipelined' if x[3] == 2 else 'plain'] for x in gshapes],
                'path': 'the same group kernels, one connectome per launch set, connectomes in '
                        'sequence, each on its fastest shape alone (threads, cluster, kernel)'}
        return finish_mixed(args, wl, gs, world, rank, value, ms_per_step, clk, kern_ms, n_kern,
                            plain, torch, dist, barrier)

    # end-to-end through the public API: pinned host state in, FC out
    host_x0 = gs.x0.cpu().pin_memory()
    host_fc = torch.empty((wl['couplings'].size, wl['conn'].nnode, wl['conn'].nnode),
                          dtype=torch.float32).pin_memory() if wl['target'] is not None else None
    host_state = torch.empty_like(gs.sw.state, device='cpu').pin_memory()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        x0_dev = host_x0.cuda(non_blocking=True)
        gs.reset(x0_dev)
        _, fc = gs.run()
        if fc is not None:
            host_fc.copy_(fc[0], non_blocking=True)
        else:
            host_state.copy_(gs.sw.state, non_blocking=True)
        torch.cuda.synchronize()
    barrier()
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], device='cuda')
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_s = float(te.item())
    h2d = host_x0.numel() * 4
    d2h = (host_fc.numel() if host_fc is not None else host_state.numel()) * 4
    e2e = {'value': round(world * node_steps(wl) * args.steps / e2e_s, 1), 'unit': UNIT,
           'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': int(d2h)}

    line = {'metric': METRIC, 'value': round(value, 1), 'unit': UNIT, 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms_per_step, 3),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded connectomes: log-normal weights, uniform lengths)',
            'config': workload_config(wl), 'e2e': e2e,
            'gpu_launches': gs.launches_per_step() * args.steps,
            'roofline': roofline_entry(wl, gs.ns, kern_ms, args.steps),
            'clocks': clk, 'tpn': gs.tpn}
    line['config']['path'] = gs.path
    if rank == 0 and world == 1 and wl['name'] == 'kuramoto':
        # the reference's own GPU kernel beside the engine: at this workload's
        # size and at the DSL's default 32 x 32 sweep (1024 work items)
        line['reference_gpu'] = {
            'config_size': reference_gpu_kuramoto(wl, wl['couplings'].size),
            'sweep_1024': reference_gpu_kuramoto(wl, 1024),
            'engine_sweep_1024': engine_kuramoto_items(wl, 1024)}
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = (cpu_baseline_lems(wl) if wl['name'].startswith('lems')
                                else cpu_baseline(wl))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def finish_mixed(args, wl, gs, world, rank, value, ms_per_step, clk, kern_ms, n_kern, plain,
                 torch, dist, barrier):
    "e2e and the JSON line of the uneven-batch workload."
    host_x0 = [x.cpu().pin_memory() for x in gs.x0]
    host_st = [torch.empty_like(s.state, device='cpu').pin_memory() for s in gs.sets]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gs.reset([h.cuda(non_blocking=True) for h in host_x0])
        gs.run()
        for h, s in zip(host_st, gs.sets):
            h.copy_(s.state, non_blocking=True)
        torch.cuda.synchronize()
    barrier()
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], device='cuda')
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_s = float(te.item())
    nbytes = sum(h.numel() * 4 for h in host_x0)
    e2e = {'value': round(world * node_steps(wl) * args.steps / e2e_s, 1), 'unit': UNIT,
           'h2d_bytes_per_step': int(nbytes), 'd2h_bytes_per_step': int(nbytes)}
    if gs.path == 'groups':
        shapes = ', '.join('N=%d: %s %d threads x %d CTAs' % (
            s.N, 'pipelined' if tp == 2 else 'plain', t, c)
            for s, (t, c, _, tp) in zip(gs.sets, gs.batch.shapes))
        if gs.batch.step_ms is not None:
            shapes += '; groups banded into launch priorities by estimated run time'
        path = ('lane-interleaved groups (8 instances per lane slice), launch shapes per '
                'connectome %s[%s], ' % ('from the makespan-aware tuner ' if gs.batch.tuning
                                         else '', shapes))
    else:
        path = 'per-instance persistent kernels, '
    path += 'one CUDA graph' if gs.batch.graph is not None else 'direct launches'
    line = {'metric': METRIC, 'value': round(value, 1), 'unit': UNIT, 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms_per_step, 3),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded connectomes: log-normal weights, uniform lengths)',
            'config': dict(workload_config(wl), path=path),
            'e2e': e2e,
            'gpu_launches': gs.launches_per_step() * args.steps,
            'roofline': roofline_entry(wl, gs.ns, kern_ms, args.steps),
            'clocks': clk, 'plain': plain,
            'batched_vs_plain': round(value / plain['value'], 3) if plain else None}
    if plain and 'groups' in plain:
        line['batched_vs_plain_groups'] = round(value / plain['groups']['value'], 3)
    if gs.path == 'groups' and gs.batch.tuning:
        tun = gs.batch.tuning
        line['tuner'] = {k: (round(v, 3) if isinstance(v, float) else v) for k, v in tun.items()
                         if k in ('ms', 'default_ms', 'full_ms', 'full_default_ms', 'scale',
                                  'kept_default')}
        line['tuner']['trials'] = len(tun['trials'])
        line['tuner']['banded'] = tun['step_ms'] is not None
    if rank == 0 and world == 1 and not args.no_cpu:
        sample = gs.accuracy_run() if gs.path == 'groups' else None
        line['cpu_baseline'] = cpu_baseline_mixed(wl, sample, gs.sets if sample else None)
        acc = line['cpu_baseline'].pop('parity', None)
        if acc:
            line.update(acc)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def adjoint_finish(args, wl, gs, torch, world, rank, barrier_fn=None):
    "Time the adjoint fit (device-resident and end to end) and print its line."
    import torch.distributed as dist

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        gs.run()
    barrier()
    flush, wl['l2_note'] = l2_policy(torch)
    timer = StepTimer(torch, flush)
    clocks = ClockSampler(int(os.environ.get('LOCAL_RANK', '0')))
    clocks.start()
    timer.start()
    for _ in range(args.steps):
        timer.before_step()
        gs.run()
        timer.after_step()
    timer.stop()
    barrier()
    clocks.hold(gs.run)
    clk = clocks.stop()
    gs.prob.check()   # the status words of every timed call's kernels
    total_ms = timer.ms()
    t = torch.tensor([total_ms], device='cuda')
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    ms = total_ms / args.steps
    value = world * node_steps(wl) * args.steps / (total_ms / 1e3)
    # end to end: host G, eta in; gradients and loss back on the host
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loss = gs.prob.forward(wl['couplings'], wl['eta'])
        dG, deta = gs.prob.backward()
        out = (loss.cpu(), dG.cpu(), deta.cpu())
    barrier()
    e2e_s = time.perf_counter() - t0
    gs.prob.check()
    h2d = wl['couplings'].nbytes + wl['eta'].nbytes
    d2h = sum(o.numel() * o.element_size() for o in out)
    err = gs.grad_error()
    # forward, recomputation and reverse pass each stream the rings and state
    bpn = 3 * algorithmic_bytes_per_node_step(wl, 2)
    peaks = {}
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        peaks = json.load(open(p))
    hbm = peaks.get('hbm_gbs') or 6800.0
    ach = bpn * node_steps(wl) / (ms / 1e3) / 1e9
    line = {'metric': METRIC, 'value': round(value, 1), 'unit': UNIT, 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms, 3),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded connectome and target FC)',
            'config': dict(workload_config(wl), checkpoint_every=wl['ckpt'],
                           loss='MSE of FC (r series) vs target', gradients='G [256], eta [256, 84]',
                           path=gs.path),
            'e2e': {'value': round(world * node_steps(wl) * args.steps / e2e_s, 1), 'unit': UNIT,
                    'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': int(d2h)},
            'gpu_launches': gs.launches_per_step() * args.steps,
            'roofline': {'bound': 'hbm', 'achieved': round(ach, 1), 'peak': hbm, 'unit': 'GB/s',
                         'frac': round(ach / hbm, 4), 'traffic': None,
                         'peak_source': 'measured' if peaks.get('hbm_gbs') else 'fallback',
                         'algorithmic_bytes_per_node_step': round(bpn, 2),
                         'note': 'value counts forward node-steps over forward + backward time; '
                                 'bytes = 3 passes (forward, recomputation, reverse) of 4E + 16'},
            'gradient_rel_err_vs_fp64': err, 'clocks': clk}
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline_adjoint(wl)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def mixed_parity(orc, sample, sets, x0s, cores):
    """State error of the sampled instances of the benchmarked batch (GPU,
    first 1000 steps) against the oracle run on the same instances: the
    FP32 restatement and the FP64 one (max |gpu - oracle| / max |oracle|,
    worst over the sampled instances)."""
    e32, e64, desc = 0.0, 0.0, []
    for smp, gset, x0 in zip(sample, sets, x0s):
        idx = smp['idx']
        sub = _SubSet(gset, idx, x0)
        got = smp['state'].astype(np.float64)
        for real in ('f32', 'f64'):
            r = orc.run_groups_like(sub, sub.x0, smp['nsteps'], real=real, nthreads=cores)['state']
            r = np.asarray(r, np.float64)
            err = float(np.abs(got - r).max() / max(np.abs(r).max(), 1e-30))
            if real == 'f32':
                e32 = max(e32, err)
            else:
                e64 = max(e64, err)
        desc.append('N=%d: instances %s' % (gset.N, [int(i) for i in idx]))
    return {'state_rel_err_vs_oracle': float('%.3g' % e32),
            'state_rel_err_vs_fp64': float('%.3g' % e64),
            'parity_sample': '%d steps from the initial state, %s; tolerance 1e-4' % (
                sample[0]['nsteps'], '; '.join(desc))}


class _SubSet:
    """The view of a GroupSet that the oracle's run_groups_like reads,
    restricted to some instances (same delays, parameters, seeds, ids)."""

    def __init__(self, gs, idx, x0):
        import torch
        self.n = len(idx)
        for a in ('N', 'ns', 'flags', 'model_id', 'cfun_id', 'row_np', 'col_np', 'w_np', 'dt',
                  'sigma', 'consts', 'cf_b', 'cf_p', 'seed', 'trace_every', 'trace_len',
                  'trace_nobs', 'bold_period', 'bold_len', 'delay_tables', 'lognh', 'gtab'):
            setattr(self, a, getattr(gs, a))
        self.bold_obs = gs.bold_obs
        ii = torch.from_numpy(np.asarray(idx)).cuda()
        self._gi = gs._gi[ii]
        self._li = gs._li[ii]
        self.gnparam = gs.gnparam
        self.grp_of = gs.grp_of[idx]
        self.cf_a = gs.cf_a[idx]
        self.inst_ids = gs.inst_ids[idx]
        self.x0 = np.asarray(x0, np.float32)[idx]


def cpu_baseline_mixed(wl, sample=None, sets=None, budget_s=12.0):
    """The oracle on a bounded sample of the uneven batch (instances of every
    connectome); with `sample` (MixedStep.accuracy_run) it also checks the
    GPU states of the sampled instances against the oracle ('parity')."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import pyoracle as orc
    from tvb_hpc import model as mdl
    m = getattr(mdl, wl['model'])()
    kid, consts, sigma = m.engine_spec()
    cores = os.cpu_count() or 1
    parity = None
    if sample is not None:
        parity = mixed_parity(orc, sample, sets, [p['x0'] for p in wl['parts']], cores)
    done_ns, el_tot, desc = 0.0, 0.0, []
    for p in wl['parts']:
        c = p['conn']
        n_inst = min(p['couplings'].size, cores)
        delays = np.stack([c.delays(s, wl['dt'], 'ceil') for s in p['speeds'][:n_inst]])
        nh = int(2 ** np.ceil(np.log2(delays.max() + 2)))
        def run(nsteps):
            t = time.perf_counter()
            orc.run(kid, 0, c.row, c.col, c.wnz, nh, nsteps, wl['dt'], delays,
                    p['couplings'][:n_inst], p['nparam'][:n_inst, :, 0], p['x0'][:n_inst],
                    flags=orc.F_NOISE, sigma=sigma, consts=consts, seed=p['seed'], nthreads=cores)
            return time.perf_counter() - t

        probe = 100
        per_step = run(probe) / probe
        nsteps = int(np.clip(budget_s / len(wl['parts']) / max(per_step, 1e-9), probe, 50000))
        el = run(nsteps)
        done_ns += n_inst * c.nnode * nsteps
        el_tot += el
        desc.append('N=%d: %d inst x %d steps' % (c.nnode, n_inst, nsteps))
    # the second shape: one instance per call on one core, as the
    # reference's examples run their sweeps (hackathon.py:67-69)
    c = wl['parts'][0]['conn']
    p = wl['parts'][0]
    d1 = c.delays(p['speeds'][0], wl['dt'], 'ceil')[None]
    nh = int(2 ** np.ceil(np.log2(d1.max() + 2)))
    n1 = 2000
    t = time.perf_counter()
    orc.run(kid, 0, c.row, c.col, c.wnz, nh, n1, wl['dt'], d1, p['couplings'][:1],
            p['nparam'][:1, :, 0], p['x0'][:1], flags=orc.F_NOISE, sigma=sigma, consts=consts,
            seed=p['seed'], nthreads=1)
    one = c.nnode * n1 / (time.perf_counter() - t)
    out = {'value': round(done_ns / el_tot, 1), 'unit': UNIT, 'cores': cores, 'kind': 'port',
           'sample': '; '.join(desc) + ' (%.1f s), oracle C + OpenMP, -O3' % el_tot,
           'one_instance_one_core': {'value': round(one, 1), 'unit': UNIT,
                                     'sample': 'N=%d, 1 instance x %d steps' % (c.nnode, n1)}}
    if parity is not None:
        out['parity'] = parity
    return out


def serve_window(rate, seconds, max_inst, chunk, conns, seed=7, drain_s=60.0, sample_s=0.5,
                 max_ctas=None):
    """One serving run: Poisson arrivals at `rate` per second for `seconds`
    (models Kuramoto / 2-D oscillator / MPR, N in {68, 84, 192, 400, 998},
    instances log-uniform in 1..max_inst, steps log-uniform in 1k..100k, 10 %
    of MPR requests with FC-fit gradients) into Server(native=True) with a
    180 GB budget; ticks until every request is done or `drain_s` after the
    window, then cancels what is left.  Sampled every `sample_s`: the
    requests in the system (arrived, not finished) and the work backlog
    (node-steps arrived minus node-steps handed to the device: taken, or in
    a chunk running now).  The queue
    kept up when the backlog does not grow over the second half of the
    window (least-squares slope below 5 % of the offered node-steps/s) and
    no request was left at the cut-off; served node-steps/s count every
    step taken up to the cut-off."""
    import torch
    from tvb_hpc import serve
    rng = np.random.default_rng(seed)
    n_req = max(1, int(rate * seconds))
    reqs = serve.random_requests(n_req, rate, rng, conns, inst=(1, max_inst), steps=(1000, 100000))
    srv = serve.Server(chunk=chunk, native=True, max_ctas=max_ctas)
    t_start = time.perf_counter()
    for r in reqs:
        r.arrival += t_start
        srv.submit(r)
    samples, next_s = [], 0.0
    stop = t_start + seconds + drain_s
    while srv.busy and time.perf_counter() < stop:
        srv.run(until_empty=False)
        now = time.perf_counter()
        if now - t_start >= next_s:
            arr = [r for r in reqs if r.arrival <= now]
            finished = sum(1 for r in arr if r.finished is not None)
            # work not yet handed to the device: the pool's running chunks
            # count as taken (they are on the GPU; completed-only counts would
            # show the running chunks of a rolling pool as a growing backlog)
            backlog = (sum(r.node_steps for r in arr if r.error is None)
                       - srv.work_done(arr, issued=True))
            samples.append((round(now - t_start, 2), len(arr) - finished, float('%.4g' % backlog)))
            next_s += sample_s
    t_cut = time.perf_counter() - t_start
    work = srv.work_done(reqs)
    left = [r for r in reqs if r.finished is None]
    for r in left:
        srv.cancel(r.rid)
    srv._collect(wait=True)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_start
    done = [r for r in reqs if r.finished is not None and r.error is None]
    failed = [r for r in reqs if r.error is not None]
    lat = np.array([r.finished - r.arrival for r in done]) if done else np.zeros(1)
    half = [x for x in samples if seconds / 2 <= x[0] <= seconds]

    def slope(k):
        return (float(np.polyfit([x[0] for x in half], [x[k] for x in half], 1)[0])
                if len(half) > 2 else 0.0)

    offered = sum(r.node_steps for r in reqs) / seconds
    return {
        'rate_per_s': rate, 'window_s': seconds, 'requests': n_req, 'completed': len(done),
        'failed': len(failed), 'left_at_cutoff': len(left),
        'gradient_requests': sum(1 for r in reqs if r.want_grad),
        'p50_latency_s': round(float(np.percentile(lat, 50)), 3),
        'p99_latency_s': round(float(np.percentile(lat, 99)), 3),
        'latency_of': 'completed requests',
        'offered_node_steps_per_s': round(offered, 1),
        'served_node_steps_per_s': round(work / max(t_cut, 1e-9), 1),
        'wall_s': round(wall, 2),
        'in_system_slope_per_s': round(slope(1), 3),
        'backlog_slope_node_steps_per_s': float('%.4g' % slope(2)),
        'queue_kept_up': bool(slope(2) < 0.05 * offered and not left),
        'samples_t_insystem_backlog': samples[::max(1, len(samples) // 60)],
    }, reqs


def serve_arm(args):
    """Serving loop at the configured rate and window (default: 50 requests
    per second for 60 s, up to 4096 instances, 1k-100k steps, 10 % FC-fit
    gradient requests, 180 GB budget): p50/p99 latency, offered vs served
    node-steps/s, requests in the system over time and whether the queue
    kept up; then a sweep of arrival rates over shorter windows for the
    largest rate the queue keeps up with; then the plain paths on the same
    requests (each alone, group kernel and per-step kernel)."""
    import torch
    torch.cuda.set_device(0)
    from tvb_hpc import network, serve, _native
    _native.load()
    conns = []
    for k, (N, dens, _) in enumerate(MIXED_SPEC):
        w, ln = network.synthetic_connectome(N, dens, seed=k)
        conns.append(network.Connectivity.from_dense(w, ln))
    # warm-up: load every kernel once, the FC-fit gradient path included
    warm = serve.Server(chunk=args.serve_chunk, native=True)
    for r in serve.random_requests(8, 1e6, np.random.default_rng(1), conns[:2], inst=(1, 2),
                                   steps=(200, 300), grad_frac=1.0):
        warm.submit(r)
    warm.run()
    torch.cuda.synchronize()
    main, reqs = serve_window(args.serve_rate, args.serve_seconds, args.serve_max_inst,
                              args.serve_chunk, conns, drain_s=args.serve_drain,
                              max_ctas=args.serve_max_ctas)
    sweep = []
    for rate in [float(x) for x in args.serve_sweep.split(',') if x]:
        res, _ = serve_window(rate, args.serve_sweep_seconds, args.serve_max_inst, args.serve_chunk,
                              conns, seed=11, drain_s=args.serve_drain,
                              max_ctas=args.serve_max_ctas)
        res.pop('samples_t_insystem_backlog')
        sweep.append(res)
    kept = [x['rate_per_s'] for x in sweep if x['queue_kept_up']]
    # a second reading of the same runs: the requests in the system do not
    # grow over the second half of the window (slope below 5 % of the arrival
    # rate) and none is left at the cut-off
    kept_req = [x['rate_per_s'] for x in sweep
                if x['left_at_cutoff'] == 0 and x['in_system_slope_per_s'] < 0.05 * x['rate_per_s']]
    if args.serve_no_plain:
        plain_groups = plain = {'value': None}
    else:
        plain_groups = serve_plain_groups(reqs, budget_s=args.serve_plain_seconds)
        plain = serve_plain(reqs, budget_s=args.serve_plain_seconds)
    served = main['served_node_steps_per_s']
    line = {'metric': METRIC, 'value': served, 'unit': UNIT, 'n_gpus': 1,
            'steps': 1, 'warmup': 1, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded connectomes)',
            'config': {'workload': 'serve', 'rate_per_s': args.serve_rate,
                       'admission_cap_ctas': args.serve_max_ctas,
                       'window_s': args.serve_seconds, 'max_instances': args.serve_max_inst,
                       'steps': '1k-100k log-uniform', 'gradient_fraction_of_mpr': 0.1,
                       'chunk_steps': args.serve_chunk, 'hbm_budget_gb': 180,
                       'path': 'Server(native=True): C++ pool (group kernels, pipelined where '
                               'the delays allow) for requests without gradients, Python path '
                               '+ FC-fit adjoint worker for gradient requests'},
            'serve': main,
            'rate_sweep': sweep,
            'largest_rate_kept_up': max(kept) if kept else None,
            'largest_rate_kept_up_by_requests': max(kept_req) if kept_req else None,
            'plain_groups': plain_groups,
            'plain': plain,
            'served_vs_plain_groups': (round(served / plain_groups['value'], 3)
                                       if plain_groups['value'] else None),
            'served_vs_plain': round(served / plain['value'], 3) if plain['value'] else None}
    print(json.dumps(line), flush=True)


def serve_plain_groups(reqs, budget_s=20.0):
    """The best plain path on the same requests: each request alone on the
    group kernel (GroupSet, pipelined where the delays allow), one launch
    set per request, requests one after the other in arrival order, until
    `budget_s` of GPU time is spent (gradient requests run forward only)."""
    import torch
    from tvb_hpc import groups, scheme, serve
    done, el, n_req = 0.0, 0.0, 0
    for r in sorted(reqs, key=lambda r: r.arrival):
        if el >= budget_s:
            break
        M, C, noise = serve.MODELS[r.model]
        m = M()
        cf = C(m)
        scm = scheme.EulerMaryuyamaStep(r.dt) if noise else scheme.EulerStep(r.dt)
        try:
            gs = groups.GroupSet(m, cf, scm, r.conn, dt=r.dt, couplings=r.couplings,
                                 speeds=r.speeds, state0=r.x0, nparam=r.nparam, seed=r.seed)
        except ValueError:
            continue
        gs.set_shape(*groups.pipelined_shape(gs))
        left = int(r.nsteps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        while left > 0 and el + (time.perf_counter() - t0) < budget_s:
            n = min(20000, left)
            gs.run(n)
            left -= n
        el += time.perf_counter() - t0
        done += float(r.couplings.size) * r.conn.nnode * (r.nsteps - left)
        n_req += 1
        del gs
    return {'value': round(done / el, 1) if el > 0 else None, 'unit': UNIT, 'requests': n_req,
            'seconds': round(el, 3),
            'path': 'each request alone: group kernel (pipelined where the delays allow), '
                    'chunks of 20000 steps'}


def serve_plain(reqs, budget_s=20.0):
    """The plain path on the same requests: each request alone, as one
    sweep of the per-step kernel launched in PLAIN_CHUNK-step chunks and
    synchronised after each chunk (the reference launcher's loop,
    dsl/dsl_cuda/example/cuda_run.py:124-142), requests one after the other
    in arrival order, until `budget_s` of GPU time is spent; returns the
    measured node-steps/s (gradient requests run forward only)."""
    import torch
    from tvb_hpc import engine, scheme, serve
    done, el, n_req = 0.0, 0.0, 0
    for r in sorted(reqs, key=lambda r: r.arrival):
        if el >= budget_s:
            break
        M, C, noise = serve.MODELS[r.model]
        m = M()
        cf = C(m)
        scm = scheme.EulerMaryuyamaStep(r.dt) if noise else scheme.EulerStep(r.dt)
        sw = engine.Sweep(m, cf, scm, r.conn, dt=r.dt, couplings=r.couplings, speeds=r.speeds,
                          state0=r.x0, nparam=r.nparam, seed=r.seed, blocked=False, tpn=2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        left = r.nsteps
        while left > 0 and el + (time.perf_counter() - t0) < budget_s:
            n = min(PLAIN_CHUNK, left)
            sw.run(n)          # synchronises and checks the status word
            left -= n
        el += time.perf_counter() - t0
        done += float(r.couplings.size) * r.conn.nnode * (r.nsteps - left)
        n_req += 1
    return {'value': round(done / el, 1) if el > 0 else None, 'unit': UNIT, 'requests': n_req,
            'seconds': round(el, 3),
            'path': 'each request alone: per-step kernel, %d-step launches, host sync per launch'
                    % PLAIN_CHUNK}


def reference_arm(args):
    "The reference path's CPU implementation (the oracle port) on host cores."
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]()
    vals = []
    base = (cpu_baseline_mixed if wl['name'].startswith('mixed') else
            cpu_baseline_lems if wl['name'].startswith('lems') else
            cpu_baseline_adjoint if wl['name'] == 'adjoint' else cpu_baseline)
    for i in range(args.warmup + args.steps):
        cb = base(wl, budget_s=args.ref_seconds)
        if i >= args.warmup:
            vals.append(cb['value'])
    v = float(np.median(vals))
    cb['value'] = round(v, 1)
    wl['l2_note'] = 'host arm: the CPU caches, not timed on the device'
    line = {'metric': METRIC, 'value': round(v, 1), 'unit': UNIT, 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded connectomes: log-normal weights, uniform lengths)', 'impl': 'reference',
            'config': workload_config(wl), 'cpu_baseline': cb,
            'e2e': {'value': round(v, 1), 'unit': UNIT, 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split('\n')[1])
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--workload', default='mixed', choices=sorted(WORKLOADS) + ['serve'])
    ap.add_argument('--serve-rate', type=float, default=50.0)
    ap.add_argument('--serve-seconds', type=float, default=60.0)
    ap.add_argument('--serve-max-inst', type=int, default=4096)
    ap.add_argument('--serve-drain', type=float, default=60.0,
                    help='seconds after the arrival window before unfinished requests are cancelled')
    ap.add_argument('--serve-sweep', default='4,6,8,10',
                    help='arrival rates of the stability sweep (comma-separated, empty: none)')
    ap.add_argument('--serve-sweep-seconds', type=float, default=60.0)
    ap.add_argument('--serve-max-ctas', type=int, default=None,
                    help='native pool admission cap in resident CTAs (0: none; default: the pool\'s)')
    ap.add_argument('--serve-no-plain', action='store_true', help='skip the plain denominators')
    ap.add_argument('--serve-chunk', type=int, default=5000)
    ap.add_argument('--serve-plain-seconds', type=float, default=20.0)
    ap.add_argument('--impl', default='engine', choices=['engine', 'reference'])
    ap.add_argument('--no-cpu', action='store_true', help='skip the cpu_baseline leg')
    ap.add_argument('--ref-seconds', type=float, default=8.0)
    ap.add_argument('--tpn', type=int, default=None, help='fix the gather width (skip autotune)')
    ap.add_argument('--warps', type=int, default=None, help='fix the CTA width of the blocked kernel')
    ap.add_argument('--path', default='groups', choices=['groups', 'instances'],
                    help='lane-interleaved groups (separable couplings) or per-instance kernels')
    ap.add_argument('--no-graph', action='store_true',
                    help='launch the batch directly instead of replaying a CUDA graph')
    ap.add_argument('--no-tune', action='store_true',
                    help='mixed batch: rule-based launch shapes instead of the batch tuner')
    ap.add_argument('--pipelined', action='store_true',
                    help='with --no-tune: the pipelined kernel on its smallest cluster where it '
                         'applies (groups.pipelined_shape), else the plain default')
    args = ap.parse_args()
    if args.impl == 'reference':
        reference_arm(args)
    elif args.workload == 'serve':
        serve_arm(args)
    else:
        gpu_arm(args)


if __name__ == '__main__':
    main()
