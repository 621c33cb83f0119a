"""
Serving loop with continuous batching for sweep requests.

A request is a parameter sweep: a model (Kuramoto, G2DO or MPR) on a
connectome, a number of instances, a number of steps, seeds -- optionally
with FC-fit gradients (MPR, through tvb_hpc.adjoint).  The server keeps every
admitted request's state, parameters and history rings resident in device
memory and advances all of them together:

  tick:
    1. admit queued requests (arrival time <= now) while their device
       footprint fits the HBM budget;
    2. advance every active request by min(chunk, steps left): requests run
       as lane-interleaved groups (tvbg_group_run, one forked stream per
       request), gradient requests as one persistent batch launch per model
       (tvbg_batch_run), all on the device at once;
    3. retire requests that reached their step count: copy the final state
       to the host, free the device memory, record latency; FC-fit gradient
       requests then run their recomputation and adjoint on a worker thread
       (own stream) and finish when it does.

Requests that arrive while a tick runs are admitted while the device runs
that tick (their state is built on a side stream) and join at the next
tick, as slots and memory free up; their work overlaps on the device with
the requests already running.  Chunk boundaries are exact (the step kernels
resume bit-for-bit from the resident state and ring), and every request
keeps its own Philox key (request seed, request-local instance id) and
launch shape, so a request's result is the same alone and in any mix.

The reference has no serving layer; its CUDA launcher runs one sweep per
call and copies results back after every chunk
(dsl/dsl_cuda/example/cuda_run.py:124-142).
"""

import concurrent.futures
import time
from dataclasses import dataclass, field

import numpy as np

from . import model as mdl, coupling as cpl, scheme as sch
from .engine import InstanceSet, Batch
from .groups import GroupSet, GroupBatch
from .utils import getLogger

LOG = getLogger(__name__)

MODELS = {
    'Kuramoto': (mdl.Kuramoto, cpl.Kuramoto, False),
    'G2DO': (mdl.Generic2dOscillator, cpl.Diff, True),
    'MPR': (mdl.MPR, cpl.Linear, True),
}


@dataclass
class Request:
    rid: int
    model: str
    conn: object
    couplings: np.ndarray
    speeds: np.ndarray
    x0: np.ndarray
    nsteps: int
    nparam: object = None
    seed: int = 0
    dt: float = 0.1
    want_grad: bool = False
    target: object = None
    arrival: float = 0.0
    # filled by the server
    admitted: float = None
    finished: float = None
    state: np.ndarray = None
    grad: tuple = None
    steps_done: int = 0
    iset: object = field(default=None, repr=False)
    nbytes: int = 0
    error: str = None       # why the request failed (it can never fit the budget)

    @property
    def node_steps(self):
        return float(self.couplings.size) * self.conn.nnode * self.nsteps

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def footprint(req):
    """Device bytes a request needs (rings, state, parameters, edges),
    estimated; a gradient request adds the FC-fit adjoint's memory
    (adjoint_bytes), which it holds until its gradients are done."""
    from .engine import plan_ring
    N, I = req.conn.nnode, req.couplings.size
    d = req.conn.delays(float(np.min(req.speeds)), req.dt, 'ceil')
    lognh = plan_ring(int(d.min()), int(d.max()), extra=8)[0]
    ring = N * ((1 << lognh) + 8) * 4
    base = I * (ring + N * 4 * 6 + 512) + req.conn.nnz * 8 * len(np.unique(req.speeds))
    if req.want_grad and req.model == 'MPR' and req.target is not None:
        base += adjoint_bytes(I, N, int(req.nsteps), 1 << lognh)
    return base


def adjoint_bytes(I, N, T, nh, checkpoint_every=100, trace_budget=2 << 30):
    """Device bytes of adjoint.FCFit for I instances, N nodes, T steps:
    the rate series (FP32 trace), dL/dr (FP32), the loss scratch (FC and A),
    one state + ring checkpoint per chunk of checkpoint_every steps, the
    recomputation (windows of segments: r, V, S traces and working copies of
    their checkpoints, at most trace_budget) and the adjoint ring."""
    C = int(checkpoint_every)
    S = -(-T // C)
    series = I * T * N * (4 + 4)               # r trace and dL/dr (FP32)
    ckpt = S * I * N * (nh + 8 + 2) * 4
    per_seg = I * C * N * 3 * 4 + I * N * (nh + 8 + 2) * 4
    recompute = max(per_seg, min(S * per_seg, int(trace_budget)))
    return series + ckpt + recompute + I * N * N * (8 * 2 + 4) + I * N * 8 * 3


class Server:
    """
    Continuous-batching server.  `hbm_budget` bounds the device bytes of the
    admitted requests; `chunk` is the number of steps every active request
    advances per tick.  With `native=True` the requests without gradients
    run in the C++ pool (NativeServer, sharing the budget and the ticks)
    and only the gradient requests take the Python path.
    """

    def __init__(self, hbm_budget=180e9, chunk=2000, clock=time.perf_counter, native=False,
                 max_ctas=None):
        import torch
        self.torch = torch
        self.budget = float(hbm_budget)
        self.chunk = int(chunk)
        self.clock = clock
        self.queue = []
        self.active = []
        self.done = []
        self.used = 0
        self.ticks = 0
        self.node_steps = 0.0
        # wall time split per phase (admission incl. set-up, launch
        # preparation, device, retirement)
        self.phase_s = dict(admit=0.0, prepare=0.0, device=0.0, retire=0.0)
        self.side = torch.cuda.Stream()
        self.grad_stream = torch.cuda.Stream()
        self.pool = concurrent.futures.ThreadPoolExecutor(max_workers=1)
        self.pending = []
        self.cancelled = []
        self.failed = []
        # requests without gradients in the C++ pool: waiting for their
        # arrival here, then in the pool until done
        self.native = NativeServer(hbm_budget, chunk, clock, max_ctas) if native else None
        self.native_wait = []
        self.native_busy = False
        self._native_seen = 0

    def submit(self, req):
        if self.native is not None and not req.want_grad:
            self.native_wait.append(req)
        else:
            self.queue.append(req)

    @property
    def busy(self):
        "Work is queued, running or computing gradients."
        return bool(self.queue or self.active or self.pending or self.native_wait
                    or self.native_busy)

    def _native_tick(self):
        """Hand arrived requests to the pool and run one pool tick (its
        chunks overlap this tick's Python-path launches on the device).  The
        pool admits within what the Python path leaves of the budget, so the
        two together never hold more than the budget."""
        from . import _native as nat
        now = self.clock()
        keep = []
        for r in sorted(self.native_wait, key=lambda r: r.arrival):
            if r.arrival > now:
                keep.append(r)
                continue
            try:
                self.native.submit(r)
            except nat.TvbgError as e:
                if e.code == nat.TVBG_EUNSUPPORTED:
                    self.queue.append(r)   # delays too short for the group kernel: per-step kernel
                elif e.code == nat.TVBG_EINVAL:
                    self._fail(r, str(e))  # e.g. the request alone exceeds the budget
                else:
                    raise
        self.native_wait = keep
        self.native.set_budget(max(0, int(self.budget - self.used)))
        a, q = self.native.tick()
        self.native_busy = bool(a or q)
        for r in self.native.done[self._native_seen:]:
            self.done.append(r)
            self.node_steps += r.node_steps
        self._native_seen = len(self.native.done)

    def poll(self, rid):
        """State of request `rid`: 'queued', 'active' (its steps are running),
        'gradient' (its FC-fit gradients are being computed), 'done',
        'cancelled', 'failed' (it can never fit the budget; req.error says why),
        or None if the server has never seen it."""
        if self.native is not None:
            if any(r.rid == rid for r in self.native_wait):
                return 'queued'
            st = self.native.poll(rid)
            if st is not None:
                return st
        for name, reqs in (('queued', self.queue), ('active', self.active),
                           ('gradient', [r for r, _ in self.pending]), ('done', self.done),
                           ('cancelled', self.cancelled), ('failed', self.failed)):
            if any(r.rid == rid for r in reqs):
                return name
        return None

    def cancel(self, rid):
        """Drop a queued or active request between ticks; an active one gives
        its device memory back at once.  Returns True if it was dropped (a
        request already in its gradient phase or done is not)."""
        if self.native is not None:
            for r in self.native_wait:
                if r.rid == rid:
                    self.native_wait.remove(r)
                    self.cancelled.append(r)
                    return True
            if self.native.poll(rid) is not None:
                return self.native.cancel(rid)
        for lst in (self.queue, self.active):
            for r in lst:
                if r.rid == rid:
                    lst.remove(r)
                    if r.iset is not None:
                        self.used -= r.nbytes
                        r.iset = None
                    self.cancelled.append(r)
                    return True
        return False

    def _admit(self, now, into=None):
        """Admit queued requests that have arrived and fit the budget; their
        device state is built on the current stream and appended to `into`
        (default: the active list)."""
        torch = self.torch
        into = self.active if into is None else into
        keep = []
        for req in sorted(self.queue, key=lambda r: r.arrival):
            if req.arrival > now:
                keep.append(req)
                continue
            need = footprint(req)
            if need > self.budget:     # can never fit: fail it rather than queue it forever
                self._fail(req, 'device footprint %d bytes exceeds the budget %d' % (
                    need, int(self.budget)))
                continue
            free = torch.cuda.mem_get_info()[0]
            held = self.used + (self.native.used() if self.native is not None else 0)
            if held + need > self.budget or need > free:
                keep.append(req)
                continue
            req.iset = self._make_set(req)
            req.admitted = self.clock()
            req.nbytes = need
            self.used += need
            into.append(req)
        self.queue = keep

    def _fail(self, req, why):
        req.error = why
        req.finished = self.clock()
        self.failed.append(req)

    @staticmethod
    def _make_set(req):
        """Lane-interleaved groups (every model/coupling pair the server offers),
        per-instance kernels for gradient requests (the adjoint recomputes
        from per-instance rings) and where the group kernel's blocks do not
        fit the delays."""
        M, C, noise = MODELS[req.model]
        m = M()
        cf = C(m)
        scm = (sch.EulerMaryuyamaStep(req.dt) if (noise and not req.want_grad)
               else sch.EulerStep(req.dt))
        kw = dict(dt=req.dt, couplings=req.couplings, speeds=req.speeds, state0=req.x0,
                  nparam=req.nparam, seed=req.seed)
        if not req.want_grad:
            try:
                return GroupSet(m, cf, scm, req.conn, **kw)
            except ValueError:      # delays too short for the group kernel's blocks
                pass
        return InstanceSet(m, cf, scm, req.conn, blocked=False if req.want_grad else 'auto', **kw)

    def _retire(self, req):
        req.state = req.iset.state.cpu().numpy()
        req.iset = None
        if req.want_grad and req.model == 'MPR' and req.target is not None:
            # FC-fit gradients (recomputed forward + adjoint) run on a worker
            # thread with its own stream, so they hold up no tick; the
            # request keeps its bytes (its footprint counts the adjoint)
            # until they are done
            self.pending.append((req, self.pool.submit(self._gradient, req)))
            return
        self.used -= req.nbytes
        req.finished = self.clock()
        self.done.append(req)

    def _gradient(self, req):
        from .adjoint import FCFit
        torch = self.torch
        with torch.cuda.stream(self.grad_stream):
            prob = FCFit(req.conn, req.dt, float(req.speeds[0]), req.x0, req.target, req.nsteps)
            prob.forward(req.couplings, np.asarray(req.nparam).reshape(req.couplings.size, -1))
            out = tuple(t.cpu().numpy() for t in prob.backward())
            prob.check()   # the status words of its kernels
        del prob
        torch.cuda.empty_cache()   # give the adjoint's memory back for admission
        return out

    def _collect(self, wait=False):
        "Finish the gradient requests whose worker job is done."
        keep = []
        for req, fut in self.pending:
            if wait or fut.done():
                req.grad = fut.result()
                self.used -= req.nbytes
                req.finished = self.clock()
                self.done.append(req)
            else:
                keep.append((req, fut))
        self.pending = keep

    def tick(self):
        "Admit, advance every active request by one chunk, retire; returns work done."
        t_a = time.perf_counter()
        self._admit(self.clock())
        t_p = time.perf_counter()
        self.phase_s['admit'] += t_p - t_a
        if not self.active:
            if self.native is not None:
                self._native_tick()
                self.phase_s['device'] += time.perf_counter() - t_p
                self._collect()
                self.ticks += 1
            return 0.0
        by_model, grouped = {}, []
        for req in self.active:
            if isinstance(req.iset, GroupSet):
                grouped.append(req)
            else:
                by_model.setdefault((req.model, req.want_grad), []).append(req)
        batches = []
        work = 0.0
        if grouped:
            steps = [min(self.chunk, r.nsteps - r.steps_done) for r in grouped]
            gb = GroupBatch([r.iset for r in grouped], steps)
            gb.launch()
            batches.append((gb, grouped, steps))
        for reqs in by_model.values():
            steps = [min(self.chunk, r.nsteps - r.steps_done) for r in reqs]
            b = Batch([r.iset for r in reqs], steps)
            b.launch()
            batches.append((b, reqs, steps))
        for b, reqs, steps in batches:
            work += sum(r.couplings.size * r.conn.nnode * n for r, n in zip(reqs, steps))
        done = self.torch.cuda.Event()
        done.record()          # after every launch (forked streams join the current one)
        t_d = time.perf_counter()
        self.phase_s['prepare'] += t_d - t_p
        # while the device runs this chunk, admit what has arrived meanwhile:
        # the new requests' device state is built on a side stream and they
        # join at the next tick
        fresh = []
        if self.queue:
            with self.torch.cuda.stream(self.side):
                self._admit(self.clock(), into=fresh)
        t_s = time.perf_counter()
        self.phase_s['admit'] += t_s - t_d
        if self.native is not None:
            self._native_tick()
            # the pool's requests go on at their own pace while this tick's
            # Python-path chunk runs
            while not done.query():
                self._native_tick()
                if not self.native_busy:
                    time.sleep(0.0005)
        # wait for this tick's launches and the admissions' copies only (a
        # gradient job may be running on its own stream)
        done.synchronize()
        self.side.synchronize()
        t_r = time.perf_counter()
        self.phase_s['device'] += t_r - t_s
        for b, reqs, steps in batches:
            b.status.check()
            for r, n in zip(reqs, steps):
                r.steps_done += n
                r.iset.t += n
        finished = [r for r in self.active if r.steps_done >= r.nsteps]
        self.active = [r for r in self.active if r.steps_done < r.nsteps] + fresh
        for r in finished:
            self._retire(r)
        self._collect()
        self.phase_s['retire'] += time.perf_counter() - t_r
        self.ticks += 1
        self.node_steps += work
        return work

    def run(self, until_empty=True, max_ticks=None):
        while self.busy:
            if max_ticks is not None and self.ticks >= max_ticks:
                break
            if not (self.active or self.queue or self.native_wait or self.native_busy):
                self._collect(wait=True)     # only gradient jobs are left
                break
            waiting = self.queue + self.native_wait
            if not self.active and not self.native_busy and waiting:
                nxt = min(r.arrival for r in waiting)
                wait = nxt - self.clock()
                if wait > 0:
                    time.sleep(min(wait, 0.05))
            self.tick()
            if not until_empty:
                break
        return self.done

    def work_done(self, reqs, issued=False):
        """Node-steps taken so far by `reqs` (submitted to this server),
        finished or not; with `issued`, the pool's running chunks count too
        (the work handed to the device)."""
        total = 0.0
        for r in reqs:
            if r.error is not None:
                continue
            if r.finished is not None and r.state is not None:
                steps = r.nsteps
            elif self.native is not None and r.rid in self.native.reqs:
                steps = (self.native.steps_issued(r.rid) if issued
                         else self.native.steps_done(r.rid))
            else:
                steps = r.steps_done
            total += float(r.couplings.size) * r.conn.nnode * steps
        return total

    def stats(self):
        lat = np.array([r.latency for r in self.done if r.latency is not None])
        out = {'requests': len(self.done), 'ticks': self.ticks, 'node_steps': self.node_steps,
               'phase_s': {k: round(v, 3) for k, v in self.phase_s.items()}}
        if lat.size:
            out.update(p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)))
        return out


class NativeServer:
    """
    The serving pool in native code (tvbg_serve_*): the same continuous
    batching as Server for requests without gradients, run by the C++ pool
    -- requests copied in, admitted by the HBM budget, advanced chunk by
    chunk on per-request streams (each at its own pace), retired,
    polled and cancelled by id.
    Each request's result equals lane-interleaved groups of the same inputs
    (GroupSet), alone or in any mix.
    """

    def __init__(self, hbm_budget=180e9, chunk=2000, clock=time.perf_counter, max_ctas=None):
        import ctypes
        from . import _native as nat
        self.nat = nat
        self.lib = nat.load()
        self.clock = clock
        h = ctypes.c_void_p()
        nat.check(self.lib.tvbg_serve_create(int(hbm_budget), int(chunk), None, ctypes.byref(h)))
        self.h = h
        if max_ctas is not None:    # admission cap in resident CTAs (0: none; -1: the default)
            nat.check(self.lib.tvbg_serve_set_concurrency(h, int(max_ctas)))
        self.reqs = {}          # rid -> (Request, native id, kept host arrays)
        self.by_nid = {}        # native id -> rid
        self.done = []
        self.ticks = 0
        self._fin = np.zeros(4096, np.int64)

    def close(self):
        if self.h is not None:
            self.lib.tvbg_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, req):
        """Copy a request into the pool (queued until it fits); gradient
        requests need Server."""
        import ctypes
        nat = self.nat
        if req.want_grad:
            raise ValueError('gradient requests run on Server (FC-fit adjoint)')
        M, C, noise = MODELS[req.model]
        m = M()
        cf = C(m)
        kid, consts, sigma = m.engine_spec()
        cid, _, cf_b, cf_p = cf.engine_spec()
        conn = req.conn
        I, N = req.couplings.size, conn.nnode
        keep = dict(
            row=np.ascontiguousarray(conn.row, np.int32),
            col=np.ascontiguousarray(conn.col, np.int32),
            w=np.ascontiguousarray(conn.wnz, np.float32),
            ln=np.ascontiguousarray(conn.lnz, np.float32),
            G=np.ascontiguousarray(req.couplings, np.float32),
            sp=np.ascontiguousarray(np.broadcast_to(np.asarray(req.speeds, np.float32), (I, ))),
            x0=np.ascontiguousarray(np.broadcast_to(np.asarray(req.x0, np.float32),
                                                    (I, N, m.nsvar))),
        )
        npar = len(m.param_sym)
        npm = (np.broadcast_to(m.node_params(N), (I, N, npar)) if req.nparam is None
               else np.broadcast_to(np.asarray(req.nparam, np.float32).reshape(I, N, -1), (I, N, npar)))
        keep['np'] = np.ascontiguousarray(npm, np.float32)
        q = nat.tvbg_serve_request()
        q.model, q.cfun, q.N, q.nnz = kid, cid, N, conn.nnz
        q.row, q.col = keep['row'].ctypes.data, keep['col'].ctypes.data
        q.weights, q.lengths = keep['w'].ctypes.data, keep['ln'].ctypes.data
        q.n_inst, q.npar = I, npar
        q.couplings, q.speeds = keep['G'].ctypes.data, keep['sp'].ctypes.data
        q.state0, q.nparam = keep['x0'].ctypes.data, keep['np'].ctypes.data
        q.nsteps, q.dt, q.rounding = int(req.nsteps), float(req.dt), 1
        q.seed = int(req.seed) & ((1 << 64) - 1)
        q.flags = nat.F_NOISE if (noise and np.any(np.asarray(sigma) != 0)) else 0
        q.cf_b = float(cf_b) if isinstance(cf_b, (int, float, np.number)) else 0.0
        q.cf_p[:] = [float(v) for v in np.asarray(cf_p, np.float32)]
        q.sigma[:] = [float(v) for v in np.asarray(sigma, np.float32)[:4]]
        q.consts[:] = [float(v) for v in np.asarray(consts, np.float32)]
        nid = ctypes.c_int64()
        nat.check(self.lib.tvbg_serve_admit(self.h, ctypes.byref(q), ctypes.byref(nid)))
        self.reqs[req.rid] = (req, nid.value, m.nsvar)
        self.by_nid[nid.value] = req.rid
        return nid.value

    def tick(self):
        """One pool tick (admit, start idle requests' chunks, take finished
        chunks as they end); the requests retired in it are fetched by id.
        Returns (active, queued)."""
        import ctypes
        a, q = ctypes.c_int32(), ctypes.c_int32()
        self.nat.check(self.lib.tvbg_serve_tick(self.h, ctypes.byref(a), ctypes.byref(q)))
        self.ticks += 1
        now = self.clock()
        n = ctypes.c_int32()
        while True:
            self.nat.check(self.lib.tvbg_serve_finished(self.h, self._fin.ctypes.data,
                                                        self._fin.size, ctypes.byref(n)))
            for nid in self._fin[:n.value].tolist():
                req, _, ns = self.reqs[self.by_nid[nid]]
                req.finished = now
                out = np.zeros((req.couplings.size, req.conn.nnode, ns), np.float32)
                st = ctypes.c_int32()
                self.nat.check(self.lib.tvbg_serve_poll(self.h, nid, ctypes.byref(st), out.ctypes.data))
                req.state = out
                self.done.append(req)
            if n.value < self._fin.size:
                break
        return a.value, q.value

    def poll(self, rid):
        "'queued', 'active', 'done', 'cancelled', or None for an unknown request."
        import ctypes
        if rid not in self.reqs:
            return None
        st = ctypes.c_int32()
        self.nat.check(self.lib.tvbg_serve_poll(self.h, self.reqs[rid][1], ctypes.byref(st), None))
        return {0: 'queued', 1: 'active', 2: 'done', 3: 'cancelled'}[st.value]

    def cancel(self, rid):
        "Drop a queued or active request; False if it is unknown, done or cancelled."
        if self.poll(rid) not in ('queued', 'active'):
            return False
        self.nat.check(self.lib.tvbg_serve_cancel(self.h, self.reqs[rid][1]))
        return True

    def footprint(self, rid):
        "Device bytes request rid takes once admitted."
        import ctypes
        u, f = ctypes.c_int64(), ctypes.c_int64()
        self.nat.check(self.lib.tvbg_serve_usage(self.h, self.reqs[rid][1], ctypes.byref(u),
                                                 ctypes.byref(f)))
        return f.value

    def steps_done(self, rid):
        "Steps request rid has taken so far."
        import ctypes
        d = ctypes.c_int64()
        self.nat.check(self.lib.tvbg_serve_progress(self.h, self.reqs[rid][1], ctypes.byref(d)))
        return int(d.value)

    def steps_issued(self, rid):
        "Steps of request rid handed to the device: taken plus the chunk running now."
        import ctypes
        d = ctypes.c_int64()
        self.nat.check(self.lib.tvbg_serve_issued(self.h, self.reqs[rid][1], ctypes.byref(d)))
        return int(d.value)

    def set_budget(self, nbytes):
        "Admission budget of the following ticks (at most the creation budget)."
        self.nat.check(self.lib.tvbg_serve_set_budget(self.h, int(nbytes)))

    def used(self):
        "Device bytes held by admitted requests."
        import ctypes
        u, f = ctypes.c_int64(), ctypes.c_int64()
        self.nat.check(self.lib.tvbg_serve_usage(self.h, 0, ctypes.byref(u), ctypes.byref(f)))
        return u.value

    def run(self):
        "Tick until nothing is queued or active; returns the finished requests."
        while True:
            a, q = self.tick()
            if a == 0 and q == 0:
                return self.done


def random_requests(n, rate, rng, conns, models=('Kuramoto', 'G2DO', 'MPR'), inst=(1, 4096),
                    steps=(1000, 100000), grad_frac=0.1, dt=0.1, t0=0.0):
    """Poisson arrivals at `rate` per second; model uniform, connectome
    uniform over `conns`, instance count and step count log-uniform."""
    out = []
    t = t0
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        name = models[rng.integers(len(models))]
        conn = conns[rng.integers(len(conns))]
        I = int(np.exp(rng.uniform(np.log(inst[0]), np.log(inst[1] + 1))))
        I = max(1, min(I, inst[1]))
        T = int(np.exp(rng.uniform(np.log(steps[0]), np.log(steps[1]))))
        N = conn.nnode
        want_grad = name == 'MPR' and rng.random() < grad_frac
        if name == 'Kuramoto':
            x0 = rng.uniform(0, 2 * np.pi, (I, N, 1))
            nparam = rng.normal(2 * np.pi * 0.01, 0.001, (I, N, 1))
            G = np.logspace(-2, 1, I)
        elif name == 'G2DO':
            x0 = rng.uniform(-0.5, 0.5, (I, N, 2))
            nparam = None
            G = np.logspace(-3, 0, I)
        else:
            x0 = np.stack([rng.uniform(0.05, 0.3, (I, N)), rng.uniform(-1.5, -0.5, (I, N))], -1)
            nparam = rng.uniform(-6, -4, (I, N, 1))
            G = np.logspace(-2, -0.5, I)
        target = np.corrcoef(rng.normal(size=(N, 40))) if want_grad else None
        out.append(Request(rid=k, model=name, conn=conn, couplings=G.astype(np.float32),
                           speeds=np.full(I, 4.0, np.float32), x0=x0.astype(np.float32),
                           nsteps=T, nparam=None if nparam is None else nparam.astype(np.float32),
                           seed=1000 + k, dt=dt, want_grad=want_grad, target=target, arrival=t))
    return out
