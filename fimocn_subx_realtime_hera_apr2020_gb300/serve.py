"""Forecast-advance serving with continuous batching.

A request asks to advance a state on grid level glvl with nvl layers and
ntra tracers by `steps` dynamics steps: its own host state, or a seeded
balanced state that the library's kernels make on the device in the slot it
is admitted to (milliseconds, where the numpy generator takes seconds at
glvl 7).  Requests on the same
grid (glvl, nvl) share a pool: one context whose ensemble slots are the
batch, advanced together by one fused launch sequence per step
(fim_step_active, one CUDA-graph replay).  A pool carries `max_tracers`
tracer slots; a request with fewer tracers leaves the rest at zero.  Tracers
are advected independently of one another, so a request's own tracers evolve
exactly as in a context of its own size.  Every slot carries its own step
counter and AB3 slots, so a request admitted while others are mid-forecast
joins at the next step boundary; a finished slot is freed for the next
request.  Pools are created while free HBM allows (admission by memory; a
pool takes fewer slots when memory is short) and each pool runs on its own
stream, so different grids overlap on the device.  States stay resident in
HBM for the whole forecast.
"""
import heapq
import time
from dataclasses import dataclass, field

import numpy as np

from .config import FimConfig, default_dt
from .dycore import Dycore
from .grid import Grid
from .state import synthetic_state_device


@dataclass(order=True)
class Request:
    arrival: float
    rid: int = field(compare=False)
    glvl: int = field(compare=False)
    nvl: int = field(compare=False)
    ntra: int = field(compare=False)
    steps: int = field(compare=False)
    seed: int = field(compare=False, default=0)
    # the request's own initial state (host arrays in the reference layout,
    # as State.load takes them); None: the seeded balanced state made on
    # the device
    fields: dict = field(compare=False, default=None, repr=False)
    t_queue: float = field(compare=False, default=None)
    t_admit: float = field(compare=False, default=None)
    t_done: float = field(compare=False, default=None)
    result: dict = field(compare=False, default=None)

    @property
    def key(self):
        return (self.glvl, self.nvl)

    @property
    def work(self):
        """cell-level-steps of the request"""
        return (10 * 4 ** self.glvl + 2) * self.nvl * self.steps


# tracers a launch of a pool's fused tracer kernels takes (0: the library's
# choice, all of them while their scratch stays under ~48 GB).  Short chunks
# would leave room for more slots, but each launch stages a patch's tables,
# coefficients and mass fluxes once for its tracers: pools with 3-tracer
# chunks served the default stream at 8.5e8 cell-level-steps/s against
# 1.0e9 with whole chunks.
POOL_TRACER_CHUNK = 0


def state_bytes(glvl, nvl, ntra, precision, tracer_chunk=POOL_TRACER_CHUNK):
    """Device bytes of one member slot of a pool context: the state's fields,
    the step's edge fields and the kernels' scratch, as the library allocates
    them (fused tracer transport, no class-B tracers), plus 5%; with the
    library's tracer chunks the scratch is counted for every tracer."""
    nip = 10 * 4 ** glvl + 2
    w = 8 if precision == "f64" else 4
    T = ntra
    tch = min(ntra, tracer_chunk) if tracer_chunk > 0 else ntra
    intf = (nvl + 1) / nvl
    words = (3 + 3 * intf + 1          # us vs dp, pr ex ph, mp
             + 2 * T + 12 + 6 * T       # tr trdp, u v dp dpl AB3, trc trl AB3
             + 18 + 1 + intf + 1        # massfx, ws sdot relvor
             + 7 * 6 + 6                # edge fields, theta's trc_edg
             + 12 * tch                 # fused tracer scratch
             + 11 + 2 + 2 * intf)       # cnuity, momtum, hybgen scratch
    if precision != "f64":
        words += 3                      # float-float Montgomery potential, theta of the edge values
    return int(nip * nvl * words * w * 1.05)


class Pool:
    """One batched context (all slots share the grid and the configuration)."""

    def __init__(self, key, precision, slots, collect, ntra, priority=0):
        import torch
        glvl, nvl = key
        self.key = key
        self.ntra = ntra
        self.grid = Grid.cached(glvl)
        self.cfg = FimConfig(nvl=nvl, ntra=ntra, dt=default_dt(glvl), precision=precision, members=slots,
                             stream_priority=priority, tracer_chunk=POOL_TRACER_CHUNK)
        self.dyc = Dycore(self.grid, self.cfg)
        self.st = self.dyc.state()
        for m in range(slots):
            self.st.set_active(m, False)
        self.slots = [None] * slots
        self.collect = collect
        self.stream = torch.cuda.ExternalStream(self.dyc.stream)

    def free_slot(self):
        for i, r in enumerate(self.slots):
            if r is None:
                return i
        return -1

    def admit(self, req, now):
        m = self.free_slot()
        if req.fields is None:
            own = FimConfig(nvl=self.cfg.nvl, ntra=req.ntra, dt=self.cfg.dt, precision=self.cfg.precision)
            # on the pool's stream, ahead of the slot's initialisation
            synthetic_state_device(self.st, m, self.grid, own, req.seed, sigma_ps=200.0, noise=0.5)
        else:
            fields = dict(req.fields)
            src = np.asarray(fields["tr3d"]).reshape(-1)
            tr = np.zeros(self.ntra * self.grid.nip * self.cfg.nvl, src.dtype)
            tr[:src.size] = src
            fields["tr3d"] = tr
            self.st.load(fields, member=m)
        # the slot's padded tracers (zero) are left out of every step's work
        self.st.set_tracers(m, req.ntra)
        self.st.init_member(m)  # dyn_init for this slot only; activates it
        req.t_admit = now
        self.slots[m] = req

    def active(self):
        return any(r is not None for r in self.slots)

    def idle(self):
        """Nothing of the pool's is still running on the device."""
        return self.stream.query()

    def step(self):
        self.st.step_active(use_graph=True)

    def finished(self):
        done = []
        for m, r in enumerate(self.slots):
            if r is not None and self.st.member_its(m) >= r.steps:
                done.append(m)
        return done

    def retire(self, m, now):
        r = self.slots[m]
        res = {}
        own = r.ntra * self.grid.nip * self.cfg.nvl
        if self.collect:
            for name in self.collect:
                a = self.st.download(name, m)
                res[name] = a[:own] if name in ("tr3d", "trdp") else a
        qtrcr, bud = self.st.budget(m)
        res["qmass"] = bud["qmass"]
        res["qtrcr"] = qtrcr[:r.ntra]
        r.result = res
        r.t_done = now
        self.st.set_active(m, False)
        self.slots[m] = None
        return r

    def close(self):
        self.st.free()
        self.dyc.close()


class Server:
    """Continuous-batching request loop over resident device states."""

    def __init__(self, precision="f32", slots=8, hbm_fraction=0.9, collect=("us3d", "tr3d"), max_tracers=21,
                 priorities=True, grids=()):
        # grid levels whose tables are built at start-up rather than by the
        # first request on them (glvl 7: ~0.4 s of host work)
        for glvl in grids:
            Grid.cached(glvl)
        self.precision = precision
        self.slots = slots
        # pools on smaller grids get higher stream priorities: their short
        # steps' blocks go first when blocks of a larger grid's step finish
        self.priorities = priorities
        self.max_tracers = max_tracers
        self.hbm_fraction = hbm_fraction
        self.collect = collect
        self.pools = {}

    def _free_hbm(self):
        import torch
        free, total = torch.cuda.mem_get_info()
        return free - (1 - self.hbm_fraction) * total

    def _pool_for(self, req):
        p = self.pools.get(req.key)
        if p is not None:
            return p
        if req.ntra > self.max_tracers:
            raise ValueError("request %d has %d tracers, the server at most %d" % (req.rid, req.ntra,
                                                                                 self.max_tracers))
        per_slot = state_bytes(req.glvl, req.nvl, self.max_tracers, self.precision)
        if per_slot > self._free_hbm():
            # evict idle pools first, then refuse for now (the request waits)
            for k in [k for k, v in self.pools.items() if not v.active()]:
                self.pools.pop(k).close()
        slots = self.slots
        while slots > 1 and per_slot * slots > self._free_hbm():
            slots //= 2
        if per_slot * slots > self._free_hbm():
            return None
        prio = -max(0, 8 - req.glvl) if self.priorities else 0
        p = Pool(req.key, self.precision, slots, self.collect, self.max_tracers, priority=prio)
        self.pools[req.key] = p
        return p

    def run(self, requests, realtime=True):
        """Serve `requests` (arrival in seconds from start); returns them done."""
        import torch
        pending = list(requests)
        heapq.heapify(pending)
        waiting = []
        done = []
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        while pending or waiting or any(p.active() for p in self.pools.values()):
            t = now()
            while pending and (pending[0].arrival <= t or not realtime):
                r = heapq.heappop(pending)
                # latency counts from arrival, or from entry into the queue
                # when arrivals are not replayed in real time
                r.t_queue = r.arrival if realtime else t
                waiting.append(r)
                if not realtime:
                    break
            # each pool goes at its own pace: a pool whose last step is done
            # retires its finished requests, takes waiting ones into its free
            # slots and enqueues its next step on its own stream, while the
            # steps of other pools are still running
            idle = {k: p.idle() for k, p in self.pools.items()}
            for k, p in self.pools.items():
                if idle[k]:
                    for m in p.finished():
                        done.append(p.retire(m, now()))
            still = []
            for r in waiting:
                p = self._pool_for(r)
                if p is not None and p.free_slot() >= 0 and idle.get(r.key, True):
                    p.admit(r, now())
                else:
                    still.append(r)
            waiting = still
            launched = False
            for k, p in self.pools.items():
                if idle.get(k, True) and p.active():
                    p.step()
                    launched = True
            if not launched:
                if not any(p.active() for p in self.pools.values()) and pending and realtime:
                    time.sleep(max(0.0, min(pending[0].arrival - now(), 0.01)))
                else:
                    time.sleep(2e-4)  # every active pool's step is still running
        torch.cuda.synchronize()
        return done

    def close(self):
        for p in self.pools.values():
            p.close()
        self.pools = {}


def poisson_requests(n, rate, seed, glvls=(5, 6, 7), nvls=(38, 64), tracers=(4, 20), steps=(24, 240)):
    """Seeded Poisson arrival stream of the served workload mix."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        out.append(Request(arrival=t, rid=i, glvl=int(rng.choice(glvls)), nvl=int(rng.choice(nvls)),
                           ntra=int(rng.integers(tracers[0], tracers[1] + 1)) + 1,
                           steps=int(rng.integers(steps[0], steps[1] + 1)), seed=5000 + i))
    return out


def latency_stats(done):
    lat = np.array([r.t_done - r.t_queue for r in done])
    work = sum(r.work for r in done)
    span = max(r.t_done for r in done) - min(r.t_queue for r in done)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "requests": len(done), "cell_level_steps_per_s": work / span}
