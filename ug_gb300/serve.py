"""Serving loop: continuous batching of 3D diffusion solves on resident pools.

A request is (arrival time, refinement count L, seed): the unit cube's Kuhn
tetrahedra refined L times, k = exp(g) from the seed (correlation `corr`,
variance `var`), the seeded uniform right-hand side -- the problem
``Generator(DIFFUSION3D, L, seed, corr, var)`` describes.  The server keeps,
per depth L, pools of slots (gmg_pool_*: one batched hierarchy of the cached
topology each, sized at start-up from the device's free memory), and runs one
event loop:

* arrived requests wait in a queue per depth; whenever a pool of that depth
  is idle between two iterations and has free slots, they are admitted (their
  matrices and right-hand side are assembled on the device in the free slot);
* every pool with active slots launches its next ls iteration (a replayed
  CUDA graph) on its own stream, so pools overlap on the GPU;
* a finished iteration is polled without blocking; slots whose request met
  its stopping test are fetched (solution to the host) and freed at once.

Latency = completion time - arrival time (queueing, assembly and all
iterations included); throughput = completed requests / makespan.
"""
from __future__ import annotations

import ctypes as C
import gc
import time
from dataclasses import dataclass, field

import numpy as np

from . import GmgError, LResult, _err, lib


@dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the stream
    nref: int
    seed: int
    start: float = -1.0
    done: float = -1.0
    iters: int = 0
    converged: bool = False
    x: np.ndarray | None = None


def poisson_stream(count: int, rate: float, levels=(2, 7), seed: int = 5) -> list[Request]:
    """`count` requests with exponential inter-arrival times (mean 1/rate),
    depths uniform in levels[0]..levels[1], per-request seeds."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    L = rng.integers(levels[0], levels[1] + 1, size=count)
    return [Request(i, float(t[i]), int(L[i]), 100000 + 7919 * i + seed) for i in range(count)]


def cube_unknowns(nref: int) -> int:
    return ((1 << nref) + 1) ** 3


def slot_bytes(nref: int) -> int:
    """Device bytes one slot of depth nref needs (matrices in FP64/FP32 block
    CSR and sliced ELLPACK, transfer, vectors), from the cube's pattern: 15
    entries per row (27 neighbours in the Freudenthal stencil minus 12)."""
    total = 0
    for l in range(nref + 1):
        n = cube_unknowns(l)
        nnz = 15 * n
        total += nnz * (4 + 8 + 4) * 2 + n * (8 * 8 + 40)
    return int(total * 1.15)


def pool_bytes(nref: int, nslots: int) -> int:
    """Device bytes of a pool: its slots plus the admission's FP64 field of
    the finest level (one coefficient per tetrahedron)."""
    return nslots * slot_bytes(nref) + 6 * 8 ** nref * 8


class Pool:
    """One gmg_pool: `nslots` slots of depth `nref`, or (depths given) one slot
    per entry of `depths`, each of its own depth: a mixed pool, whose every
    iteration runs the V-cycles of all its requests level by level together.
    mesh: 3 the cubes UG's red rules refine (UG's own hierarchies), 1 the
    Freudenthal triangulation."""

    def __init__(self, nref: int, nslots: int, smoother: str = "gs", red: float = 1e-8, maxit: int = 100,
                 device: int = 0, stream=None, field_fp64: bool = True, depths=None, mesh: int = 3):
        h = C.c_void_p()
        d = np.ascontiguousarray(depths if depths is not None else [nref] * nslots, np.int32)
        if lib().gmg_pool_create_mesh(mesh, d.ctypes.data, len(d), smoother.encode(), red, maxit, device,
                                      C.byref(h)):
            _err("gmg_pool_create_mesh")
        self.depths = [int(x) for x in d]
        self.mesh = mesh
        self._h = h
        if not field_fp64 and lib().gmg_pool_set_field_precision(h, 1):
            _err("gmg_pool_set_field_precision")
        self.nref, self.nslots = max(self.depths), len(self.depths)
        if stream is not None:
            lib().gmg_pool_set_stream(h, stream)
        self.n_top_of = []
        for k in range(self.nslots):
            dk, nt = C.c_int(), C.c_int()
            lib().gmg_pool_slot_info(h, k, C.byref(dk), C.byref(nt))
            self.n_top_of.append(nt.value)
        self.n_top = max(self.n_top_of)
        self.free = list(range(self.nslots))
        self.active: dict[int, object] = {}
        self.busy = False
        self._done = np.zeros(self.nslots, np.int32)

    def free_slot(self, depth: int):
        """A free slot of this depth, or None."""
        for k in self.free:
            if self.depths[k] == depth:
                return k
        return None

    def admit(self, slot: int, seed: int, corr: float, var: float):
        if lib().gmg_pool_admit(self._h, slot, seed, corr, var):
            _err("gmg_pool_admit")

    def launch(self):
        if lib().gmg_pool_launch(self._h):
            _err("gmg_pool_launch")
        self.busy = True

    def poll(self):
        """None while the iteration runs, else the list of finished slots."""
        nd = C.c_int()
        r = lib().gmg_pool_poll(self._h, C.byref(nd), self._done.ctypes.data)
        if r < 0:
            _err("gmg_pool_poll")
        if r == 0:
            return None
        self.busy = False
        return [int(k) for k in self._done[:nd.value]]

    def fetch(self, slot: int, want_x: bool = True):
        lr = LResult()
        x = np.empty(self.n_top_of[slot]) if want_x else None
        if lib().gmg_pool_fetch(self._h, slot, None if x is None else x.ctypes.data, C.byref(lr)):
            _err("gmg_pool_fetch")
        return x, lr

    def slot_matrix(self, slot: int, level: int, nnz: int) -> np.ndarray:
        v = np.empty(nnz)
        if lib().gmg_pool_slot_matrix(self._h, slot, level, v.ctypes.data):
            _err("gmg_pool_slot_matrix")
        return v

    def solve(self, seed: int, corr: float = 0.1, var: float = 1.0, slot: int | None = None, depth=None):
        """One request alone in this pool (blocking): (x, LResult)."""
        if slot is None:
            slot = self.free_slot(self.depths[0] if depth is None else depth)
        self.free.remove(slot)
        self.admit(slot, seed, corr, var)
        while True:
            self.launch()
            while (done := self.poll()) is None:
                pass
            if slot in done:
                x, lr = self.fetch(slot)
                self.free.append(slot)
                return x, lr

    def close(self):
        if getattr(self, "_h", None):
            lib().gmg_pool_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def free_device_memory(device: int = 0) -> int:
    import torch
    return int(torch.cuda.mem_get_info(device)[0])


@dataclass
class ServeStats:
    completed: int
    makespan_s: float
    p50_ms: float
    p99_ms: float
    mean_ms: float
    throughput: float
    iterations_mean: float
    all_converged: bool
    per_depth: dict = field(default_factory=dict)
    breakdown: dict = field(default_factory=dict)


class Server:
    """Pools sized from free device memory, and the event loop.

    layout[L] = (pools, slots per pool) per depth.  Large depths get one-slot
    pools (one instance saturates the GPU's bandwidth and a pool iterates all
    of its slots, busy or not); small depths share few pools of many slots
    (their cycles are latency-bound, so batching them is what pays).  Two or
    more pools per depth let a request start while another pool of its depth
    is mid-iteration.  `mixed` lists groups of depths whose pools are shared:
    a group's pools are mixed pools holding, per depth of the group, that
    depth's slots per pool (the group has the largest pool count of its
    depths), so requests of different mesh sizes run their V-cycles level by
    level in the same iterations."""

    DEFAULT = {1: (2, 8), 2: (2, 8), 3: (2, 8), 4: (2, 8), 5: (2, 4), 6: (3, 1), 7: (4, 1), 8: (2, 1)}

    def __init__(self, depths=range(2, 8), layout=None, hbm_fraction: float = 0.5, smoother: str = "gs",
                 red: float = 1e-8, maxit: int = 100, corr: float = 0.1, var: float = 1.0, device: int = 0,
                 slots=None, field_fp64: bool = False, mixed=(), grow_after_ms: float | None = None,
                 grow_reserve: float = 0.1, mesh: int = 3):
        """field_fp64: admissions evaluate the coefficient field in FP64 (the
        host generator's problem to 1e-12; on GB300 ~12 ms of FP64 work per
        depth-7 admission, more than a 200 req/s stream leaves) instead of
        FP32 (~2 ms, k within ~1e-6).

        grow_after_ms: a depth whose requests have waited this long for a
        free slot gets one more pool of its layout's shape, if the device's
        free memory (queried at that moment) covers it with grow_reserve of
        the device left over; the pool is created and warmed on a helper
        thread while the loop keeps serving, and joins the loop when ready
        (None: the pools are fixed).

        mesh: 3 (default) the cubes refined by UG's red rules, 1 the
        Freudenthal triangulation."""
        import torch
        self.corr, self.var = corr, var
        self.field_fp64 = field_fp64
        self.mesh = mesh
        self.grow_after_ms, self.grow_reserve = grow_after_ms, grow_reserve
        self._args = (smoother, red, maxit, device)
        self.grown = []  # (seconds into the stream, depth) of every pool added while serving
        depths = list(depths)
        if layout is None:
            layout = {L: ((1, slots[L]) if slots else self.DEFAULT.get(L, (2, 1))) for L in depths}
        budget = hbm_fraction * free_device_memory(device)
        need = sum(pool_bytes(L, m) * n for L, (n, m) in layout.items())
        if need > budget:  # shrink the largest depths' pool counts to the budget
            for L in sorted(layout, reverse=True):
                while need > budget and layout[L][0] > 1:
                    need -= pool_bytes(L, layout[L][1])
                    layout[L] = (layout[L][0] - 1, layout[L][1])
        if need > budget:
            raise GmgError(f"pools need {need / 1e9:.1f} GB, {budget / 1e9:.1f} GB available")
        self.layout = dict(layout)
        groups = [tuple(g) for g in mixed if all(L in layout for L in g)]
        grouped = {L for g in groups for L in g}
        self.mixed_depths = grouped
        groups += [(L,) for L in depths if L not in grouped]
        self.groups = groups
        self.pools = {L: [] for L in depths}  # depth -> the pools with slots of that depth
        self.all_pools = []
        self.streams = []
        for g in groups:
            for _ in range(max(layout[L][0] for L in g)):
                st = torch.cuda.Stream(device=device)
                self.streams.append(st)
                if len(g) == 1:
                    pool = Pool(g[0], layout[g[0]][1], smoother, red, maxit, device, st.cuda_stream, field_fp64,
                                mesh=mesh)
                else:
                    dep = [L for L in g for _ in range(layout[L][1])]
                    pool = Pool(0, 0, smoother, red, maxit, device, st.cuda_stream, field_fp64, depths=dep,
                                mesh=mesh)
                self.all_pools.append(pool)
                for L in g:
                    self.pools[L].append(pool)
        self.slots = {L: sum(p.depths.count(L) for p in self.pools[L]) for L in depths}

    def warm(self, seed: int = 1):
        """One request of each of its depths through every pool: the first
        iteration allocates the solver's temporaries and the second captures
        the iteration's CUDA graph -- work that must not stall the event loop
        later."""
        for p in self.all_pools:
            for d in sorted(set(p.depths)):
                p.solve(seed, self.corr, self.var, depth=d)

    def _grow(self, L: int, ready: list):
        """Create and warm one more pool of depth L (helper thread); the
        event loop adds it from `ready`."""
        import torch
        smoother, red, maxit, device = self._args
        torch.cuda.set_device(device)
        st = torch.cuda.Stream(device=device)
        pool = Pool(L, self.layout[L][1], smoother, red, maxit, device, st.cuda_stream, self.field_fp64,
                    mesh=self.mesh)
        pool.solve(1, self.corr, self.var)
        torch.cuda.current_stream(device).synchronize()
        ready.append((L, pool, st))

    def _may_grow(self, L: int) -> bool:
        import torch
        smoother, red, maxit, device = self._args
        free, total = torch.cuda.mem_get_info(device)
        return free - pool_bytes(L, self.layout[L][1]) >= self.grow_reserve * total

    def run(self, requests: list[Request], keep_x: bool = False) -> ServeStats:
        """Serve the stream; latency breakdown per request: queue wait
        (admission - arrival) and service (completion - admission); the
        loop's host calls are timed too (the longest ones are reported), so
        a latency tail can be traced to queueing, a slow host call or the
        device.  Python's cyclic garbage collector is paused during the
        loop (a full collection over the process's objects is a pause of
        tens to hundreds of ms that would land on every request in flight)."""
        pending = {L: [] for L in self.pools}
        order = sorted(requests, key=lambda r: r.arrival)
        nxt = 0
        done_count = 0
        host_ops = []  # (seconds, kind, depth) of every admit / launch / poll / fetch
        gaps = []      # wall time of each pass of the loop
        gc_was = gc.isenabled()
        gc.collect()
        gc.disable()
        pc = time.perf_counter
        t0 = pc()
        tprev = t0
        ready, growing, waiting_since = [], set(), {}
        import threading
        while done_count < len(order):
            tl = pc()
            gaps.append(tl - tprev)
            tprev = tl
            now = tl - t0
            while ready:  # pools a helper thread finished
                L, pool, st = ready.pop()
                self.streams.append(st)
                self.all_pools.append(pool)
                self.pools[L].append(pool)
                self.slots[L] += pool.nslots
                growing.discard(L)
                self.grown.append((now, L))
            while nxt < len(order) and order[nxt].arrival <= now:
                pending[order[nxt].nref].append(order[nxt])
                nxt += 1
            progressed = False
            for pool in self.all_pools:
                if pool.busy:
                    ta = pc()
                    fin = pool.poll()
                    host_ops.append((pc() - ta, "poll", pool.nref))
                    if fin is None:
                        continue
                    progressed = True
                    tnow = pc() - t0
                    for k in fin:
                        req = pool.active.pop(k)
                        ta = pc()
                        x, lr = pool.fetch(k, keep_x)
                        host_ops.append((pc() - ta, "fetch", pool.depths[k]))
                        req.done, req.iters, req.converged = tnow, lr.iters, bool(lr.converged)
                        req.x = x
                        pool.free.append(k)
                        done_count += 1
            # admissions between two iterations (pools already iterating
            # first, so requests batch), then the next iterations
            for L, q in pending.items():
                if not q:
                    continue
                for pool in sorted(self.pools[L], key=lambda p: -len(p.active)):
                    while q and not pool.busy:
                        k = pool.free_slot(L)
                        if k is None:
                            break
                        req = q.pop(0)
                        pool.free.remove(k)
                        ta = pc()
                        req.start = ta - t0
                        pool.admit(k, req.seed, self.corr, self.var)
                        host_ops.append((pc() - ta, "admit", L))
                        pool.active[k] = req
                        progressed = True
            for pool in self.all_pools:
                if pool.active and not pool.busy:
                    ta = pc()
                    pool.launch()
                    host_ops.append((pc() - ta, "launch", pool.nref))
            if self.grow_after_ms is not None:  # demand-driven growth by free device memory
                for L, q in pending.items():
                    if not q:
                        waiting_since.pop(L, None)
                        continue
                    w0 = waiting_since.setdefault(L, now)
                    if L not in growing and L not in self.mixed_depths and (now - w0) * 1e3 >= self.grow_after_ms \
                            and self._may_grow(L):
                        growing.add(L)
                        threading.Thread(target=self._grow, args=(L, ready), daemon=True).start()
            if not progressed:
                if nxt < len(order) and not any(p.busy for p in self.all_pools):
                    wait = order[nxt].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.002))
        if gc_was:
            gc.enable()
        makespan = max(r.done for r in order)
        lat = np.array([(r.done - r.arrival) * 1e3 for r in order])
        wait = np.array([(r.start - r.arrival) * 1e3 for r in order])
        serv = np.array([(r.done - r.start) * 1e3 for r in order])
        host_ops.sort(key=lambda o: -o[0])
        by_kind = {}
        for dt, kind, L in host_ops:
            e = by_kind.setdefault(kind, [0, 0.0, 0.0])
            e[0] += 1; e[1] += dt; e[2] = max(e[2], dt)
        breakdown = {
            "queue_wait_ms": {"p50": float(np.percentile(wait, 50)), "p99": float(np.percentile(wait, 99)),
                              "max": float(wait.max())},
            "service_ms": {"p50": float(np.percentile(serv, 50)), "p99": float(np.percentile(serv, 99)),
                           "max": float(serv.max())},
            "host_calls": {k: {"count": c, "total_ms": t * 1e3, "max_ms": m * 1e3} for k, (c, t, m) in by_kind.items()},
            "longest_host_calls_ms": [[round(dt * 1e3, 3), kind, L] for dt, kind, L in host_ops[:5]],
            "longest_loop_pass_ms": float(max(gaps) * 1e3) if gaps else 0.0,
        }
        per = {}
        for L in self.pools:
            ls = np.array([(r.done - r.arrival) * 1e3 for r in order if r.nref == L])
            if ls.size:
                per[L] = {"count": int(ls.size), "p50_ms": float(np.percentile(ls, 50)),
                          "p99_ms": float(np.percentile(ls, 99)), "pools": len(self.pools[L]),
                          "slots": self.slots[L]}
        return ServeStats(len(order), makespan, float(np.percentile(lat, 50)), float(np.percentile(lat, 99)),
                          float(lat.mean()), len(order) / makespan, float(np.mean([r.iters for r in order])),
                          all(r.converged for r in order), per, breakdown)

    def close(self):
        for p in self.all_pools:
            p.close()
