"""A request loop over resident models: continuous batching of range-analysis queries.

The reference has no serving path; this module turns the query kernels into a service.
Models stay resident on the device (one packed blob each).  Requests of three kinds
arrive from any thread:

* ``RayRequest``: cast a tile of rays against one model (queries.cast_rays),
* ``ClosestRequest``: closest points of a query batch on one model
  (kd_tree.closest_point, persistent per-query traversal),
* ``IntersectRequest``: does model A, moved by a rigid transform, meet model B
  (kd_tree.find_any_intersection)?

A scheduler thread admits queued requests while their estimated device memory fits the
budget, groups the closest-point requests of an admission wave into multi-model
launches (batched.closest_point_packed) of at most ``closest_group_points`` points,
smallest first, and issues each launch on one of a pool of CUDA streams, so work
admitted later overlaps work already on the device.  A
completion thread polls the streams' events, copies results to the host and resolves
the request futures; latency is measured from submission to resolution.
"""
from __future__ import annotations

import collections
import dataclasses
import queue
import threading
import time
from concurrent.futures import Future, ThreadPoolExecutor

import numpy as np

from . import _io, _lib, batched, kd_tree, queries
from .implicit_mlp_utils import generate_implicit_from_params
from .mlp import device_model, prepend_op, spatial_transformation


@dataclasses.dataclass
class RayRequest:
    model: int
    roots: np.ndarray
    dirs: np.ndarray
    opts: dict = None


@dataclasses.dataclass
class ClosestRequest:
    model: int
    points: np.ndarray
    eps: float = 1e-3
    node_budget: int = 1 << 16   # nodes per query; past it the result is an upper bound


@dataclasses.dataclass
class IntersectRequest:
    model_a: int
    model_b: int
    R: np.ndarray
    t: np.ndarray
    eps: float = 1e-3


@dataclasses.dataclass
class _Pending:
    req: object
    future: Future
    t_submit: float
    bytes: int


def estimate_bytes(req):
    """Device memory a request holds while in flight (inputs, outputs, workspace)."""
    if isinstance(req, RayRequest):
        n = len(req.roots)
        return 24 * n + 12 * n + 28 * n + 4096
    if isinstance(req, ClosestRequest):
        return 12 * len(req.points) + 16 * len(req.points) + 4096
    return (1 << 20) * 12 * 8   # intersection: node arrays for 1M nodes per level, 4 levels buffers


class Server:
    def __init__(self, params_list, mode='affine_fixed', budget_bytes=40 << 30, n_streams=4, lower=(-1., -1., -1.),
                 upper=(1., 1., 1.), conservative=True):
        import torch
        self.torch = torch
        self.params = list(params_list)
        self.func, _ = generate_implicit_from_params(self.params[0], mode, conservative=conservative)
        self.table = batched.ModelTable(self.params)
        self.lower = np.asarray(lower, np.float32)
        self.upper = np.asarray(upper, np.float32)
        self.budget = int(budget_bytes)
        self.intersect_max_nodes = 1 << 20   # per search level; larger searches fail fast
        self.closest_group_points = 4096     # closest-point points per multi-model launch
        # ray tiles and closest-point launches on separate stream pools, so a light ray
        # tile never queues behind a heavy closest-point launch on the same stream
        self.streams = {'rays': [torch.cuda.Stream() for _ in range(max(1, n_streams // 2))],
                        'closest': [torch.cuda.Stream() for _ in range(max(1, n_streams - n_streams // 2))]}
        self._rr_kind = {'rays': 0, 'closest': 0}

        # intersections synchronise per search level: they run on their own workers/streams
        self._isect_pool = ThreadPoolExecutor(max_workers=2)
        self._isect_streams = [torch.cuda.Stream() for _ in range(2)]
        self._isect_rr = 0
        self._rr = 0
        self._q = queue.Queue()
        self._inflight = collections.deque()
        self._inflight_bytes = 0
        self._lock = threading.Condition()
        self._stop = False
        self.latencies = []
        self.kind_latencies = collections.defaultdict(list)
        self.completed = 0
        self.budget_exhausted = 0   # closest-point launches in which a query spent its node budget
        self._sched = threading.Thread(target=self._schedule, daemon=True)
        self._done = threading.Thread(target=self._complete, daemon=True)
        self._device = torch.cuda.current_device()
        self._sched.start()
        self._done.start()

    # ------------------------------------------------------------------ client side
    def submit(self, req):
        fut = Future()
        self._q.put(_Pending(req, fut, time.perf_counter(), estimate_bytes(req)))
        return fut

    def close(self):
        with self._lock:
            self._stop = True
            self._lock.notify_all()
        self._q.put(None)
        self._sched.join()
        self._done.join()
        self._isect_pool.shutdown(wait=True)

    def stats(self):
        lat = np.array(self.latencies) * 1e3
        if lat.size == 0:
            return {"completed": 0}
        per_kind = {k: {"n": len(v), "p50_ms": float(np.percentile(np.array(v) * 1e3, 50)),
                        "p99_ms": float(np.percentile(np.array(v) * 1e3, 99))}
                    for k, v in self.kind_latencies.items() if v}
        return {"completed": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "closest_budget_exhausted": self.budget_exhausted, "by_kind": per_kind}

    # ------------------------------------------------------------------ scheduler
    def _next_stream(self, kind):
        pool = self.streams[kind]
        s = pool[self._rr_kind[kind] % len(pool)]
        self._rr_kind[kind] += 1
        return s

    def _schedule(self):
        torch = self.torch
        torch.cuda.set_device(self._device)
        waiting = collections.deque()
        while True:
            # drain the queue without blocking when work is waiting for admission
            try:
                item = self._q.get(timeout=0.0005 if waiting else None)
                if item is None:
                    if not waiting:
                        break
                else:
                    waiting.append(item)
                    while True:
                        try:
                            nxt = self._q.get_nowait()
                        except queue.Empty:
                            break
                        if nxt is None:
                            self._q.put(None)
                            break
                        waiting.append(nxt)
            except queue.Empty:
                pass
            # admission wave: everything that fits the budget right now
            wave = []
            with self._lock:
                while waiting and self._inflight_bytes + waiting[0].bytes <= self.budget:
                    p = waiting.popleft()
                    self._inflight_bytes += p.bytes
                    wave.append(p)
                if not wave and waiting and self._inflight_bytes == 0:
                    p = waiting.popleft()   # larger than the whole budget: run it alone
                    self._inflight_bytes += p.bytes
                    wave.append(p)
            if wave:
                self._launch(wave)
            elif waiting:
                with self._lock:
                    self._lock.wait(timeout=0.001)
            if self._stop and not waiting and self._q.empty():
                break
        with self._lock:
            self._inflight.append(None)
            self._lock.notify_all()

    def _launch(self, wave):
        torch = self.torch
        cps = [p for p in wave if isinstance(p.req, ClosestRequest)]
        rays = [p for p in wave if isinstance(p.req, RayRequest)]
        isects = [p for p in wave if isinstance(p.req, IntersectRequest)]
        # ray tiles first: they are light and their streams are their own
        for p in rays:
            s = self._next_stream('rays')
            with torch.cuda.stream(s):
                opts = p.req.opts or queries.get_default_cast_opts()
                out = queries.cast_rays((self.func,), (self.table.models[p.req.model],),
                                        np.asarray(p.req.roots, np.float32), np.asarray(p.req.dirs, np.float32),
                                        opts, return_device=True)
                ev = torch.cuda.Event()
                ev.record(s)
            self._push(('rays', [p], out[:3], ev))
        groups = collections.defaultdict(list)
        for p in cps:
            groups[(float(p.req.eps), int(p.req.node_budget))].append(p)
        # split each (eps, budget) group into launches of at most `closest_group_points`
        # points, smallest requests first, so a small request never waits for the
        # slowest query of a large one
        launches = []
        for key, grp in groups.items():
            grp = sorted(grp, key=lambda p: len(p.req.points))
            cur, n = [], 0
            for p in grp:
                k = len(p.req.points)
                if cur and n + k > self.closest_group_points:
                    launches.append((key, cur))
                    cur, n = [], 0
                cur.append(p)
                n += k
            if cur:
                launches.append((key, cur))
        for (eps, budget), grp in launches:
            # the wave's closest-point requests with one (eps, budget): one multi-model launch
            s = self._next_stream('closest')
            with torch.cuda.stream(s):
                counts = np.array([len(p.req.points) for p in grp], np.int64)
                offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
                pts = np.concatenate([np.asarray(p.req.points, np.float32).reshape(-1, 3) for p in grp])
                status = torch.zeros(1, dtype=torch.int32, device='cuda')
                dist, loc = batched.closest_point_packed(self.func, self.table, [p.req.model for p in grp], offs,
                                                         counts, pts, self.lower, self.upper, eps,
                                                         status=status, node_budget=budget)
                ev = torch.cuda.Event()
                ev.record(s)
            self._push(('closest', grp, (dist, loc, offs, counts, status), ev))
        for p in isects:
            s = self._isect_streams[self._isect_rr % len(self._isect_streams)]
            self._isect_rr += 1
            self._isect_pool.submit(self._run_intersection, p, s)

    def _run_intersection(self, p, s):
        torch = self.torch
        torch.cuda.set_device(self._device)
        out, exc = None, None
        try:
            with torch.cuda.stream(s):
                pa = prepend_op(self.params[p.req.model_a], spatial_transformation())
                pa['0000.spatial_transformation.R'] = np.asarray(p.req.R, np.float32)
                pa['0000.spatial_transformation.t'] = np.asarray(p.req.t, np.float32)
                pb = prepend_op(self.params[p.req.model_b], spatial_transformation())
                out = kd_tree.find_any_intersection((self.func, self.func), (pa, pb), self.lower, self.upper,
                                                    p.req.eps, max_nodes=self.intersect_max_nodes)
        except Exception as e:   # capacity or budget exhausted: the request fails, the server goes on
            exc = e
        now = time.perf_counter()
        with self._lock:
            self._inflight_bytes -= p.bytes
            self.latencies.append(now - p.t_submit)
            self.kind_latencies['intersect'].append(now - p.t_submit)
            self.completed += 1
            self._lock.notify_all()
        if exc is not None:
            p.future.set_exception(exc)
        else:
            p.future.set_result(out)

    def _push(self, rec):
        with self._lock:
            self._inflight.append(rec)
            self._lock.notify_all()

    # ------------------------------------------------------------------ completion
    def _complete(self):
        torch = self.torch
        torch.cuda.set_device(self._device)
        while True:
            with self._lock:
                while not self._inflight:
                    self._lock.wait()
                rec = self._inflight[0]
                if rec is None:
                    return
            kind, pend, out, ev = rec
            if not ev.query():
                time.sleep(0.0002)
                # look for any finished record, not just the oldest
                with self._lock:
                    ready = None
                    for r in self._inflight:
                        if r is not None and r[3].query():
                            ready = r
                            break
                    if ready is None:
                        continue
                    self._inflight.remove(ready)
                    rec = ready
            else:
                with self._lock:
                    self._inflight.popleft()
            self._finish(rec)

    def _finish(self, rec):
        kind, pend, out, ev = rec
        ev.synchronize()
        now = time.perf_counter()
        if kind == 'closest':
            dist, loc, offs, counts, status = out
            code = int(status.item())
            if code == _lib.NIQ_ERR_TIMEOUT:
                # some query spent its node budget: its distance is an upper bound; the
                # results are still delivered and the event is counted
                with self._lock:
                    self.budget_exhausted += 1
            elif code != 0:
                if code == _lib.NIQ_ERR_CAPACITY:
                    err = _lib.NIQCapacityError(code, "closest-point stack depth exceeded")
                else:
                    err = _lib.NIQError(code, "closest-point traversal failed")
                with self._lock:
                    for p in pend:
                        self._inflight_bytes -= p.bytes
                for p in pend:
                    p.future.set_exception(err)
                return
            d, l_ = dist.cpu().numpy(), loc.cpu().numpy()
            results = [(d[o:o + c], l_[o:o + c]) for o, c in zip(offs, counts)]
        else:
            results = [tuple(x.cpu().numpy() for x in out)]
        now = time.perf_counter()
        with self._lock:
            for p, r in zip(pend, results):
                self._inflight_bytes -= p.bytes
                self.latencies.append(now - p.t_submit)
                self.kind_latencies[kind].append(now - p.t_submit)
                self.completed += 1
            self._lock.notify_all()
        for p, r in zip(pend, results):
            p.future.set_result(r)


class NativeServer:
    """The same request kinds served by the library's native runtime (niq_server_create,
    niq_batch_submit / niq_batch_poll in include/niq.h): lanes of worker threads with their
    own CUDA streams and pre-allocated scratch take slices of the requests -- ray tiles of
    ``slice_rays`` rays first, closest-point slices of ``slice_queries`` queries and
    intersections after them -- as they free up.  ``submit`` returns a Future; a
    completion thread polls the tickets and copies the results to the host."""

    def __init__(self, params_list, mode='affine_fixed', n_lanes=4, slice_rays=16384, slice_queries=1024,
                 lane_scratch_bytes=512 << 20, lower=(-1., -1., -1.), upper=(1., 1., 1.), conservative=True):
        import torch
        self.torch = torch
        self.params = list(params_list)
        self.func, _ = generate_implicit_from_params(self.params[0], mode, conservative=conservative)
        self.models = [device_model(p) for p in self.params]
        self.lower = np.asarray(lower, np.float32)
        self.upper = np.asarray(upper, np.float32)
        self.L = _lib.load()
        so = _lib.ServerOpts(int(n_lanes), int(slice_rays), int(slice_queries), int(lane_scratch_bytes))
        h = _lib.C.c_void_p()
        _lib.check(self.L.niq_server_create(_lib.C.byref(so), _lib.C.byref(h)))
        self.handle = h
        self._lock = threading.Condition()
        self._pending = {}
        self._stop = False
        self.latencies = []
        self.kind_latencies = collections.defaultdict(list)
        self.completed = 0
        self.budget_exhausted = 0
        self._device = torch.cuda.current_device()
        self._done = threading.Thread(target=self._complete, daemon=True)
        self._done.start()

    def _request(self, kind, model):
        r = _lib.Request()
        r.kind = kind
        r.model = model.handle.value
        r.opts = self.func.bound_opts()
        r.lower = (_lib.C.c_float * 3)(*self.lower.tolist())
        r.upper = (_lib.C.c_float * 3)(*self.upper.tolist())
        return r

    def submit(self, req):
        """Queue a RayRequest, ClosestRequest or IntersectRequest; returns a Future of the
        results as the Python Server returns them."""
        torch = self.torch
        fut = Future()
        t0 = time.perf_counter()
        keep = []
        if isinstance(req, RayRequest):
            kind = 'rays'
            opts = req.opts or queries.get_default_cast_opts()
            roots = torch.from_numpy(np.ascontiguousarray(req.roots, np.float32)).cuda()
            dirs = torch.from_numpy(np.ascontiguousarray(req.dirs, np.float32)).cuda()
            n = roots.shape[0]
            t = torch.empty(n, dtype=torch.float32, device='cuda')
            hit = torch.empty(n, dtype=torch.int32, device='cuda')
            cnt = torch.empty(n, dtype=torch.int32, device='cuda')
            r = self._request(_lib.NIQ_REQ_RAYS, self.models[req.model])
            r.cast = _lib.cast_opts(opts)
            r.n, r.in0, r.in1 = n, roots.data_ptr(), dirs.data_ptr()
            r.out_f, r.out_i, r.out_i2 = t.data_ptr(), hit.data_ptr(), cnt.data_ptr()
            keep = [roots, dirs]
            outs = (t, hit, cnt)
        elif isinstance(req, ClosestRequest):
            kind = 'closest'
            q = torch.from_numpy(np.ascontiguousarray(req.points, np.float32)).cuda()
            n = q.shape[0]
            dist = torch.empty(n, dtype=torch.float32, device='cuda')
            loc = torch.empty((n, 3), dtype=torch.float32, device='cuda')
            r = self._request(_lib.NIQ_REQ_CLOSEST, self.models[req.model])
            r.n, r.in0, r.out_f, r.out_f2 = n, q.data_ptr(), dist.data_ptr(), loc.data_ptr()
            r.eps, r.node_budget = float(req.eps), int(req.node_budget or 0)
            keep = [q]
            outs = (dist, loc)
        else:
            kind = 'intersect'
            pa = prepend_op(self.params[req.model_a], spatial_transformation())
            pa['0000.spatial_transformation.R'] = np.asarray(req.R, np.float32)
            pa['0000.spatial_transformation.t'] = np.asarray(req.t, np.float32)
            pb = prepend_op(self.params[req.model_b], spatial_transformation())
            ma, mb = device_model(pa), device_model(pb)
            found = torch.zeros(1, dtype=torch.int32, device='cuda')
            loc = torch.empty(3, dtype=torch.float32, device='cuda')
            r = self._request(_lib.NIQ_REQ_INTERSECT, ma)
            r.model_b = mb.handle.value
            r.n, r.eps, r.node_capacity = 1, float(req.eps), 1 << 20
            r.out_i, r.out_f2 = found.data_ptr(), loc.data_ptr()
            keep = [ma, mb]
            outs = (found, loc)
        # the inputs are on the device before a lane (another stream) reads them
        torch.cuda.current_stream().synchronize()
        ticket = _lib.C.c_int64()
        _lib.check(self.L.niq_batch_submit(self.handle, _lib.C.byref(r), _lib.C.byref(ticket)))
        with self._lock:
            self._pending[ticket.value] = (kind, fut, t0, outs, keep)
            self._lock.notify_all()
        return fut

    def _complete(self):
        self.torch.cuda.set_device(self._device)
        done, status = _lib.C.c_int32(), _lib.C.c_int32()
        while True:
            with self._lock:
                while not self._pending and not self._stop:
                    self._lock.wait()
                if self._stop and not self._pending:
                    return
                tickets = list(self._pending)
            finished = []
            for tk in tickets:
                _lib.check(self.L.niq_batch_poll(self.handle, tk, _lib.C.byref(done), _lib.C.byref(status)))
                if done.value:
                    finished.append((tk, status.value))
            if not finished:
                time.sleep(0.0002)
                continue
            for tk, st in finished:
                with self._lock:
                    kind, fut, t0, outs, _ = self._pending.pop(tk)
                if st not in (0, _lib.NIQ_ERR_TIMEOUT):
                    fut.set_exception(_lib.NIQError(st, f"{kind} request failed"))
                    continue
                if st == _lib.NIQ_ERR_TIMEOUT:
                    self.budget_exhausted += 1
                if kind == 'intersect':
                    f, loc = outs
                    found = bool(f.item())
                    res = (True, 1, 2, loc.cpu().numpy()) if found else (False, 0, 0, loc.cpu().numpy())
                else:
                    res = tuple(o.cpu().numpy() for o in outs)
                now = time.perf_counter()
                with self._lock:
                    self.latencies.append(now - t0)
                    self.kind_latencies[kind].append(now - t0)
                    self.completed += 1
                fut.set_result(res)

    def stats(self):
        return Server.stats(self)

    def close(self):
        with self._lock:
            self._stop = True
            self._lock.notify_all()
        self._done.join()
        _lib.check(self.L.niq_server_destroy(self.handle))
