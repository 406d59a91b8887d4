"""Benchmark of the range-analysis query engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config tree|rays|batched]

Default workload (--config tree): the level-set kd-tree + hierarchical marching cubes of
a 3->64x4->1 ReLU MLP fitted to the SDF of 12 spheres, bisected 24 times (256^3 leaves,
affine_fixed with outward rounding), then marching cubes on every unknown leaf.  One
step = one full build + extraction.  ``value`` is bounded boxes per second of the
persistent form with the model resident on the device; ``e2e`` is the same through the
public Python API (kd_tree.hierarchical_marching_cubes) with the root box sent from the
host and the triangles read back every step.  The plain form (one launch + host sync
per level, the reference's loop structure) is measured beside it.

Multi-GPU: the path has no exchange step, so N GPUs run N independent replicas of the
workload (torchrun, one rank per GPU); value = all ranks' boxes / max-over-ranks time.

The default line also carries the plain-method ray cast at its stated size
(``rays_plain_method``: 128^2 rays, persistent vs plain, end to end and roofline) and a
bounded sample of the precision workload (``precision_sample``: 3xTF32 tensor-core vs FP32
products at 256 noise terms); ``--no-extras`` leaves them out.

--impl reference times the oracle's C/OpenMP restatement of the reference's algorithm
(oracle/cpu_tree.c; the reference itself is JAX and cannot run here) on all host cores:
each step builds the same 24-bisection tree and runs marching cubes on its leaves.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = 'neural-implicit-queries_gb300'

SPLIT_DEPTH = 24          # 256^3 leaves
CPU_DEPTH = 24            # the CPU baseline builds the same 256^3 tree


def mlp_macs(params):
    niq = importlib.import_module(PKG)
    return sum(A.shape[0] * A.shape[1] for A, _, _ in niq.mlp.spec_layers(params))


def box_flops(params, v=3):
    """Algorithmic FLOPs of one bounded box: 2 (v + 2) S, S = sum in*out."""
    return 2 * (v + 2) * mlp_macs(params)


def max_over_ranks(vals, world):
    """Each value's maximum over the ranks (all_reduce MAX); identity for one rank."""
    if world <= 1:
        return list(vals)
    import torch
    import torch.distributed as dist
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    tt = torch.tensor(list(vals), dtype=torch.float64, device=dev)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return tt.tolist()


def replica_rate(units_per_rank, t_max, world):
    """Whole-job rate of independent replicas: every rank's units over the slowest rank's time."""
    return world * units_per_rank / t_max


def dist_info():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


class ClockSampler:
    """SM clock and throttle reasons sampled during the timed region: NVML read through
    ctypes every 10 ms (nvmlDeviceGetClockInfo, nvmlDeviceGetCurrentClocksEventReasons),
    else nvidia-smi every 200 ms.  Read-only; no setting of the GPU is touched."""
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
    # nvmlClocksEventReason bits
    REASONS = {0x8: 'hw_slowdown', 0x40: 'hw_thermal_slowdown', 0x20: 'sw_thermal_slowdown', 0x4: 'sw_power_cap'}

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.thread = None
        self.rows = []

    def _nvml(self):
        import ctypes
        try:
            nv = ctypes.CDLL('libnvidia-ml.so.1')
        except OSError:
            return None
        if nv.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        if nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.gpu), ctypes.byref(h)) != 0:
            return None
        return nv, h

    def _poll(self, nv, h):
        import ctypes
        mhz, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        get_reasons = getattr(nv, 'nvmlDeviceGetCurrentClocksEventReasons', None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        while not self._stop:
            if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0 and get_reasons(h, ctypes.byref(rs)) == 0:
                self.rows.append((float(mhz.value), float(mx.value), int(rs.value)))
            time.sleep(0.01)

    def __enter__(self):
        import threading
        self._stop = False
        handle = self._nvml()
        if handle is not None:
            self.thread = threading.Thread(target=self._poll, args=handle, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(['nvidia-smi', f'--id={self.gpu}', f'--query-gpu={self.FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ''
        self._stop = True
        if self.thread is not None:
            self.thread.join(timeout=5)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        if self.rows:
            sm = [r[0] for r in self.rows]
            reasons = sorted({name for r in self.rows for bit, name in self.REASONS.items() if r[2] & bit})
            return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(r[1] for r in self.rows),
                    "reasons": reasons, "samples": len(self.rows), "source": "NVML, 10 ms"}
        rows = []
        for line in (self.out or '').strip().splitlines():
            p = [x.strip() for x in line.split(',')]
            if len(p) >= 9:
                rows.append(p)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace('.', '', 1).isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].replace('.', '', 1).isdigit())
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == 'active'})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows), "source": "nvidia-smi, 200 ms"}


def flush_l2(buf):
    buf.add_(1.0)


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    torch.cuda.set_device(local)
    niq = importlib.import_module(PKG)
    lib = importlib.import_module(PKG + '._lib')
    io = importlib.import_module(PKG + '._io')
    kd = niq.kd_tree
    params = niq.workloads.spheres_sdf_model()
    f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=True)
    lower, upper = np.full(3, -1., np.float32), np.ones(3, np.float32)
    model = niq.mlp.device_model(params)
    L = lib.load()
    bo = f.bound_opts()
    eng = lib.C.c_int32(-1)
    lib.check(L.niq_tree_engine(model.handle, lib.C.byref(bo), lib.C.byref(eng)))
    tree_engine = {0: "fp32 tile engine (k_tree)", 1: "tensor cores, 3xTF32 hidden layers (k_tree_tc)",
                   2: "growing-term engine"}[eng.value]
    stream = torch.cuda.current_stream()
    l2buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device='cuda')  # 256 MiB > 129 MB L2

    # ---- device-resident form: tree (one cooperative launch) + HMC extraction
    cap = 1 << 23
    ws_bytes = L.niq_tree_workspace_size(cap, 0)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device='cuda')
    counts = torch.zeros(4, dtype=torch.int64, device='cuda')
    hws = torch.empty(L.niq_hmc_workspace_size(), dtype=torch.uint8, device='cuda')
    tri_cap = 1 << 23
    tris = torch.empty((tri_cap, 3, 3), dtype=torch.float32, device='cuda')
    ntri = torch.zeros(1, dtype=torch.int64, device='cuda')
    lo3 = (lib.C.c_float * 3)(*lower.tolist())
    hi3 = (lib.C.c_float * 3)(*upper.tolist())

    def tree_step(plain=False):
        if plain == 'batches':   # the reference's schedule: one launch per 2048 nodes
            lib.check(L.niq_levelset_tree_batches(model.handle, lib.C.byref(bo), lo3, hi3, args.split_depth, 0, 0.0,
                                                  0, 2048, cap, io.ptr(counts), io.ptr(ws), ws_bytes,
                                                  stream.cuda_stream))
            return
        fn = L.niq_levelset_tree_plain if plain else L.niq_levelset_tree
        lib.check(fn(model.handle, lib.C.byref(bo), lo3, hi3, args.split_depth, 0, 0.0, 0, cap, io.ptr(counts),
                     io.ptr(ws), ws_bytes, stream.cuda_stream))

    def hmc_step():
        # marching cubes on the leaves (n_subcell_depth 0): shared lattice corners once
        n_leaves = int(counts_host[0])
        lo, hi = kd._tree_nodes(ws, cap, 0, 0, n_leaves)
        lib.check(L.niq_hmc_extract_lattice(model.handle, n_leaves, io.ptr(lo), io.ptr(hi), lo3, hi3, args.split_depth,
                                            io.ptr(tris), tri_cap, io.ptr(ntri), io.ptr(lws), lws.numel(),
                                            stream.cuda_stream))

    tree_step()
    counts_host = counts.cpu().numpy()
    n_boxes = int(counts_host[3])
    lws = torch.empty(L.niq_hmc_lattice_workspace_size(lo3, hi3, args.split_depth, int(counts_host[0])),
                      dtype=torch.uint8, device='cuda')
    hmc_step()
    n_tris = int(ntri.item())

    def timed(fn_step, K, W):
        for _ in range(W):
            fn_step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        times = []
        for _ in range(K):
            flush_l2(l2buf)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn_step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return times

    tree_t, hmc_t = [], []

    def full_step():
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        tree_step()
        e1.record(stream)
        hmc_step()
        e2.record(stream)
        e2.synchronize()
        tree_t.append(e0.elapsed_time(e1) / 1e3)
        hmc_t.append(e1.elapsed_time(e2) / 1e3)

    with ClockSampler(local) as clk:
        step_times = timed(full_step, args.steps, args.warmup)
    tree_t, hmc_t = tree_t[args.warmup:], hmc_t[args.warmup:]
    t_step = sum(step_times) / len(step_times)
    if args.quick:   # profiling runs: the timed steps only
        print(json.dumps({"quick": True, "ms_per_step": t_step * 1e3, "boxes": n_boxes}))
        return

    # ---- plain form (per-level launches + host syncs), same tree
    plain_times = timed(lambda: tree_step(plain=True), max(3, args.steps // 2), 1)
    t_plain = sum(plain_times) / len(plain_times)
    # ---- the reference's schedule with the same kernel: launches of 2048 nodes
    batch_times = timed(lambda: tree_step(plain='batches'), max(2, args.steps // 3), 1)
    t_batch = sum(batch_times) / len(batch_times)

    # ---- e2e through the public API: host root box in, host triangles out
    def e2e_step():
        return kd.hierarchical_marching_cubes(f, params, lower, upper, args.split_depth // 3, n_subcell_depth=0)
    for _ in range(args.warmup):
        out = e2e_step()
    torch.cuda.synchronize()
    e2e_times = []
    for _ in range(args.steps):
        flush_l2(l2buf)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = e2e_step()
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    t_e2e = sum(e2e_times) / len(e2e_times)

    # ---- the CPU reference arm's work: the same tree and marching cubes in the reference's
    #      arithmetic (no outward rounding), end to end through the same call
    f_ref, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=False)
    bo_ref = f_ref.bound_opts()
    lib.check(L.niq_levelset_tree(model.handle, lib.C.byref(bo_ref), lo3, hi3, args.split_depth, 0, 0.0, 0, cap,
                                  io.ptr(counts), io.ptr(ws), ws_bytes, stream.cuda_stream))
    n_boxes_ref = int(counts.cpu().numpy()[3])

    def e2e_ref_step():
        return kd.hierarchical_marching_cubes(f_ref, params, lower, upper, args.split_depth // 3, n_subcell_depth=0)
    for _ in range(args.warmup):
        out_ref = e2e_ref_step()
    torch.cuda.synchronize()
    ref_times = []
    for _ in range(max(3, args.steps // 2)):
        flush_l2(l2buf)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out_ref = e2e_ref_step()
        torch.cuda.synchronize()
        ref_times.append(time.perf_counter() - t0)
    t_e2e_ref = sum(ref_times) / len(ref_times)

    # ---- max over ranks
    t_step, t_e2e, t_plain, t_batch, t_e2e_ref = max_over_ranks([t_step, t_e2e, t_plain, t_batch, t_e2e_ref], world)
    value = replica_rate(n_boxes, t_step, world)
    bf = box_flops(params)
    t_tree = sum(tree_t) / len(tree_t)
    line = {
        "metric": "bounded boxes/s (level-set tree 256^3 + HMC, 12-sphere ReLU 3x64x4 MLP, affine_fixed)",
        "value": value, "unit": "boxes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (fitted 12-sphere SDF MLP, committed weights)",
        "config": dict(WORKLOAD_CONFIG, split_depth=args.split_depth, parallelism=f"replicas x{world}"),
        "details": {"leaves": int(counts_host[0]), "boxes_per_step": n_boxes, "triangles_per_step": n_tris,
                    "arithmetic": "affine_fixed with outward rounding (every bound conservative)",
                    "tree_engine": tree_engine,
                    "l2": "flushed: 256 MiB write between timed steps"},
        "e2e": {"value": replica_rate(n_boxes, t_e2e, world), "unit": "boxes/s", "h2d_bytes_per_step": 24,
                "d2h_bytes_per_step": int(out.nbytes) + 32, "ms_per_step": t_e2e * 1e3,
                "api": "kd_tree.hierarchical_marching_cubes(depth=8, n_subcell_depth=0)"},
        "e2e_reference_arithmetic": {
            "value": replica_rate(n_boxes_ref, t_e2e_ref, world), "unit": "boxes/s", "ms_per_step": t_e2e_ref * 1e3,
            "boxes_per_step": n_boxes_ref, "triangles_per_step": int(len(out_ref)),
            "api": "kd_tree.hierarchical_marching_cubes(depth=8, n_subcell_depth=0), conservative=False",
            "note": "the work of the CPU reference arm: the tree and marching cubes without outward rounding"},
        "plain": {"value": replica_rate(n_boxes, t_plain, world), "unit": "boxes/s", "ms_per_step": t_plain * 1e3,
                  "form": "one launch + host sync per level (niq_levelset_tree_plain)",
                  "persistent_speedup": t_plain / (sum(tree_t) / len(tree_t))},
        "plain_reference_schedule": {
            "value": replica_rate(n_boxes, t_batch, world), "unit": "boxes/s", "ms_per_step": t_batch * 1e3,
            "form": "the reference's schedule on the same kernel: one launch per 2048 nodes, host sync per level "
                    "(niq_levelset_tree_batches)",
            "persistent_speedup": t_batch / (sum(tree_t) / len(tree_t))},
        "phases_ms": {"tree": t_tree * 1e3, "hmc": sum(hmc_t) / len(hmc_t) * 1e3,
                      "tree_min": min(tree_t) * 1e3, "tree_max": max(tree_t) * 1e3},
        "roofline": tree_roofline(eng.value, n_boxes, bf, t_tree, params, local),
        "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_extras:
        line["rays_plain_method"] = rays_plain_method(niq, args.steps, args.warmup, l2buf)
        line["precision_sample"] = precision_sample(niq, args.steps, args.warmup)
        line["batched_sample"] = batched_sample(niq, args.steps, args.warmup)
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(params)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


# DRAM bytes per classified box of the tree kernels: ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one k_tree launch on this workload (24 bisections, the timed
# step after the L2 flush): 0.48 MB read, 16.67 MB written -- the 727,581 unknown leaves
# of 24 B; the level arrays stay in L2.  Keyed by the engine code of niq_tree_engine.
TREE_DRAM_BYTES_PER_BOX = {0: (475392 + 16673536) / 3735843}
TREE_DRAM_SOURCE = {0: "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_tree launch on the 24-bisection "
                       "tree (0.48 MB read, 16.67 MB written for 3,735,843 boxes: the leaf output)"}


def tree_roofline(engine, n_boxes, bf, t_tree, params, device):
    """Roofline of the tree kernel: algorithmic FLOPs (2 (v + 2) S per box) over the
    tree phase's CUDA-event time.  The FP32 engine is bound by the FP32 FMA pipe; the
    tensor-core engine executes the four signed rows of every hidden layer as 3 tf32
    products per FLOP on the tensor pipe (tf32 ceiling measured live, tf32_peak_tflops)
    and the err row and the linearisations on the FP32 pipe, so both fractions are given."""
    hidden = sum(A.shape[0] * A.shape[1] for A, _, _ in importlib.import_module(PKG).mlp.spec_layers(params)[1:-1])
    achieved = n_boxes * bf / t_tree / 1e12
    fp32_peak = fp32_peak_tflops(device)
    fp32_nominal = fp32_nominal_tflops(device)
    tf32_peak = tf32_peak_tflops() if engine == 1 else None
    per_box = TREE_DRAM_BYTES_PER_BOX.get(engine)
    out = {"kernel": "k_tree_tc (persistent level-set tree, tensor cores)" if engine == 1
           else "k_tree (persistent level-set tree)",
           "achieved": achieved, "unit": "TFLOP/s", "flops_per_box": bf,
           "traffic": per_box * n_boxes if per_box is not None else None,
           "traffic_source": TREE_DRAM_SOURCE.get(engine, "not captured for this kernel")}
    if engine == 1:
        tensor = n_boxes * 3 * 2 * 4 * hidden / t_tree / 1e12
        out.update({"bound": "tensor", "peak": tf32_peak, "frac": achieved / tf32_peak,
                    "tensor_pipe_tflops": tensor, "tensor_pipe_frac": tensor / tf32_peak,
                    "fp32_peak": fp32_peak, "frac_of_fp32_peak": achieved / fp32_peak,
                    "peak_source": TF32_PEAK_SOURCE + "; FP32: " + FP32_PEAK_SOURCE})
    else:
        out.update({"bound": "fp32", "peak": fp32_peak, "frac": achieved / fp32_peak,
                    "nominal_peak": fp32_nominal, "frac_of_nominal": achieved / fp32_nominal,
                    "peak_source": FP32_PEAK_SOURCE})
    return out


def rays_plain_method(niq, steps, warmup, l2buf):
    """The plain-method workload at its stated size: 128 x 128 rays of the 3->32x3->1 ReLU
    model (He-normal seed 0, median-biased), affine_fixed with outward rounding, 64 steps,
    eye at distance 3 aimed at the origin, 60 degree field of view.  Persistent (one
    launch) and plain (one launch + host compaction per iteration) forms with the rays
    resident on the device, and end to end through queries.cast_rays with host arrays in
    and out.  Roofline: 10 S FLOP per ray-step (one v = 1 segment bound, 6 S, and two
    point evaluations, 4 S; S = 2,176 MACs) against the FP32 FMA peak."""
    import torch
    params = niq.workloads.plain_small_model()
    f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=True)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    eye = np.array([0., 0., 3.], np.float32)
    look, up, _ = niq.render.look_at(eye)
    roots, dirs = niq.render.generate_camera_rays(eye, look, up, res=128, fov_deg=60.)
    rt, dt = torch.from_numpy(roots).cuda(), torch.from_numpy(dirs).cuda()
    n = roots.shape[0]
    stream = torch.cuda.current_stream()
    out = {}
    for form, persistent in (("persistent", True), ("plain", False)):
        for _ in range(warmup):
            r = niq.queries.cast_rays((f,), (params,), rt, dt, opts, persistent=persistent, return_device=True)
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            flush_l2(l2buf)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = niq.queries.cast_rays((f,), (params,), rt, dt, opts, persistent=persistent, return_device=True)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        t = sum(ts) / len(ts)
        out[form] = {"value": n / t, "unit": "rays/s", "ms_per_step": t * 1e3,
                     "ray_steps": int(r[2].sum().item()), "hits": int((r[1] > 0).sum().item())}
    # end to end: host roots/dirs in, host t/hit_id/count out, every step
    for _ in range(warmup):
        niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
    ts = []
    for _ in range(steps):
        flush_l2(l2buf)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t_, hid, cnt, _ = niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
        ts.append(time.perf_counter() - t0)
    te = sum(ts) / len(ts)
    macs = mlp_macs(params)
    fl = 10 * macs * out["persistent"]["ray_steps"]
    peak = fp32_peak_tflops(torch.cuda.current_device())
    ach = fl / (out["persistent"]["ms_per_step"] * 1e-3) / 1e12
    out["persistent"]["e2e"] = {"value": n / te, "unit": "rays/s", "ms_per_step": te * 1e3,
                                "h2d_bytes_per_step": int(roots.nbytes + dirs.nbytes),
                                "d2h_bytes_per_step": int(t_.nbytes + hid.nbytes + cnt.nbytes + 8),
                                "api": "queries.cast_rays (numpy in, numpy out)"}
    nominal = fp32_nominal_tflops(torch.cuda.current_device())
    out["persistent"]["roofline"] = {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                                     "frac": ach / peak, "nominal_peak": nominal, "frac_of_nominal": ach / nominal,
                                     "flops_per_ray_step": 10 * macs, "peak_source": FP32_PEAK_SOURCE}
    out["persistent_vs_plain"] = out["plain"]["ms_per_step"] / out["persistent"]["ms_per_step"]
    out["config"] = {"workload": "cast_rays_plain_method", "model": "relu 3-32x3-1 he-normal seed 0",
                     "rays": n, "n_max_step": 64, "mode": "affine_fixed conservative",
                     "l2": "flushed between timed steps"}
    return out


def precision_sample(niq, steps, warmup):
    """The precision workload on a bounded sample: ReLU 3->256x8->1 (seed 7, median-biased),
    affine_truncate with 256 noise terms, conservative, the 3xTF32 tensor-core products
    against FP32 FMA.  1024 boxes of half-width 0.01 are classified per form, and an 8x8
    strided sample of the 1024x1024 ray image (every 128th ray per axis) is cast: a
    segment costs about 237 MFLOP at 256 terms, so the full image takes minutes.
    Roofline of the tensor-core classification: 3 tf32 products per algorithmic FLOP
    against the dense tf32 peak (half the measured bf16 burst)."""
    import torch
    params = niq.workloads.precision_model()
    eye = np.array([0., 0., 3.], np.float32)
    look, up, _ = niq.render.look_at(eye)
    roots, dirs = niq.render.generate_camera_rays(eye, look, up, res=1024, fov_deg=60.)
    sub = (np.arange(0, 1024, 128)[:, None] * 1024 + np.arange(0, 1024, 128)[None, :]).reshape(-1)
    rs, ds = torch.from_numpy(roots[sub]).cuda(), torch.from_numpy(dirs[sub]).cuda()
    opts = niq.queries.get_default_cast_opts()
    dims = [(A.shape[0], A.shape[1], act) for A, _, act in niq.mlp.spec_layers(params)]
    fl, rows = 0, 3
    for i, o, act in dims:
        fl += 2 * (rows + 2) * i * o
        if act != 'none':
            rows = min(rows + o, 256)
    rng = np.random.default_rng(3)
    nb = 1024
    c = torch.from_numpy(rng.uniform(-0.8, 0.8, (nb, 3)).astype(np.float32)).cuda()
    vv = torch.from_numpy(np.tile((0.01 * np.eye(3, dtype=np.float32))[None], (nb, 1, 1))).cuda()

    def timed(fn, k, w):
        for _ in range(w):
            r = fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return r, sum(ts) / len(ts)
    out = {}
    dm = niq.mlp.device_model(params)   # the resident model: no per-call hashing of its weights
    for name, products in (("3xtf32", "3xtf32"), ("fp32", "fp32")):
        f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_truncate', conservative=True,
                                                                    products=products, affine_n_truncate=256)
        _, tb = timed(lambda: f.bounds_general_box(dm, c, vv), max(1, steps // 4), 1)
        r, tr = timed(lambda: niq.queries.cast_rays((f,), (dm,), rs, ds, opts, return_device=True), 1, 1)
        out[name] = {"boxes_per_s": nb / tb, "classify_ms": tb * 1e3, "rays_per_s": rs.shape[0] / tr,
                     "cast_ms": tr * 1e3, "ray_steps": int(r[2].sum().item()),
                     "achieved_tflops": nb * fl / tb / 1e12}
    tf32_peak = tf32_peak_tflops()
    a3 = 3 * out["3xtf32"]["achieved_tflops"]
    out["3xtf32"]["roofline"] = {"bound": "tensor", "achieved": a3, "peak": tf32_peak, "unit": "TFLOP/s",
                                 "frac": a3 / tf32_peak, "peak_source": TF32_PEAK_SOURCE}
    out["tensor_vs_fp32"] = {"boxes": out["3xtf32"]["boxes_per_s"] / out["fp32"]["boxes_per_s"],
                             "rays": out["3xtf32"]["rays_per_s"] / out["fp32"]["rays_per_s"]}
    out["config"] = {"workload": "precision_relu256x8_truncate256", "boxes": nb, "rays": int(rs.shape[0]),
                     "flop_per_box": fl, "sample": "8x8 strided rays of the 1024x1024 image"}
    return out


def batched_sample(niq, steps, warmup, n_models=64, node_budget=2048):
    """A bounded sample of the batched workload: the first 64 of its 512 MLPs (widths
    U{16..128}, depths U{2..6}, ReLU or TanH), each with 64-4096 closest-point queries drawn
    as the full workload draws them (workloads.batched_queries for 64 models),
    eps 1e-3, in one persistent launch with autotuned chunking, against one single-model
    persistent launch per model.  Both forms stop a query after `node_budget` nodes (the
    networks are untrained, their bounds loose); the count of such queries is reported."""
    import torch
    models = niq.workloads.batched_models(n_models)
    qs = niq.workloads.batched_queries(n_models)
    f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(models[0], 'affine_fixed', conservative=True)
    table = niq.batched.ModelTable(models)
    counts = np.array([len(q) for q in qs], np.int64)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    allq = torch.from_numpy(np.concatenate(qs)).cuda()
    lo, hi = np.full(3, -1.2, np.float32), np.full(3, 1.2, np.float32)
    jm = np.arange(n_models, dtype=np.int32)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    tuned, _ = niq.autotune.tune_batched(f, table, jm, offs, counts, allq, lo, hi, 1e-3, node_budget=node_budget,
                                         chunks=(64, 128), ctas=(1,), reps=1, use_cache=False)

    def batched_step():
        niq.batched.closest_point_packed(f, table, jm, offs, counts, allq, lo, hi, 1e-3, status=status,
                                         node_budget=node_budget)
    for _ in range(max(1, warmup // 3)):
        batched_step()
    torch.cuda.synchronize()
    ts = []
    for _ in range(max(1, steps // 5)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        batched_step()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    t_b = sum(ts) / len(ts)
    n_spent, n_nodes = niq.batched.stats()
    # one single-model persistent launch per model (the same traversal and budget)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(n_models):
        niq.kd_tree.closest_point(f, table.models[i], lo, hi, allq[offs[i]:offs[i] + counts[i]], eps=1e-3,
                                  persistent=True, node_budget=node_budget, strict=False)
    torch.cuda.synchronize()
    t_p = time.perf_counter() - t0
    nq = int(counts.sum())
    return {"value": nq / t_b, "unit": "queries/s", "ms_per_step": t_b * 1e3,
            "plain_per_model_calls": {"value": nq / t_p, "unit": "queries/s", "ms_per_step": t_p * 1e3},
            "batched_vs_plain": t_p / t_b, "autotuned": tuned,
            "nodes_per_s": n_nodes / t_b, "nodes_per_pass": n_nodes,
            "queries_spent_budget": n_spent, "fraction_spent_budget": n_spent / max(nq, 1),
            "config": {"workload": "batched_closest_point", "models": n_models, "queries": nq, "eps": 1e-3,
                       "node_budget": node_budget,
                       "sample": "the first 64 of the 512 models, queries drawn for 64 models (a full pass "
                                 "over all 512 takes about 30 s)",
                       "note": "a query that spends its node budget keeps its best candidate, an upper bound"}}


WORKLOAD_CONFIG = {"workload": "levelset_tree_hmc", "model": "relu 3-64x4-1 spheres12", "split_depth": SPLIT_DEPTH,
                   "hmc": "marching cubes on every unknown leaf (depth 8, n_subcell_depth 0)"}


def cpu_tree_hmc_step(layers, depth, cores):
    """One step of the workload on the host cores through the oracle's C/OpenMP
    restatement (oracle/cpu_tree.c): the level-set tree to ``depth`` bisections in the
    reference's arithmetic, then marching cubes on every unknown leaf.  Returns
    (boxes classified, triangles)."""
    from oracle import cpu_tree
    _, nb, leaves = cpu_tree.levelset_tree(layers, -np.ones(3), np.ones(3), depth, threads=cores, want_leaves=True)
    tris = cpu_tree.hmc_leaves(layers, leaves, threads=cores)
    return nb, tris.shape[0]


def cpu_baseline(params, seconds=20.0, depth=CPU_DEPTH):
    """The oracle's C/OpenMP restatement (oracle/cpu_tree.c, float32, the reference's
    arithmetic) on every host core: the same tree + marching-cubes step, repeated for up
    to ``seconds`` (at most 3 times); the NumPy oracle's rate on a 15-bisection tree is
    reported beside it."""
    from oracle import ref_np as R
    niq = importlib.import_module(PKG)
    layers = niq.mlp.spec_layers(params)
    cores = os.cpu_count()
    t0 = time.perf_counter()
    boxes, reps, ntri = 0, 0, 0
    while True:
        nb, ntri = cpu_tree_hmc_step(layers, depth, cores)
        boxes += nb
        reps += 1
        if time.perf_counter() - t0 > seconds or reps >= 3:
            break
    dt = time.perf_counter() - t0
    f = R.generate_implicit(params, 'affine_fixed')
    t1 = time.perf_counter()
    d = R.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=15)
    np_rate = d['n_boxes_classified'] / (time.perf_counter() - t1)
    return {"value": boxes / dt, "unit": "boxes/s", "cores": cores, "kind": "port",
            "sample": f"oracle/cpu_tree.c (C, OpenMP on {cores} threads): level-set tree of the same model to "
                      f"{depth} bisections ({boxes // reps} boxes) and marching cubes on its leaves ({ntri} "
                      f"triangles), x{reps}",
            "numpy_oracle_boxes_per_s": np_rate}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    niq = importlib.import_module(PKG)
    params = niq.workloads.spheres_sdf_model()
    layers = niq.mlp.spec_layers(params)
    cores = os.cpu_count()
    depth = CPU_DEPTH
    for _ in range(args.warmup):
        cpu_tree_hmc_step(layers, depth - 6, cores)
    times, boxes, ntri = [], 0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        boxes, ntri = cpu_tree_hmc_step(layers, depth, cores)
        times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    v = boxes / t
    line = {"impl": "reference",
            "metric": "bounded boxes/s (level-set tree 256^3 + HMC, 12-sphere ReLU 3x64x4 MLP, affine_fixed)",
            "value": v, "unit": "boxes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (fitted 12-sphere SDF MLP, committed weights)",
            "config": dict(WORKLOAD_CONFIG, parallelism=f"replicas x{world}"),
            "details": {"boxes_per_step": int(boxes), "triangles_per_step": int(ntri), "host_cores": cores,
                        "arithmetic": "the reference's: float32, round to nearest, no outward rounding",
                        "note": "the reference is JAX, which is absent; the oracle's C/OpenMP restatement of its "
                                "tree and marching cubes runs on the host cores"},
            "cpu_baseline": {"value": v, "unit": "boxes/s", "cores": cores, "kind": "port",
                             "sample": f"oracle/cpu_tree.c tree to {depth} bisections ({boxes} boxes) + marching "
                                       f"cubes ({ntri} triangles), OpenMP on {cores} threads"},
            "e2e": {"value": v, "unit": "boxes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_rays(args):
    """Plain-method config: 3->32x3->1 ReLU (He-normal seed 0, median-biased), camera at
    distance 3 looking at the origin, 60 deg FOV, n_max_step 64, affine_fixed."""
    import torch
    niq = importlib.import_module(PKG)
    params = niq.workloads.plain_small_model()
    f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=True)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    look, up, _ = niq.render.look_at(np.array([0., 0., 3.], np.float32))
    out = {"metric": "rays/s (cast_rays, 3x32x3 ReLU MLP, affine_fixed)", "unit": "rays/s", "config": {}}
    if args.quick:   # profiling runs: the persistent 128^2 cast only
        roots, dirs = niq.render.generate_camera_rays(np.array([0., 0., 3.], np.float32), look, up, res=128, fov_deg=60.)
        rt, dt = torch.from_numpy(roots).cuda(), torch.from_numpy(dirs).cuda()
        dm = niq.mlp.device_model(params)
        for _ in range(args.warmup + args.steps):
            r = niq.queries.cast_rays((f,), (dm,), rt, dt, opts, return_device=True)
        torch.cuda.synchronize()
        c = r[2].cpu().numpy()
        print(json.dumps({"quick": True, "rays": int(c.size), "ray_steps": int(c.sum()), "max_steps": int(c.max()),
                          "steps_hist_by_8": np.bincount(np.minimum(c, 64) // 8).tolist()}))
        return
    for res in (128, 1024):
        roots, dirs = niq.render.generate_camera_rays(np.array([0., 0., 3.], np.float32), look, up, res=res, fov_deg=60.)
        rt, dt = torch.from_numpy(roots).cuda(), torch.from_numpy(dirs).cuda()
        res_out = {}
        for form, persistent in (("persistent", True), ("plain", False)):
            for _ in range(args.warmup):
                r = niq.queries.cast_rays((f,), (params,), rt, dt, opts, persistent=persistent, return_device=True)
            torch.cuda.synchronize()
            times = []
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                r = niq.queries.cast_rays((f,), (params,), rt, dt, opts, persistent=persistent, return_device=True)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1) / 1e3)
            t = sum(times) / len(times)
            steps = int(r[2].sum().item())
            res_out[form] = {"rays_per_s": res * res / t, "ms": t * 1e3, "ray_steps_per_s": steps / t,
                             "hits": int((r[1] > 0).sum().item())}
        res_out["persistent_speedup"] = res_out["plain"]["ms"] / res_out["persistent"]["ms"]
        # the frustum cast of the same image (src/queries.py:178-587), 16x16 initial frusta
        eye = np.array([0., 0., 3.], np.float32)
        left = np.cross(look, up).astype(np.float32)
        cam = (eye, look, up, left, 60., 60., res, res)
        fo = dict(opts)
        fo['n_side_init'] = 16
        for _ in range(max(1, args.warmup)):
            fr = niq.queries.cast_rays_frustum((f,), (params,), cam, fo)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fr = niq.queries.cast_rays_frustum((f,), (params,), cam, fo)
        torch.cuda.synchronize()
        tf_ = (time.perf_counter() - t0) / args.steps
        res_out["frustum"] = {"pixels_per_s": res * res / tf_, "ms": tf_ * 1e3, "frustum_steps": int(fr[3]),
                              "hits": int((fr[1] > 0).sum()), "timing": "wall clock incl. host loop and D2H"}
        out["config"][f"{res}x{res}"] = res_out
    out["value"] = out["config"]["1024x1024"]["persistent"]["rays_per_s"]
    print(json.dumps(out))


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
    except (OSError, ValueError):
        return {}


def tf32_peak_tflops():
    """The tensor-core ceiling of the 3xTF32 engine's dense step, measured live on this GPU
    (niq_tc_tf32_rate: the engine's own MMA sequence, no staging or epilogue)."""
    lib = importlib.import_module(PKG + '._lib')
    L = lib.load()
    v = lib.C.c_float(0.)
    lib.check(L.niq_tc_tf32_rate(4096, lib.C.byref(v), None))
    return float(v.value)


TF32_PEAK_SOURCE = ("tcgen05 kind::tf32 rate of the engine's dense step measured live on this GPU "
                    "(niq_tc_tf32_rate); MEASURED_PEAKS.json has no tf32 figure")


def fp32_nominal_tflops(device=0):
    """FP32 FMA pipe, nominal: SMs x 128 lanes x 2 FLOP x the measured maximum SM clock."""
    import torch
    sm_max = float(measured_peaks().get('sm_max_mhz', 2070.0))
    return torch.cuda.get_device_properties(device).multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12


_FP32_RATE = {}


def fp32_peak_tflops(device=0):
    """The FP32 FMA ceiling measured live on this GPU (niq_fp32_fma_rate: packed fp32x2 FMA
    chains on registers, every SM busy), at the clock the GPU holds now; measured once."""
    if device not in _FP32_RATE:
        lib = importlib.import_module(PKG + '._lib')
        L = lib.load()
        v = lib.C.c_float(0.)
        lib.check(L.niq_fp32_fma_rate(8192, lib.C.byref(v), None))
        _FP32_RATE[device] = float(v.value)
    return _FP32_RATE[device]


FP32_PEAK_SOURCE = ("packed fp32x2 FMA rate measured live on this GPU (niq_fp32_fma_rate); MEASURED_PEAKS.json "
                    "has no FP32 figure; nominal = SMs x 128 lanes x 2 FLOP x the measured maximum SM clock")


def run_precision(args):
    """Deep-model config: ReLU 3->256x8->1 (He-normal seed 7, median-biased output), rays
    from an eye at distance 3 aimed at the origin, 60 deg FOV, the reference's default
    cast options.  'affine_truncate' with 256 noise terms costs about 2 x 258 x 256 x 256
    FLOP per layer and segment, so the casts use a strided 32x32 sample of the 1024x1024
    image (every 32nd ray in each direction); 1024 boxes of half-width 0.01 are classified
    per form.  Forms: 'affine_fixed' (FP32 FMA tile engine) and 'affine_truncate' 256
    with FP32 FMA products or 3xTF32 tensor-core products."""
    import torch
    niq = importlib.import_module(PKG)
    params = niq.workloads.precision_model()
    eye = np.array([0., 0., 3.], np.float32)
    look, up, _ = niq.render.look_at(eye)
    roots, dirs = niq.render.generate_camera_rays(eye, look, up, res=1024, fov_deg=60.)
    opts = niq.queries.get_default_cast_opts()
    layers = niq.mlp.spec_layers(params)
    dims = [(A.shape[0], A.shape[1], act) for A, _, act in layers]

    def box_flop(v, K=None):
        """2 (rows) in out per layer: base, err and the noise rows; 'affine_truncate'
        appends out rows after each activation and keeps K."""
        tot, rows = 0, v
        for i, o, act in dims:
            tot += 2 * (rows + 2) * i * o
            if K is not None and act != 'none':
                rows = min(rows + o, K)
        return tot

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            r = fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return r, sum(ts) / len(ts)
    sub = (np.arange(0, 1024, 32)[:, None] * 1024 + np.arange(0, 1024, 32)[None, :]).reshape(-1)
    rs = torch.from_numpy(roots[sub]).cuda()
    ds = torch.from_numpy(dirs[sub]).cuda()
    rng = np.random.default_rng(3)
    nb = 1024
    c = torch.from_numpy(rng.uniform(-0.8, 0.8, (nb, 3)).astype(np.float32)).cuda()
    vv = torch.from_numpy(np.tile((0.01 * np.eye(3, dtype=np.float32))[None], (nb, 1, 1))).cuda()
    peak32 = fp32_peak_tflops(torch.cuda.current_device())
    tf32_peak = tf32_peak_tflops()
    forms = [("affine_fixed", 'affine_fixed', {}, 'auto', box_flop(3)),
             ("affine_truncate256_fp32", 'affine_truncate', {'affine_n_truncate': 256}, 'fp32', box_flop(3, 256)),
             ("affine_truncate256_3xtf32", 'affine_truncate', {'affine_n_truncate': 256}, '3xtf32', box_flop(3, 256))]
    out = {"metric": "rays/s and bounded boxes/s, ReLU 3x256x8 MLP (32x32 strided rays of 1024^2)",
           "unit": "rays/s", "config": {"workload": "precision_relu256x8", "rays": int(rs.shape[0]),
                                        "boxes": nb, "conservative": True}}
    if args.quick:   # profiling runs: the tensor-core classification only
        forms = forms[2:]
    dm = niq.mlp.device_model(params)   # the resident model: no per-call hashing of its weights
    for name, mode, kw, products, fl in forms:
        f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=True,
                                                                    products=products, **kw)
        if args.quick:
            _, tb = timed(lambda: f.bounds_general_box(dm, c, vv), 1, 1)
            print(json.dumps({"quick": True, "classify_ms": tb * 1e3, "boxes": nb}))
            return
        r, t = timed(lambda: niq.queries.cast_rays((f,), (dm,), rs, ds, opts, return_device=True), 1, 1)
        _, tb = timed(lambda: f.bounds_general_box(dm, c, vv), 3, 1)
        tf = nb * fl / tb / 1e12
        row = {"rays_per_s": rs.shape[0] / t, "cast_ms": t * 1e3, "ray_steps": int(r[2].sum().item()),
               "hits": int((r[1] > 0).sum().item()), "boxes_per_s": nb / tb, "classify_ms": tb * 1e3,
               "flop_per_box": fl, "achieved_tflops": tf}
        if products == '3xtf32':
            row["tensor_tflops"] = 3 * tf
            row["roofline"] = {"bound": "tensor", "achieved": 3 * tf, "peak": tf32_peak, "unit": "TFLOP/s",
                               "frac": 3 * tf / tf32_peak, "peak_source": TF32_PEAK_SOURCE}
        else:
            row["roofline"] = {"bound": "fp32", "achieved": tf, "peak": peak32, "unit": "TFLOP/s", "frac": tf / peak32,
                               "peak_source": FP32_PEAK_SOURCE}
        out[name] = row
    out["value"] = out["affine_truncate256_3xtf32"]["rays_per_s"]
    out["tensor_vs_fp32_classify"] = out["affine_truncate256_3xtf32"]["boxes_per_s"] / \
        out["affine_truncate256_fp32"]["boxes_per_s"]
    print(json.dumps(out))


def run_batched(args):
    """Batched config: 512 MLPs (widths U{16..128}, depths U{2..6}, ReLU or TanH),
    64-4096 closest-point queries each, eps 1e-3, all in one persistent launch; compared
    with one single-model persistent launch per model.  On untrained networks a query
    may need millions of nodes, so both forms stop a query after --node-budget nodes
    (its best candidate so far is an upper bound) and do the same work."""
    import torch
    niq = importlib.import_module(PKG)
    n_models = args.n_models
    t0 = time.perf_counter()
    models = niq.workloads.batched_models(n_models)
    qs = niq.workloads.batched_queries(n_models)
    t_gen = time.perf_counter() - t0
    f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(models[0], 'affine_fixed', conservative=True)
    table = niq.batched.ModelTable(models)
    counts = np.array([len(q) for q in qs], np.int64)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    allq = torch.from_numpy(np.concatenate(qs)).cuda()
    lo, hi = np.full(3, -1.2, np.float32), np.full(3, 1.2, np.float32)
    jm = np.arange(n_models, dtype=np.int32)

    status = torch.zeros(1, dtype=torch.int32, device='cuda')

    def batched_step():
        return niq.batched.closest_point_packed(f, table, jm, offs, counts, allq, lo, hi, 1e-3, status=status,
                                                node_budget=args.node_budget)
    # launch parameters picked by the autotuner (untimed) on a sample of the models: each
    # candidate is one full pass, and a pass over all 512 models takes tens of seconds
    nt = min(n_models, 64)
    tuned, tune_ms = niq.autotune.tune_batched(f, table, jm[:nt], offs[:nt], counts[:nt], allq, lo, hi, 1e-3,
                                               node_budget=args.node_budget, reps=1, use_cache=False)
    for _ in range(args.warmup):
        d, l_ = batched_step()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        d, l_ = batched_step()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t_b = sum(times) / len(times)
    budget_hit = int(status.item()) == niq._lib.NIQ_ERR_TIMEOUT
    n_spent, n_nodes = niq.batched.stats()   # of the last timed pass
    # the plain form: one single-model launch per model (same traversal, same budget)
    n_plain = min(n_models, args.plain_models)

    def plain_call(i):
        niq.kd_tree.closest_point(f, table.models[i], lo, hi, allq[offs[i]:offs[i] + counts[i]], eps=1e-3,
                                  persistent=True, node_budget=args.node_budget, strict=False)
    for i in range(min(2, n_plain)):
        plain_call(i)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(n_plain):
        plain_call(i)
    torch.cuda.synchronize()
    t_p = (time.perf_counter() - t0) * n_models / n_plain
    nq = int(counts.sum())
    print(json.dumps({"metric": f"closest-point queries/s ({n_models} MLPs in one launch)", "value": nq / t_b,
                      "unit": "queries/s", "ms": t_b * 1e3, "queries": nq, "models": n_models,
                      "plain_per_model_calls": {"queries_per_s": nq / t_p, "ms_extrapolated": t_p * 1e3,
                                                "models_timed": n_plain},
                      "batched_speedup": t_p / t_b, "node_budget": args.node_budget,
                      "autotuned": tuned, "autotune_ms": tune_ms, "autotune_models": nt,
                      "some_query_spent_budget": budget_hit, "queries_spent_budget": n_spent,
                      "nodes_per_s": n_nodes / t_b, "nodes_per_pass": n_nodes,
                      "fraction_spent_budget": n_spent / max(nq, 1),
                      "note": "a query that spends its node budget keeps its best candidate, an upper bound on "
                              "its distance, not the reference's result",
                      "model_generation_s": t_gen}))


def make_serving_requests(niq, n, rng, max_res=512, max_points=16384, eps=1e-3, node_budget=64):
    """The serving mix: ray tiles (64^2..max_res^2 from a random camera at distance 3),
    closest-point batches (1..max_points points, log-uniform, eps 1e-3, at most
    ``node_budget`` nodes per query: the models are untrained, their bounds loose, and a
    query that spends its budget is answered with its best candidate, an upper bound; the
    bench counts those requests) and pairwise intersection tests under a random rigid
    transform (eps 2e-2): 45% / 45% / 10%."""
    srv = niq.serve
    reqs = []
    sizes = [s for s in (64, 128, 256, 512) if s <= max_res]
    for _ in range(n):
        u = rng.random()
        m = int(rng.integers(64))
        if u < 0.45:
            res = int(rng.choice(sizes))
            eye = rng.standard_normal(3)
            eye = (3.0 * eye / np.linalg.norm(eye)).astype(np.float32)
            look, up, _ = niq.render.look_at(eye)
            roots, dirs = niq.render.generate_camera_rays(eye, look, up, res=res, fov_deg=60.)
            opts = niq.queries.get_default_cast_opts()
            opts['n_max_step'] = 64
            reqs.append(srv.RayRequest(m, roots, dirs, opts))
        elif u < 0.9:
            k = int(np.exp(rng.uniform(0, np.log(max_points))))
            reqs.append(srv.ClosestRequest(m, rng.uniform(-1.2, 1.2, (k, 3)).astype(np.float32), eps=eps,
                                           node_budget=node_budget))
        else:
            R = niq.workloads.random_rotation(rng)
            reqs.append(srv.IntersectRequest(m, int(rng.integers(64)), R,
                                             rng.uniform(-0.5, 0.5, 3).astype(np.float32), eps=2e-2))
    return reqs


def run_serve(args):
    """Served config: 64 resident MLPs (width 32-256, depth 3-8, seeds 100-163), a mixed
    request stream, 40 GB admission budget.  Measures the saturation throughput with a
    closed batch of requests, then Poisson arrivals at fractions of it, and reports
    p50/p99 latency per rate."""
    import torch
    niq = importlib.import_module(PKG)
    models = niq.workloads.serving_models(64)
    rng = np.random.default_rng(7)
    if args.serve_impl == 'native':
        srv = niq.serve.NativeServer(models, n_lanes=args.serve_lanes, slice_rays=16384, slice_queries=512,
                                     lane_scratch_bytes=512 << 20)
    else:
        srv = niq.serve.Server(models, budget_bytes=40 << 30, n_streams=4)
    # warm up every model once (packing, uploads, kernel attributes)
    warm = make_serving_requests(niq, 16, rng, max_res=64, max_points=64)
    for f in [srv.submit(r) for r in warm]:
        f.exception(timeout=600)
    # saturation: everything submitted at once
    sat = make_serving_requests(niq, args.serve_requests, rng, max_res=args.serve_max_res,
                                node_budget=args.serve_node_budget)
    t0 = time.perf_counter()
    futs = [srv.submit(r) for r in sat]
    errors = sum(1 for f in futs if f.exception(timeout=1800) is not None)
    t_sat = time.perf_counter() - t0
    peak = len(sat) / t_sat
    st_sat = srv.stats()
    spent_sat = srv.budget_exhausted
    srv.latencies.clear()
    srv.kind_latencies.clear()
    out = {"metric": "served requests/s and p50/p99 latency (64 resident MLPs, mixed requests)",
           "unit": "requests/s", "saturation": {"requests": len(sat), "seconds": t_sat, "req_per_s": peak,
                                                 "errors": errors, "by_kind": st_sat.get("by_kind"),
                                                 "closest_requests_budget_spent": spent_sat}, "rates": [],
           "config": {"workload": "serving_mix", "impl": args.serve_impl, "lanes": args.serve_lanes,
                      "closest_point": f"eps 1e-3, persistent traversal, {args.serve_node_budget} nodes per query; "
                                       "a request whose query spends the budget is answered with upper bounds "
                                       "and counted",
                      "mix": "45% ray tiles 64^2..512^2, 45% closest-point batches 1..16k points, "
                             "10% intersections under random rigid transforms"}}
    for frac in args.serve_fracs:
        rate = frac * peak
        reqs = make_serving_requests(niq, max(40, int(rate * args.serve_seconds)), rng, max_res=args.serve_max_res,
                                     node_budget=args.serve_node_budget)
        srv.latencies.clear()
        srv.kind_latencies.clear()
        srv.budget_exhausted = 0
        gaps = rng.exponential(1.0 / rate, len(reqs))
        t_start = time.perf_counter()
        t_next = t_start
        futs = []
        for r, gap in zip(reqs, gaps):
            t_next += gap
            dt = t_next - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            futs.append(srv.submit(r))
        errs = sum(1 for f in futs if f.exception(timeout=1800) is not None)
        t_all = time.perf_counter() - t_start
        st = srv.stats()
        out["rates"].append({"fraction_of_peak": frac, "offered_req_per_s": rate, "completed": st.get("completed", 0),
                             "achieved_req_per_s": len(reqs) / t_all, "p50_ms": st.get("p50_ms"),
                             "p99_ms": st.get("p99_ms"), "errors": errs, "by_kind": st.get("by_kind"),
                             "closest_requests_budget_spent": srv.budget_exhausted})
    srv.close()
    seventy = [r for r in out["rates"] if abs(r["fraction_of_peak"] - 0.7) < 1e-6]
    out["value"] = peak
    out["p99_ms_at_70pct"] = seventy[0]["p99_ms"] if seventy else None
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--config', default='tree', choices=['tree', 'rays', 'batched', 'serve', 'precision'])
    ap.add_argument('--serve-requests', type=int, default=200)
    ap.add_argument('--serve-seconds', type=float, default=10.0)
    ap.add_argument('--serve-max-res', type=int, default=512)
    ap.add_argument('--serve-fracs', type=float, nargs='+', default=[0.3, 0.5, 0.7, 0.9])
    ap.add_argument('--serve-impl', default='native', choices=['native', 'python'],
                    help='the native serving runtime (niq_batch_submit) or the Python scheduler')
    ap.add_argument('--serve-lanes', type=int, default=8)
    ap.add_argument('--serve-node-budget', type=int, default=64,
                    help='closest-point nodes per query in the serving mix (untrained networks: a 16k-point batch '
                         'at eps 1e-3 can need millions of nodes per query without one)')
    ap.add_argument('--n-models', type=int, default=512)
    ap.add_argument('--plain-models', type=int, default=64)
    ap.add_argument('--node-budget', type=int, default=2048,
                    help='closest-point nodes per query in the batched config (both forms)')
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--split-depth', type=int, default=SPLIT_DEPTH, help='bisections of the tree (24: 256^3 leaves)')
    ap.add_argument('--quick', action='store_true', help='timed steps only (for profiler runs)')
    ap.add_argument('--no-extras', action='store_true',
                    help='skip the plain-method ray cast and the precision sample in the default line')
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == 'ours' else args.warmup
    if args.impl == 'reference':
        run_reference(args)
    elif args.config == 'rays':
        run_rays(args)
    elif args.config == 'precision':
        run_precision(args)
    elif args.config == 'batched':
        run_batched(args)
    elif args.config == 'serve':
        run_serve(args)
    else:
        run_ours(args)


if __name__ == '__main__':
    main()
