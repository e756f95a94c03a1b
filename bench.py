#!/usr/bin/env python3
"""Benchmark of the ten open-earth-benchmarks stencils on GB300.

Workload (one "step"): each of the ten stencils once, FP64, on a 128 x 128 x 80 interior with
a 3-cell halo -- the all-ten-kernels configuration of the reference benchmark -- with seeded
synthetic inputs (fields.py, workload "physical", seed 1).  Metric: grid-point updates per
second over the ten kernels (10 x 1,310,720 interior points per step), in GPts/s.

* ``value``        device-resident inputs, CUDA events around K steps on the launch stream.
                   The ten stencils are independent: a step forks them onto ten streams and
                   joins them, replayed as one CUDA graph per input set.  Two input sets
                   (1.65 GB) alternate between steps; one step reads 827 MB of distinct
                   fields, so no kernel finds its inputs in the 129 MB L2.  ``sequential``:
                   the same step one stencil after another, which gives the per-kernel times.
* ``e2e``          the same step through the host entry points (oeb_<k>_f64_host) on pinned
                   host buffers, asynchronous (oeb_set_host_async): every call copies its
                   inputs in and its outputs out, pipelined across the ten calls; the step
                   ends when all outputs are in host memory.
* ``roofline``     the kernel with the largest share of the step: algorithmic bytes per
                   launch / its CUDA-event duration, against the measured HBM copy bandwidth.
* ``cpu_baseline`` the oracle's restatement of the reference OpenMP kernels on this host's
                   cores (bounded sample), rank 0 only.

``--impl reference`` times the reference's CPU implementation of the step instead (the
oracle restatement, OpenMP on all host cores; the reference's own headers are compiled
only where its source tree exists, which is not the GPU host) and prints its JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402

NX, NY, NZ, HALO, SEED = 128, 128, 80, 3, 1
WORKLOAD = "ten stencils FP64, 128x128x80 interior + 3-cell halo, physical inputs seed 1"
METRIC = "GPts/s (grid-point updates/s over the ten stencils)"
FALLBACK_HBM_GBS = 6800.0


def _measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def _dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _max_over_ranks(torch, ms, dev):
    """The largest of every rank's `ms` (every rank calls it; without a process group, `ms`)."""
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([float(ms)], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _replica_gpts(world, points_per_step, steps, ms_total):
    """Whole-job GPts/s: each rank runs the step on its own GPU and its own inputs (replicas,
    no collective in the data path), so the job updates world x points_per_step a step, over
    the slowest rank's time."""
    return world * points_per_step * steps / (ms_total * 1e-3) / 1e9


class ClockSampler:
    """SM clocks and clock-event reasons sampled over the timed region.

    NVML (libnvidia-ml, read-only queries) is polled every 2 ms from a thread between
    start() and stop(), so even a timed region of a few tens of ms gets a record; where
    NVML cannot be loaded, nvidia-smi samples every 200 ms instead.
    """

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason bits (nvml.h)
    REASON_BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
                   "hw_thermal_slowdown": 0x40}
    PERIOD_S = 0.002

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.samples = []  # (sm_mhz, max_mhz, reason bits) from NVML
        self.source = None
        self._nvml = None
        self._stop = threading.Event()
        self._t = None

    def _open_nvml(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        handle = ctypes.c_void_p()
        rc = 1
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.gpu)
            bus = "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
            rc = lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(handle))
        except Exception:
            rc = 1
        if rc != 0:
            rc = lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.gpu), ctypes.byref(handle))
        if rc != 0:
            raise RuntimeError("no NVML handle")
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        clk, mx, bits = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()

        def read():
            if lib.nvmlDeviceGetClockInfo(handle, 1, ctypes.byref(clk)) != 0:  # NVML_CLOCK_SM
                return None
            lib.nvmlDeviceGetMaxClockInfo(handle, 1, ctypes.byref(mx))
            if reasons(handle, ctypes.byref(bits)) != 0:
                bits.value = 0
            return float(clk.value), float(mx.value), int(bits.value)

        if read() is None:
            raise RuntimeError("NVML clock query failed")
        return read

    def _poll(self):
        while True:
            r = self._nvml()
            if r is not None:
                self.samples.append(r)
            if self._stop.wait(self.PERIOD_S):
                break

    def start(self):
        """Begins sampling (call just before the timed region)."""
        try:
            if self._nvml is None:
                self._nvml = self._open_nvml()
            self.source = "nvml"
            self._stop.clear()
            self._t = threading.Thread(target=self._poll, daemon=True)
            self._t.start()
            return
        except Exception:
            self._nvml = None
        try:
            self.source = "nvidia-smi"
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def stop(self):
        """Ends sampling (call right after the timed region's synchronize)."""
        if self.source == "nvml" and self._t is not None:
            self._stop.set()
            self._t.join(timeout=5)
            self._t = None
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.proc = None

    def __enter__(self):
        self.start()
        return self

    def __exit__(self, *exc):
        self.stop()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def summary(self):
        sm, mx, reasons = [], [], set()
        for c, m, b in self.samples:
            sm.append(c)
            mx.append(m)
            reasons.update(n for n, bit in self.REASON_BITS.items() if b & bit)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock query unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "sm_min_mhz": min(sm),
                "reasons": sorted(reasons), "samples": len(sm), "source": self.source,
                "window": "timed region only"}


def _make_set(pkg, fields, torch, dev, seed, names, pinned=False, dtype=np.float64, shape=None, workload="physical"):
    """Per kernel: (field Storages, scalars), every field a separate allocation."""
    nx, ny, nz = shape or (NX, NY, NZ)
    out = {}
    for name in names:
        inputs = fields.make_inputs(name, nx, ny, nz, seed=seed, workload=workload)
        outs = fields.make_outputs(name, nx, ny, nz)
        st = {}
        for k, v in {**inputs, **outs}.items():
            t = torch.from_numpy(v.astype(dtype))
            if dev is not None:
                t = t.to(dev)
            elif pinned:
                t = t.pin_memory()
            st[k] = pkg.Storage(t, HALO)
        sc = fields.make_scalars(name, seed=seed)
        if dtype == np.float32:
            sc = {k: (v if k == "dt5" else float(np.float32(v))) for k, v in sc.items()}
        out[name] = (st, sc)
    return out


def _time_steps(pkg, torch, sets, names, steps, warmup, stream, dom, clocks=None):
    """Runs warm-up steps, then `steps` timed steps; returns total ms, per-kernel mean ms, launches."""
    lib = pkg.load_library()

    def step(s, ev=None):
        for idx, name in enumerate(names):
            st, sc = s[name]
            if ev is not None:
                ev[idx][0].record(stream)
            pkg.call(name, st, sc, domain=dom, stream=stream)
            if ev is not None:
                ev[idx][1].record(stream)

    for w in range(warmup):
        step(sets[w % len(sets)])
    torch.cuda.synchronize()
    evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in names]
           for _ in range(steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    launches0 = lib.oeb_launch_count()
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.start()
    t0.record(stream)
    for s in range(steps):
        step(sets[s % len(sets)], evs[s])
    t1.record(stream)
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.stop()
    launches = lib.oeb_launch_count() - launches0
    per_kernel = {name: statistics.mean(evs[s][idx][0].elapsed_time(evs[s][idx][1]) for s in range(steps))
                  for idx, name in enumerate(names)}
    return t0.elapsed_time(t1), per_kernel, launches


def _time_concurrent(pkg, torch, sets, names, steps, warmup, dom, dev, clocks=None, ms_each=None):
    """The step with its independent stencils forked onto one stream each and joined again,
    captured as one CUDA graph per input set (oeb_graph_*) and replayed: `warmup` untimed
    replays, then `steps` replays between CUDA events on the launch stream.  With `ms_each`
    (a time per stencil) the longest stencil is issued first, then the next longest, so the
    step does not end on a long kernel started last.  Returns total ms, kernels launched in
    the timed region, and kernels per graph."""
    if ms_each:
        names = sorted(names, key=lambda n: -ms_each[n])
    import importlib
    chain = importlib.import_module("oeb_gb300.chain")
    lib = pkg.load_library()
    main = torch.cuda.Stream(device=dev)
    streams = [torch.cuda.Stream(device=dev) for _ in names]
    graphs = []
    for s in sets:
        g = chain.Graph(main)
        with g:
            fork = torch.cuda.Event()
            fork.record(main)
            for k, name in enumerate(names):
                streams[k].wait_event(fork)
                st, sc = s[name]
                pkg.call(name, st, sc, domain=dom, stream=streams[k])
            for k in range(len(names)):
                join = torch.cuda.Event()
                join.record(streams[k])
                main.wait_event(join)
        graphs.append(g)
    for w in range(warmup):
        graphs[w % len(graphs)].launch(main)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    launches0 = lib.oeb_launch_count()
    if clocks is not None:
        clocks.start()
    t0.record(main)
    for s in range(steps):
        graphs[s % len(graphs)].launch(main)
    t1.record(main)
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.stop()
    launches = lib.oeb_launch_count() - launches0
    kernels = graphs[0].kernels
    for g in graphs:
        g.close()
    return t0.elapsed_time(t1), launches, kernels


L2_BYTES = 129 * 1000 * 1000  # GB300 L2


def _time_isolated(pkg, torch, dev, st_sc, name, dom, steps, warmup):
    """One stencil alone, as its average launch duration: copies of its fields (separate
    allocations, so that no launch finds its inputs in L2) are made until they span twice the
    L2, one launch per copy is captured in a CUDA graph, and the graph is replayed between
    CUDA events on the launch stream.  Returns ms per launch, copies, timed launches."""
    import importlib
    chain = importlib.import_module("oeb_gb300.chain")
    st, sc = st_sc
    set_bytes = sum(v.data.numel() * v.data.element_size() for v in st.values())
    copies = max(2, -(-2 * L2_BYTES // set_bytes))
    sets = [st] + [{k: pkg.Storage(v.data.clone(), v.halo, nx=v.szi - 2 * v.halo if v.rank == 3 else None)
                    for k, v in st.items()} for _ in range(copies - 1)]
    main = torch.cuda.Stream(device=dev)
    g = chain.Graph(main)
    with g:
        for s in sets:
            pkg.call(name, s, sc, domain=dom, stream=main)
    reps = max(3, -(-steps // copies))
    for _ in range(max(warmup, 1)):
        g.launch(main)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(main)
    for _ in range(reps):
        g.launch(main)
    t1.record(main)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / (reps * copies)
    g.close()
    del sets
    return ms, copies, reps * copies


def _algorithmic_bytes(pkg, name, elem=8):
    return pkg.KERNELS[name].bytes_per_point(elem) * NX * NY * NZ


def _config(names, world):
    """The workload description both arms print (ours and --impl reference), so that the two
    lines name the same configuration."""
    return {"workload": WORKLOAD, "kernels": list(names), "interior": [NX, NY, NZ], "halo": HALO,
            "points_per_step": len(names) * NX * NY * NZ,
            "l2": "inputs larger than L2: two 827 MB input sets alternate between steps",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def run_ours(args):
    import torch
    rank, world, local = _dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pkg = graft.load_package()
    import importlib
    fields = importlib.import_module("oeb_gb300.fields")
    lib = pkg.load_library()
    names = [k for k in pkg.KERNELS if not args.kernels or k in args.kernels]
    sets = [_make_set(pkg, fields, torch, dev, SEED + r, names) for r in range(2)]
    stream = torch.cuda.current_stream(dev)
    dom = (NX, NY, NZ)
    if world > 1:
        torch.distributed.barrier()
    # sequential pass: per-kernel CUDA-event times (shares, roofline)
    ms_seq, per_kernel, launches_seq = _time_steps(pkg, torch, sets, names, args.steps, args.warmup, stream, dom)
    # the step: the ten stencils are independent, so they are issued on ten streams and
    # replayed as one CUDA graph per input set
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    ms_total, launches, graph_kernels = _time_concurrent(pkg, torch, sets, names, args.steps, args.warmup, dom, dev,
                                                         clocks, ms_each=per_kernel)
    ms_total = _max_over_ranks(torch, ms_total, dev)
    ms_seq = _max_over_ranks(torch, ms_seq, dev)
    if world > 1:
        torch.distributed.barrier()
    ms_step = ms_total / args.steps
    clock_summary = clocks.summary()
    pts_step = len(names) * NX * NY * NZ
    value = _replica_gpts(world, pts_step, args.steps, ms_total)
    total_k = sum(per_kernel.values())
    dom_k = max(per_kernel, key=per_kernel.get)
    peak, peak_src = _measured_peak()
    # each stencil alone: its average launch duration over back-to-back launches (graph)
    iso = {k: _time_isolated(pkg, torch, dev, sets[0][k], k, dom, args.steps, args.warmup) for k in names}
    iso_ms = {k: v[0] for k, v in iso.items()}
    add_rate, add_rate_clocks = _fp64_add_rate(pkg, local)
    achieved = _algorithmic_bytes(pkg, dom_k) / (iso_ms[dom_k] * 1e-3) / 1e9
    traffic = _ncu_traffic(dom_k)

    del sets
    torch.cuda.empty_cache()
    # end to end, measured before the other legs fill device memory (the 27 GB batch plan)
    e2e = None
    if not args.no_e2e:
        e2e = _e2e(pkg, fields, torch, args, names)
    f32 = None
    if not args.no_f32:
        sets32 = [_make_set(pkg, fields, torch, dev, SEED + r, names, dtype=np.float32) for r in range(2)]
        ms32, pk32, l32 = _time_steps(pkg, torch, sets32, names, args.steps, args.warmup, stream, dom)
        ms32c, l32c, _ = _time_concurrent(pkg, torch, sets32, names, args.steps, args.warmup, dom, dev, ms_each=pk32)
        sets32_first = sets32[0]
        del sets32
        torch.cuda.empty_cache()
        # configuration 3: FP32 at 256 x 256 x 80 with steep fronts (seed 2)
        big = (256, 256, 80)
        sets3 = [_make_set(pkg, fields, torch, dev, 2 + r, names, dtype=np.float32, shape=big, workload="fronts")
                 for r in range(2)]
        ms3, pk3, _ = _time_steps(pkg, torch, sets3, names, args.steps, args.warmup, stream, big)
        ms3c, _, _ = _time_concurrent(pkg, torch, sets3, names, args.steps, args.warmup, big, dev, ms_each=pk3)
        iso3 = {k: _time_isolated(pkg, torch, dev, sets3[0][k], k, big, args.steps, args.warmup)[0] for k in names}
        iso32 = {k: _time_isolated(pkg, torch, dev, sets32_first[k], k, dom, args.steps, args.warmup)[0]
                 for k in names}
        del sets32_first
        del sets3
        torch.cuda.empty_cache()
        pts3 = big[0] * big[1] * big[2]
        by3 = {k: pkg.KERNELS[k].bytes_per_point(4) * pts3 for k in names}
        d32 = max(pk32, key=pk32.get)
        ach32 = _algorithmic_bytes(pkg, d32, 4) / (pk32[d32] * 1e-3) / 1e9
        step_bytes32 = sum(_algorithmic_bytes(pkg, k, 4) for k in names)
        f32 = {"value": round(pts_step * args.steps / (ms32c * 1e-3) / 1e9, 4), "unit": "GPts/s",
               "ms_per_step": round(ms32c / args.steps, 4), "speedup_vs_f64": round(ms_total / ms32c, 3),
               "step_hbm_gbs": round(step_bytes32 / (ms32c / args.steps * 1e-3) / 1e9, 1),
               "issue": "as the FP64 step: the ten stencils on ten streams, one CUDA graph per input set",
               "sequential": {"value": round(pts_step * args.steps / (ms32 * 1e-3) / 1e9, 4),
                              "ms_per_step": round(ms32 / args.steps, 4),
                              "speedup_vs_f64_sequential": round(ms_seq / ms32, 3),
                              "step_hbm_gbs": round(step_bytes32 / (ms32 / args.steps * 1e-3) / 1e9, 1)},
               "roofline": {"bound": "hbm", "kernel": d32, "achieved": round(ach32, 2), "peak": _measured_peak()[0],
                            "unit": "GB/s", "frac": round(ach32 / _measured_peak()[0], 4)},
               "per_kernel_ms": {k: round(v, 5) for k, v in pk32.items()},
               "per_kernel_gbs": {k: round(_algorithmic_bytes(pkg, k, 4) / (v * 1e-3) / 1e9, 1)
                                  for k, v in pk32.items()},
               "gpu_launches": int(l32c),
               "config3_256x256x80_fronts": {
                   "value": round(len(names) * pts3 * args.steps / (ms3c * 1e-3) / 1e9, 4), "unit": "GPts/s",
                   "ms_per_step": round(ms3c / args.steps, 4),
                   "step_hbm_gbs": round(sum(by3.values()) / (ms3c / args.steps * 1e-3) / 1e9, 1),
                   "sequential": {"value": round(len(names) * pts3 * args.steps / (ms3 * 1e-3) / 1e9, 4),
                                  "ms_per_step": round(ms3 / args.steps, 4),
                                  "step_hbm_gbs": round(sum(by3.values()) / (ms3 / args.steps * 1e-3) / 1e9, 1)},
                   "per_kernel_ms": {k: round(v, 5) for k, v in pk3.items()},
                   "per_kernel_gbs": {k: round(by3[k] / (v * 1e-3) / 1e9, 1) for k, v in pk3.items()},
                   "per_kernel_frac": {k: round(by3[k] / (v * 1e-3) / 1e9 / _measured_peak()[0], 4)
                                       for k, v in pk3.items()},
                   "per_kernel_isolated_ms": {k: round(v, 5) for k, v in iso3.items()},
                   "per_kernel_isolated_frac": {k: round(by3[k] / (v * 1e-3) / 1e9 / _measured_peak()[0], 4)
                                                for k, v in iso3.items()},
                   "isolated_how": "each stencil alone, average over back-to-back launches from a CUDA graph "
                                   "over copies of its fields spanning twice the L2"},
               "per_kernel_isolated_ms": {k: round(v, 5) for k, v in iso32.items()},
               "per_kernel_isolated_frac": {k: round(_algorithmic_bytes(pkg, k, 4) / (v * 1e-3) / 1e9 /
                                                     _measured_peak()[0], 4) for k, v in iso32.items()},
               "note": "FP32 storage and arithmetic, exact limiter sign tests, error-free pressure-gradient products; "
                       "normwise error vs the FP64 oracle is stated per kernel by tests/test_gpu_fp32.py"}

    adjoint = None
    if not args.no_adjoint:
        adjoint = {"workload": "forward + adjoint of each of the ten stencils, 128x128x80 + 3-cell halo, seed 3 "
                               "(FP32 also at 256x256x80)",
                   "f64": _adjoint_leg(pkg, fields, torch, dev, args, np.float64),
                   "f32": _adjoint_leg(pkg, fields, torch, dev, args, np.float32),
                   "f32_256x256x80": _adjoint_leg(pkg, fields, torch, dev, args, np.float32, shape=(256, 256, 80))}
    chain = None
    if not args.no_chain:
        chain = {"workload": "chained step fastwavesuv->hadvuv5th->update->hdiffsmag->fvtp2d, forward + adjoint "
                             "with recomputation, one CUDA graph per step, 128x128x80, i/j halo 8, seed 3",
                 "f64": _chain_leg(pkg, fields, torch, dev, args, np.float64),
                 "f32": _chain_leg(pkg, fields, torch, dev, args, np.float32)}

    batched = None
    if not args.no_batch:
        batched = _batch_leg(pkg, fields, torch, dev, args)
    _chain_roofs(chain, batched, add_rate, peak)


    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "GPts/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; fields.py 'physical')",
        "config": _config(names, world),
        "issue": "the ten stencils are independent: each step forks them onto ten streams and joins them "
                 "(events), captured once per input set as a CUDA graph of %d kernels and replayed" % graph_kernels,
        "roofline": {"bound": "hbm", "kernel": dom_k, "achieved": round(achieved, 2), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": _algorithmic_bytes(pkg, dom_k),
                     "launch_ms": round(iso_ms[dom_k], 5),
                     "launch_ms_how": "average over %d back-to-back launches of %s alone (CUDA graph over %d "
                                      "copies of its fields spanning twice the L2), CUDA events on the launch "
                                      "stream" % (iso[dom_k][2], dom_k, iso[dom_k][1]),
                     "launch_ms_sequential_pass": round(per_kernel[dom_k], 5),
                     "fp64_pipe_active_pct": _ncu_summary(dom_k, "fp64_pipe_active_pct"),
                     "alu_pipe_active_pct": _ncu_summary(dom_k, "alu_pipe_active_pct"),
                     "fp64_pipe_roof": _fp64_pipe_roofline(names, iso_ms, dom_k, ms_step, clock_summary,
                                                           torch.cuda.get_device_properties(dev).multi_processor_count,
                                                           add_rate, add_rate_clocks),
                     "fp64_op_rates": _fp64_op_rates(pkg, torch.cuda.get_device_properties(dev).multi_processor_count,
                                                     (add_rate_clocks or {}).get("sm_mhz")),
                     "note": "the FP64 stencils are compute-bound, not HBM-bound: GB300 issues 1.6 FP64 "
                             "op/clk/SM, so the kernels run as F64i (exact integer-pipe multiply, divide, "
                             "sqrt, compare beside FP64-pipe adds); the pipe figures are ncu's "
                             "sm__pipe_fp64_cycles_active and sm__inst_executed_pipe_alu for this kernel"},
        "per_kernel_ms": {k: round(v, 5) for k, v in per_kernel.items()},
        "per_kernel_gbs": {k: round(_algorithmic_bytes(pkg, k) / (v * 1e-3) / 1e9, 1) for k, v in per_kernel.items()},
        "per_kernel_isolated_ms": {k: round(v, 5) for k, v in iso_ms.items()},
        "per_kernel_isolated_frac": {k: round(_algorithmic_bytes(pkg, k) / (v * 1e-3) / 1e9 / peak, 4)
                                     for k, v in iso_ms.items()},
        "kernel_share": {k: round(v / total_k, 4) for k, v in per_kernel.items()},
        "clocks": clock_summary,
        "gpu_launches": int(launches),
        "sequential": {"value": round(_replica_gpts(world, pts_step, args.steps, ms_seq), 4),
                       "ms_per_step": round(ms_seq / args.steps, 4), "gpu_launches": int(launches_seq),
                       "issue": "the ten stencils one after another on one stream, a CUDA event pair around each "
                                "(per_kernel_ms, kernel_share and roofline come from this pass)"},
    }
    if e2e is not None:
        line["e2e"] = e2e
    if f32 is not None:
        line["f32"] = f32
    if adjoint is not None:
        line["adjoint"] = adjoint
    if chain is not None:
        line["chain"] = chain
    if batched is not None:
        line["batched"] = batched
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = _cpu_baseline(pkg, fields, budget_s=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# configuration 4's four adjoints first, then the other six stencils' adjoints
ADJ_KERNELS = ("hdiffsmag", "hadvuv5th", "fastwavesuv", "fvtp2d", "laplace", "hdiffsa", "hadvuv", "uvbke", "nh_p_grad",
               "p_grad_c")


def _queue_behind_sleep(torch, stream, ms):
    """Enqueues on `stream` a kernel that spins for about `ms` milliseconds (at 2.07 GHz; longer
    at lower clocks), so that the calls the host enqueues next are all queued before the GPU
    reaches them: CUDA events between those calls then time the device, not the host's
    dispatch of each call."""
    with torch.cuda.stream(stream):
        torch.cuda._sleep(int(ms * 2.07e6))


def _adjoint_leg(pkg, fields, torch, dev, args, dtype, shape=(NX, NY, NZ)):
    """Forward + adjoint pairs of the ten stencils at `shape` (128x128x80 by default, seed 3):
    per kernel, the forward call and the adjoint call timed with CUDA events on the launch
    stream, two input sets alternating.  The timed calls are queued behind a sleep kernel
    (`_queue_behind_sleep`) long enough for the host to enqueue them all, so the events time
    the device even where a call's kernels are shorter than its host-side dispatch."""
    elem = 8 if dtype == np.float64 else 4
    stream = torch.cuda.current_stream(dev)
    dom = tuple(shape)
    nx, ny, nz = dom
    pts = nx * ny * nz
    peak = _measured_peak()[0]
    lib = pkg.load_library()
    out = {}
    for name in ADJ_KERNELS:
        spec = pkg.KERNELS[name]
        sets = []
        for r in range(2):
            x = fields.make_inputs(name, nx, ny, nz, seed=3 + r)
            o = fields.make_outputs(name, nx, ny, nz)
            st = {k: pkg.Storage(torch.from_numpy(v.astype(dtype)).to(dev), HALO) for k, v in {**x, **o}.items()}
            rng = np.random.default_rng([3, r])
            shape = next(iter(o.values())).shape
            yb = {n: pkg.Storage(torch.from_numpy(rng.normal(0.0, 1.0, size=shape).astype(dtype)).to(dev), HALO)
                  for n in spec.semantic_outputs}
            xb = {n: pkg.Storage(torch.zeros(shape, dtype=st[n].data.dtype, device=dev), HALO)
                  for n in pkg.ACTIVE[name]}
            sc = fields.make_scalars(name, seed=3)
            if dtype == np.float32:
                sc = {k: float(np.float32(v)) for k, v in sc.items()}
            sets.append((st, yb, xb, sc))

        def run(sv, ev=None):
            st, yb, xb, sc = sv
            if ev is not None:
                ev[0].record(stream)
            pkg.call(name, st, sc, domain=dom, stream=stream)
            if ev is not None:
                ev[1].record(stream)
            pkg.adjoint(name, st, yb, xb, sc, domain=dom, stream=stream)
            if ev is not None:
                ev[2].record(stream)

        torch.cuda.synchronize()
        t = time.perf_counter()
        for w in range(args.warmup):
            run(sets[w % 2])
        host_ms = (time.perf_counter() - t) * 1e3 / max(args.warmup, 1)
        torch.cuda.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
        l0 = lib.oeb_launch_count()
        _queue_behind_sleep(torch, stream, 3.0 * host_ms * args.steps + 2.0)
        for i in range(args.steps):
            run(sets[i % 2], evs[i])
        torch.cuda.synchronize()
        launches = lib.oeb_launch_count() - l0
        fwd = statistics.mean(e[0].elapsed_time(e[1]) for e in evs)
        adj = statistics.mean(e[1].elapsed_time(e[2]) for e in evs)
        fwd_b = spec.bytes_per_point(elem) * pts
        adj_b = len(pkg.ADJ_FIELDS[name]) * elem * pts
        pair_gbs = (fwd_b + adj_b) / ((fwd + adj) * 1e-3) / 1e9
        out[name] = {"forward_ms": round(fwd, 5), "adjoint_ms": round(adj, 5),
                     "pair_gpts": round(pts / ((fwd + adj) * 1e-3) / 1e9, 4),
                     "pair_bytes_per_point": (spec.bytes_per_point(elem) + len(pkg.ADJ_FIELDS[name]) * elem),
                     "pair_hbm_gbs": round(pair_gbs, 1), "pair_frac": round(pair_gbs / peak, 4),
                     "adjoint_hbm_gbs": round(adj_b / (adj * 1e-3) / 1e9, 1),
                     "launches_per_pair": round(launches / args.steps, 2)}
        del sets
        torch.cuda.empty_cache()
    return out


def _chain_leg(pkg, fields, torch, dev, args, dtype):
    """The chained step in both fusion groupings: hadvuv5th fused with the update (the
    library's default, the line's figures) and separate kernels (``separate``)."""
    import ctypes
    lib = pkg.load_library()
    lib.oeb_set_fusion(ctypes.c_int(1))
    res = _chain_leg_grouping(pkg, fields, torch, dev, args, dtype)
    res["grouping"] = "hadvuv5th and the update as one kernel (OEB_FUSE_HADV_UPDATE, the default)"
    lib.oeb_set_fusion(ctypes.c_int(0))
    try:
        sep = _chain_leg_grouping(pkg, fields, torch, dev, args, dtype)
    finally:
        lib.oeb_set_fusion(ctypes.c_int(1))
    res["separate"] = {"grouping": "every stage its own kernels (oeb_set_fusion(0))",
                       **{k: sep[k] for k in ("ms_per_step", "gpts", "kernels_per_step", "launches_per_step")},
                       "fused_speedup": round(sep["ms_per_step"] / res["ms_per_step"], 3)}
    return res


def _chain_leg_grouping(pkg, fields, torch, dev, args, dtype):
    """The chained dycore step forward + adjoint at 128x128x80 (i/j halo 8, seed 3), captured
    once per input set in a CUDA graph; two graphs on two input sets alternate."""
    import importlib
    chain = importlib.import_module("oeb_gb300.chain")
    stream = torch.cuda.Stream(device=dev)
    H = fields.CHAIN_HALO
    graphs, keep = [], []
    for r in range(2):
        x = fields.make_chain_inputs(NX, NY, NZ, 3 + r, halo=H)
        sc = fields.make_chain_scalars(3)
        st = {k: pkg.Storage(torch.from_numpy(v.astype(dtype)).to(dev), H, nx=NX if v.ndim == 3 else None)
              for k, v in x.items()}
        shape = x["u"].shape
        tdt = torch.float64 if dtype == np.float64 else torch.float32
        outs = {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=NX) for n in chain.OUTPUTS}
        rng = np.random.default_rng([3, r])
        seeds = {n: pkg.Storage(torch.from_numpy(rng.normal(0.0, 1.0, size=shape).astype(dtype)).to(dev), H, nx=NX)
                 for n in chain.OUTPUTS}
        grads = {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=NX) for n in ("u", "v")}
        plan = chain.ChainPlan(st["u"], (NX, NY, NZ), chain.FORWARD | chain.ADJOINT)
        with torch.cuda.stream(stream):
            plan.forward(st, sc, outs, stream=stream)
            plan.adjoint(st, sc, seeds, grads, stream=stream)
        stream.synchronize()
        g = chain.Graph(stream)
        with g:
            plan.forward(st, sc, outs, stream=stream)
            plan.adjoint(st, sc, seeds, grads, stream=stream)
        graphs.append(g)
        keep.append((st, outs, seeds, grads, plan))
    for w in range(args.warmup):
        graphs[w % 2].launch(stream)
    stream.synchronize()
    lib = pkg.load_library()
    l0 = lib.oeb_launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for i in range(args.steps):
        graphs[i % 2].launch(stream)
    t1.record(stream)
    stream.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    launches = (lib.oeb_launch_count() - l0) / args.steps
    res = {"ms_per_step": round(ms, 4), "gpts": round(NX * NY * NZ / (ms * 1e-3) / 1e9, 4),
           "kernels_per_step": graphs[0].kernels, "launches_per_step": round(launches, 1),
           "workspace_bytes": keep[0][4].nbytes}
    for g in graphs:
        g.close()
    for k in keep:
        k[4].close()
    del keep
    torch.cuda.empty_cache()
    return res


def _batch_leg(pkg, fields, torch, dev, args):
    """The uneven ensemble (48 members, nx, ny in {48..320}, nz in {40, 60, 80, 137}, FP64 or
    FP32, seed 4): every member's chained step forward + adjoint as batched persistent
    launches (autotuned), replayed from a CUDA graph; beside it the same work as per-member
    launches, also from a graph."""
    import importlib
    chain = importlib.import_module("oeb_gb300.chain")
    H = fields.CHAIN_HALO
    spec = fields.ensemble_members(48, 4)
    members = []
    for idx, (nx, ny, nz, item) in enumerate(spec):
        dt = np.float64 if item == 8 else np.float32
        x = fields.make_chain_inputs_device(nx, ny, nz, 4000 + idx, dev, dt, halo=H)
        shape = tuple(x["u"].shape)
        tdt = x["u"].dtype
        gen = torch.Generator(device=dev).manual_seed(idx)
        members.append({
            "fields": {k: pkg.Storage(v, H, nx=nx if v.dim() == 3 else None) for k, v in x.items()},
            "scalars": fields.make_chain_scalars(4), "domain": (nx, ny, nz),
            "outs": {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=nx) for n in chain.OUTPUTS},
            "seeds": {n: pkg.Storage(torch.randn(shape, generator=gen, device=dev, dtype=tdt), H, nx=nx)
                      for n in chain.OUTPUTS},
            "grads": {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=nx) for n in ("u", "v")}})
    stream = torch.cuda.Stream(device=dev)
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    plan.run(stream)
    stream.synchronize()
    t = time.perf_counter()
    plan.autotune(stream)
    stream.synchronize()
    tune_s = time.perf_counter() - t
    plan.run(stream)
    stream.synchronize()

    def timed(graph):
        for _ in range(args.warmup):
            graph.launch(stream)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            graph.launch(stream)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / args.steps

    g = chain.Graph(stream)
    with g:
        plan.run(stream)
    lib = pkg.load_library()
    l0 = lib.oeb_launch_count()
    ms_batch = timed(g)
    launches = (lib.oeb_launch_count() - l0) / (args.steps + args.warmup)
    # the same work as per-member launches
    plans = [chain.ChainPlan(m["fields"]["u"], m["domain"], chain.FORWARD | chain.ADJOINT) for m in members]

    def per_member():
        for cp, m in zip(plans, members):
            cp.forward(m["fields"], m["scalars"], m["outs"], stream=stream)
            cp.adjoint(m["fields"], m["scalars"], m["seeds"], m["grads"], stream=stream)

    per_member()
    stream.synchronize()
    g2 = chain.Graph(stream)
    with g2:
        per_member()
    ms_members = timed(g2)
    # the one-launch form: the whole step of every member in one launch of the step kernel,
    # with each k-blocking its tasks can be recorded with
    one = {}
    for kb in (2, 4):  # (kb 0 and 1 measured slower at every build)
        for per_sm in (2, 3, 4):
            plan.set_form(plan.ONE_LAUNCH, kb, per_sm)
            plan.run(stream)
            stream.synchronize()
            g3 = chain.Graph(stream)
            with g3:
                plan.run(stream)
            l0 = lib.oeb_launch_count()
            ms = timed(g3)
            launches_one = (lib.oeb_launch_count() - l0) / (args.steps + args.warmup)
            status = plan.step_status()
            wait_us, waits = plan.step_waits()  # of the last run
            g3.close()
            one[(kb, per_sm)] = (ms, launches_one, status, wait_us, waits)
    best = min(one, key=lambda k: one[k][0])
    plan.set_form(plan.PER_LAUNCH)
    pts = plan.points
    ms_one = one[best][0]
    ctas = best[1] * torch.cuda.get_device_properties(dev).multi_processor_count
    one_launch = {
        "form": "one persistent launch of the step kernel a run: every member's tasks (its recorded launches, "
                "forward then adjoint) in one ticket order, each waiting on the device for its member's previous task",
        "ms_per_run": round(ms_one, 3), "gpts": round(pts / (ms_one * 1e-3) / 1e9, 4), "kb": best[0],
        "ctas_per_sm": best[1],
        "ms_per_run_by_kb_and_ctas_per_sm": {"%d/%d" % k: round(v[0], 3) for k, v in one.items()},
        "wait_frac_by_kb_and_ctas_per_sm": {
            "%d/%d" % k: round(v[3] * 1e-3 / (v[0] * k[1] * ctas / best[1]), 4) for k, v in one.items()},
        "waits_by_kb_and_ctas_per_sm": {"%d/%d" % k: v[4] for k, v in one.items()},
        "launches_per_run": 1, "launches_counted": round(one[best][1], 1),
        "status_ok": all(v[2] == (0, -1) for v in one.values()),
        "speedup_vs_per_member_launches": round(ms_members / ms_one, 3),
        "speedup_vs_per_launch_form": round(ms_batch / ms_one, 3)}
    res = {"workload": "48 members, nx, ny uniform in {48..320 step 16}, nz in {40, 60, 80, 137}, FP64 or FP32 "
                       "(seed 4); chained step forward + adjoint with recomputation; device-generated inputs",
           "members": len(members), "fp64_members": sum(1 for s_ in spec if s_[3] == 8),
           "fp64_points": sum(a * b * c for a, b, c, e in spec if e == 8),
           "points_per_run": pts, "ms_per_run": round(ms_batch, 3), "gpts": round(pts / (ms_batch * 1e-3) / 1e9, 4),
           "batched_launches_per_run": plan.launches, "launches_counted": round(launches, 1),
           "per_member_launches_ms_per_run": round(ms_members, 3),
           "per_member_launches_per_run": g2.kernels,
           "speedup_vs_per_member_launches": round(ms_members / ms_batch, 3),
           "autotune_s": round(tune_s, 2), "plan_bytes": plan.nbytes,
           "plan_bytes_per_point": round(plan.nbytes / pts, 1),
           "tuned": _tuning_summary(plan.tuning()), "fusion": plan.fusion,
           "one_launch": one_launch}
    g.close()
    g2.close()
    for cp in plans:
        cp.close()
    plan.close()
    del members
    torch.cuda.empty_cache()
    return res


def _tuning_summary(choices):
    """How many of a plan's batched launches the autotuner gave each k-blocking, tile shape
    and launch form."""
    hist = {"kb": {}, "shape": {}, "form": {}}
    names = {"shape": {0: "32x32", 1: "32x8", 2: "64x16"}, "form": {0: "wave", 1: "cta_per_tile", 2: "per_member"}}
    for kb, shape, form in choices:
        for key, v in (("kb", kb), ("shape", shape), ("form", form)):
            label = names.get(key, {}).get(v, str(v))
            hist[key][label] = hist[key].get(label, 0) + 1
    return hist


def _ncu_summary(kernel, key):
    """A figure of `kernel`'s committed ncu summary (profiles/ncu_<kernel>_128x128x80.md)."""
    p = ROOT / "profiles" / ("ncu_%s_128x128x80.md" % kernel)
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith(key + ":"):
            try:
                return float(ln.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


# FP64-pipe thread instructions (DADD / DMUL / DFMA) per clock per SM on the GB300, measured
# by a dependent-free DADD throughput loop: 505 G/s at 2070 MHz on 152 SMs.
PIPE_MIX_PROFILE = "pipe_mix_ten_stencils_f64"


def _fp64_add_rate(pkg, gpu_index):
    """The FP64 pipe's rate on this GPU, measured here (oeb_probe_fp64_add_rate): FP64 additions
    a second over all SMs, the clocks sampled while it ran, and the additions of one launch."""
    import ctypes
    lib = pkg.load_library()
    rate, adds = ctypes.c_double(0.0), ctypes.c_double(0.0)
    with ClockSampler(gpu_index) as clocks:
        st = lib.oeb_probe_fp64_add_rate(ctypes.byref(rate), ctypes.byref(adds))
    return (rate.value if st == 0 else None), clocks.summary()


def _fp64_op_rates(pkg, sms, probe_mhz):
    """Each FP64 operation's rate on this GPU (oeb_probe_fp64_rate), in G operations a
    second and per clock per SM (at the SM clock sampled during the addition probe)."""
    import ctypes
    lib = pkg.load_library()
    out = {}
    for op, name in enumerate(("add", "mul", "fma", "div", "sqrt")):
        r = ctypes.c_double(0.0)
        if lib.oeb_probe_fp64_rate(ctypes.c_int(op), ctypes.byref(r), None) != 0:
            return None
        out[name] = {"gops": round(r.value / 1e9, 2),
                     "per_clk_per_sm": round(r.value / (sms * probe_mhz * 1e6), 3) if probe_mhz else None}
    out["how"] = ("oeb_probe_fp64_rate: 8 independent chains of the operation a thread, 8 CTAs of 256 threads an "
                  "SM, the best of 3 timed launches; div and sqrt are the compiler's IEEE-rounded sequences")
    return out


def _fp64_pipe_roofline(names, per_kernel, dom_k, ms_step, clocks_summary, sms, add_rate, rate_clocks):
    """The FP64 pipe as the roof: each kernel's FP64-pipe instructions per interior point
    (committed ncu counts) x points, over the FP64 addition rate measured on this GPU just
    before (oeb_probe_fp64_add_rate), rescaled by the ratio of the SM clock sampled during the
    timed region to the one sampled during the probe.  For the dominant kernel (iso timing)
    and for the whole concurrent step.  None without the counts or the rate."""
    per_pt = {k: _ncu_summary(PIPE_MIX_PROFILE, "fp64_instr_per_point_" + k) for k in names}
    if not add_rate or any(v is None for v in per_pt.values()):
        return None
    mhz = (clocks_summary or {}).get("sm_mhz")
    probe_mhz = (rate_clocks or {}).get("sm_mhz")
    rate = add_rate * (mhz / probe_mhz if mhz and probe_mhz else 1.0)  # thread instructions / s
    pts = NX * NY * NZ
    k_bound_ms = per_pt[dom_k] * pts / rate * 1e3
    step_bound_ms = sum(per_pt.values()) * pts / rate * 1e3
    per_clk = add_rate / (sms * probe_mhz * 1e6) if probe_mhz else None
    return {"unit": "FP64-pipe instructions", "measured_adds_per_s": round(add_rate, 1),
            "rate_per_clk_per_sm": round(per_clk, 4) if per_clk else None, "probe_sm_mhz": probe_mhz,
            "sms": sms, "sm_mhz": mhz, "kernel": dom_k, "kernel_instr_per_point": per_pt[dom_k],
            "kernel_bound_ms": round(k_bound_ms, 5), "kernel_frac": round(k_bound_ms / per_kernel[dom_k], 4),
            "step_instr_per_point": round(sum(per_pt.values()), 2), "step_bound_ms": round(step_bound_ms, 5),
            "step_frac": round(step_bound_ms / ms_step, 4),
            "source": "rate: oeb_probe_fp64_add_rate (independent __dadd_rn chains on every SM, timed here); "
                      "instructions per point: profiles/ncu_%s_128x128x80.md (ncu sm__inst_executed_pipe_fp64); "
                      "frac = bound / measured (kernel: alone, back-to-back launches; step: the concurrent "
                      "graph)" % PIPE_MIX_PROFILE}


CHAIN_PROFILE = "pipe_chain"


def _chain_roofs(chain, batched, add_rate, peak):
    """Roofline anchors of the chained and batched legs (in place): the FP64 chained step
    against its FP64-pipe bound (FP64-pipe instructions a point from the committed ncu
    counts, over the FP64 addition rate measured in this run), both precisions' DRAM traffic
    (ncu bytes a point) over the measured step time, and the batched run against the
    FP64-pipe bound of its FP64 members' points."""
    instr = _ncu_summary(CHAIN_PROFILE, "fp64_instr_per_point_chain_f64")
    pts = NX * NY * NZ
    src = "profiles/ncu_%s_128x128x80.md" % CHAIN_PROFILE
    if chain is not None:
        for prec in ("f64", "f32"):
            r = chain.get(prec)
            b = _ncu_summary(CHAIN_PROFILE, "dram_bytes_per_point_chain_" + prec)
            if not r or b is None:
                continue
            # the capture is of the step with separate kernels: its bytes over that step's time
            ms = r["separate"]["ms_per_step"] if "separate" in r else r["ms_per_step"]
            gbs = b * pts / (ms * 1e-3) / 1e9
            r["dram"] = {"bytes_per_point": b, "gbs": round(gbs, 1), "frac": round(gbs / peak, 4),
                         "source": src + " (ncu dram__bytes of the step with separate kernels) over this run's "
                                         "time of that step"}
        r = chain.get("f64")
        if r and instr and add_rate:
            bound = instr * pts / add_rate * 1e3
            r["fp64_pipe_roof"] = {"instr_per_point": instr, "bound_ms": round(bound, 4),
                                   "frac": round(bound / r["ms_per_step"], 4),
                                   "source": src + " (ncu sm__inst_executed_pipe_fp64) over the FP64 addition "
                                                   "rate measured in this run"}
    if batched is not None and instr and add_rate and batched.get("fp64_points"):
        bound = instr * batched["fp64_points"] / add_rate * 1e3
        batched["fp64_pipe_roof"] = {
            "instr_per_point": instr, "bound_ms": round(bound, 3), "frac": round(bound / batched["ms_per_run"], 4),
            "note": "the FP64 members' points at the 128x128x80 chained step's FP64-pipe instructions a point "
                    "(smaller members recompute relatively wider halos, so their true count is higher)"}


def _ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if there is one."""
    v = _ncu_summary(kernel, "dram_bytes_per_launch")
    return int(v) if v is not None else None


def _e2e(pkg, fields, torch, args, names):
    """The step through the host entry points with pinned host buffers."""
    hs = _make_set(pkg, fields, torch, None, SEED, names, pinned=True)
    dom = (NX, NY, NZ)
    h2d = d2h = 0
    for name in names:
        spec = pkg.KERNELS[name]
        st, _ = hs[name]
        for a in spec.args:
            if a.role == "in3":
                # the k-planes the kernel reads (-klo .. nz+khi-1, every row of them), rounded out
                # to 64 KB of the field's span as the host entry points copy them
                data = st[a.name].data
                plane, align = data.shape[1] * data.shape[2], 65536 // 8
                lo = (HALO - a.reach[4]) * plane // align * align
                hi = min(data.numel(), -(-(HALO + NZ + a.reach[5]) * plane // align) * align)
                h2d += (hi - lo) * 8
            elif a.role == "in1":
                h2d += st[a.name].data.numel() * 8
            elif a.role == "out3":
                ilo, ihi, jlo, jhi, klo, khi = a.reach
                d2h += (NX + ilo + ihi) * (NY + jlo + jhi) * (NZ + klo + khi) * 8

    stream = torch.cuda.Stream()
    # The calls are independent.  They are issued with the most output fields first, so the
    # part of the step after the last copy-in (that call's compute and copy-out) is a
    # one-output call's and not fvtp2d's six outputs.
    order = sorted(names, key=lambda n: -len(pkg.KERNELS[n].by_role("out3")))

    def step():
        for name in order:
            st, sc = hs[name]
            pkg.call(name, st, sc, domain=dom, stream=stream)
        stream.synchronize()  # every output of the step is in host memory

    def timed():
        for _ in range(max(1, args.warmup)):
            step()
        steps = max(1, args.steps)
        t = time.perf_counter()
        for _ in range(steps):
            step()
        return (time.perf_counter() - t) / steps

    lib = pkg.load_library()
    lib.oeb_set_host_direct(0)
    dt_staged = timed()
    lib.oeb_set_host_direct(1)
    dt_direct = timed()
    lib.oeb_set_host_async(1)
    try:
        dt = timed()
    finally:
        lib.oeb_set_host_async(0)
    pts = len(names) * NX * NY * NZ
    link = _link_rates(torch)
    # the step's transfer floor: the input bytes at the one-way rate, or all bytes at the rate
    # of both directions at once, whichever is longer (the kernels overlap the copies)
    floor_s = max(h2d / (link["h2d_gbs"] * 1e9), (h2d + d2h) / (link["bidirectional_gbs"] * 1e9))
    link.update({"floor_ms": round(floor_s * 1e3, 3), "frac_of_floor": round(floor_s / dt, 4),
                 "how": "pinned host <-> device copies of 256 MB (cudaMemcpyAsync through torch), best of 5; "
                        "bidirectional: one copy each way on two streams at once"})
    return {"value": round(pts / dt / 1e9, 4), "unit": "GPts/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": round(dt * 1e3, 3),
            "link_roofline": link,
            "path": "oeb_<k>_f64_host on pinned host buffers with oeb_set_host_async(1): the ten calls are enqueued on "
                    "one stream, most output fields first, and the step ends with its synchronisation; "
                    "each call stages the k-planes its kernel reads through device memory, and the copy-in of one "
                    "call overlaps the compute and copy-out of the previous",
            "synchronous_direct": {"value": round(pts / dt_direct / 1e9, 4), "ms_per_step": round(dt_direct * 1e3, 3),
                                   "path": "the same calls, each returning when its outputs are in host memory; the "
                                           "kernels read and write the host fields in place over NVLink-C2C"},
            "synchronous_staged": {"value": round(pts / dt_staged / 1e9, 4), "ms_per_step": round(dt_staged * 1e3, 3),
                                   "path": "the same calls, each returning when its outputs are in host memory, "
                                           "copy-in / compute / copy-out pipelined over k-slabs within the call"},
            }


def _link_rates(torch, mb=256, reps=5):
    """Host <-> device copy rates (GB/s) between pinned host memory and device memory, measured
    here: one way each, and both ways at once on two streams (their summed bytes)."""
    n = mb << 20
    h1 = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    d1 = torch.empty(n, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(n, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def best(fn, nbytes):
        t = []
        for r in range(reps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            if r:
                t.append(time.perf_counter() - t0)
        return nbytes / min(t) / 1e9

    def both():
        with torch.cuda.stream(s1):
            d1.copy_(h1, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    res = {"h2d_gbs": round(best(lambda: d1.copy_(h1, non_blocking=True), n), 1),
           "d2h_gbs": round(best(lambda: h2.copy_(d2, non_blocking=True), n), 1),
           "bidirectional_gbs": round(best(both, 2 * n), 1)}
    del h1, h2, d1, d2
    torch.cuda.empty_cache()
    return res


def _cpu_baseline(pkg, fields, budget_s=15.0, threads=None):
    """The oracle (restated reference OpenMP kernels) on this host's cores, bounded sample."""
    from oracle import oracle as orc
    threads = threads or os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    sets = {}
    for name, spec in pkg.KERNELS.items():
        inputs = fields.make_inputs(name, NX, NY, NZ, seed=SEED)
        outs = fields.make_outputs(name, NX, NY, NZ, include_scratch=True)
        sets[name] = ({**inputs, **outs}, fields.make_scalars(name, seed=SEED))
    per = {}
    steps = 0
    t_all = time.perf_counter()
    while True:
        for name, spec in pkg.KERNELS.items():
            buf, sc = sets[name]
            t = time.perf_counter()
            orc.run_oracle(spec, buf, sc, NX, NY, NZ, HALO)
            per.setdefault(name, []).append(time.perf_counter() - t)
        steps += 1
        if time.perf_counter() - t_all > budget_s or steps >= 50:
            break
    step_s = sum(statistics.mean(v) for v in per.values())
    return {"value": round(len(per) * NX * NY * NZ / step_s / 1e9, 5), "unit": "GPts/s", "cores": threads,
            "kind": "port",
            "sample": "%d steps of the ten-kernel FP64 step at 128x128x80 (oracle restatement of the reference "
                      "_openmp kernels, serial fvtp2d; OMP_NUM_THREADS=%s)" % (steps, os.environ["OMP_NUM_THREADS"]),
            "per_kernel_ms": {k: round(statistics.mean(v) * 1e3, 3) for k, v in per.items()}}


def port_vs_reference(args):
    """`--port-vs-reference`: the oracle port (oracle/oeb_oracle.c) and the reference's own
    headers compiled from source (oracle/_ref), timed on the same inputs (the 128x128x80 step,
    seed 1) with the same host threads, kernel by kernel: how well the port stands in for the
    reference where the reference tree is absent (the GPU host).  Needs the reference source
    tree; prints one JSON line."""
    pkg = graft.load_package()
    import importlib
    fields = importlib.import_module("oeb_gb300.fields")
    from oracle import oracle as orc
    threads = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    if not orc.reference_available():
        print(json.dumps({"port_vs_reference": None, "why": "the reference source tree is absent on this host"}))
        return
    per = {}
    for name, spec in pkg.KERNELS.items():
        inputs = fields.make_inputs(name, NX, NY, NZ, seed=SEED)
        sc = fields.make_scalars(name, seed=SEED)
        bufs = {}
        for kind in ("port", "reference"):
            b = {**{k: v.copy() for k, v in inputs.items()}, **fields.make_outputs(name, NX, NY, NZ,
                                                                                     include_scratch=True)}
            bufs[kind] = b

        def one(kind):
            if kind == "port":
                orc.run_oracle(spec, bufs[kind], sc, NX, NY, NZ, HALO)
            else:
                orc.run_reference(spec, bufs[kind], sc, NX, NZ, HALO, "openmp")

        times = {"port": [], "reference": []}
        for rep in range(max(args.warmup, 1) + args.steps):
            for kind in ("port", "reference"):  # interleaved, so that both see the same host state
                t = time.perf_counter()
                one(kind)
                if rep >= max(args.warmup, 1):
                    times[kind].append(time.perf_counter() - t)
        per[name] = {k: round(statistics.median(v) * 1e3, 3) for k, v in times.items()}
        per[name]["port_over_reference"] = round(per[name]["port"] / per[name]["reference"], 3)
    step = {k: sum(v[k] for v in per.values()) for k in ("port", "reference")}
    print(json.dumps({"port_vs_reference": {"workload": WORKLOAD, "threads": threads, "steps": args.steps,
                                            "step_ms": {k: round(v, 3) for k, v in step.items()},
                                            "step_port_over_reference": round(step["port"] / step["reference"], 3),
                                            "per_kernel_ms": per}}), flush=True)


def run_reference(args):
    rank, world, _ = _dist_env()
    if rank != 0:
        return
    pkg = graft.load_package()
    import importlib
    fields = importlib.import_module("oeb_gb300.fields")
    threads = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    from oracle import oracle as orc
    from oracle import build as ob
    use_ref = orc.reference_available()
    sets = {}
    for name in pkg.KERNELS:
        inputs = fields.make_inputs(name, NX, NY, NZ, seed=SEED)
        outs = fields.make_outputs(name, NX, NY, NZ, include_scratch=True)
        sets[name] = ({**inputs, **outs}, fields.make_scalars(name, seed=SEED))

    def one_step():
        for name, spec in pkg.KERNELS.items():
            buf, sc = sets[name]
            if use_ref:
                orc.run_reference(spec, buf, sc, NX, NZ, HALO, "openmp")
            else:
                orc.run_oracle(spec, buf, sc, NX, NY, NZ, HALO)

    for _ in range(args.warmup):
        one_step()
    t = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    dt = (time.perf_counter() - t) / args.steps
    value = len(pkg.KERNELS) * NX * NY * NZ / dt / 1e9
    kind = "reference" if use_ref else "port"
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": "GPts/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; fields.py 'physical')",
            "config": _config(list(pkg.KERNELS), world),
            "cpu_baseline": {"value": round(value, 5), "unit": "GPts/s", "cores": threads, "kind": kind,
                             "sample": "each step = the ten reference kernels once at 128x128x80 (_openmp "
                                       "variants, serial fvtp2d), %s, OMP_NUM_THREADS=%s" %
                                       ("reference headers compiled from source" if use_ref else
                                        "oracle restatement (reference sources absent on this host)",
                                        os.environ["OMP_NUM_THREADS"])},
            "e2e": {"value": round(value, 5), "unit": "GPts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def profile_one(args):
    """`--profile-one K[,K...]`: each K alone, `--calls` times (with `--adjoint-calls`, its
    adjoint instead, seeded with N(0, 1) output seeds), for an ncu capture (prints nothing
    timed)."""
    import torch
    pkg = graft.load_package()
    import importlib
    fields = importlib.import_module("oeb_gb300.fields")
    dtype = np.float64 if args.precision == "f64" else np.float32
    shape = tuple(args.shape)
    dev = torch.device("cuda", 0)
    names = args.profile_one.split(",")
    for name in names:
        st, sc = _make_set(pkg, fields, torch, dev, 2, [name], dtype=dtype, shape=shape, workload=args.workload)[name]
        if args.adjoint_calls:
            spec = pkg.KERNELS[name]
            like = st[spec.semantic_outputs[0]]
            rng = np.random.default_rng(1)
            yb = {n: pkg.Storage(torch.from_numpy(rng.normal(size=like.data.shape).astype(dtype)).to(dev), HALO)
                  for n in spec.semantic_outputs}
            xb = {n: pkg.Storage(torch.zeros_like(like.data), HALO) for n in pkg.ACTIVE[name]}
            for _ in range(args.calls):
                pkg.adjoint(name, st, yb, xb, sc, domain=shape)
        else:
            for _ in range(args.calls):
                pkg.call(name, st, sc, domain=shape)
    torch.cuda.synchronize()
    print(json.dumps({"profile_one": names, "adjoint": bool(args.adjoint_calls), "precision": args.precision,
                      "shape": list(shape), "calls": args.calls}))


def probe_shuffles():
    """`--probe-shuffles`: i-neighbours through L1 against warp shuffles (the library's
    oeb_probe_shuffle_neighbours: FP32, 256x256x80 + 3-cell halo, a 5-point laplacian and a
    7-cell window along i, each form timed alone over back-to-back launches)."""
    import ctypes
    pkg = graft.load_package()
    lib = pkg.load_library()
    us = (ctypes.c_double * 4)()
    bad = (ctypes.c_uint64 * 2)()
    st = lib.oeb_probe_shuffle_neighbours(us, bad)
    print(json.dumps({"probe": "shuffle_neighbours", "status": st, "shape": [256, 256, 80], "dtype": "f32",
                      "us": {"laplace_l1": round(us[0], 2), "laplace_shuffle": round(us[1], 2),
                             "window7_l1": round(us[2], 2), "window7_shuffle": round(us[3], 2)},
                      "mismatched_cells": {"laplace": bad[0], "window7": bad[1]}}))


def profile_chain(args):
    """`--profile-chain`: the chained step forward + adjoint at `--shape` (seed 3), `--calls`
    times, for an ncu capture of its kernels (prints nothing timed)."""
    import torch
    import importlib
    pkg = graft.load_package()
    fields = importlib.import_module("oeb_gb300.fields")
    chain = importlib.import_module("oeb_gb300.chain")
    dtype = np.float64 if args.precision == "f64" else np.float32
    nx, ny, nz = args.shape
    dev = torch.device("cuda", 0)
    H = fields.CHAIN_HALO
    x = fields.make_chain_inputs(nx, ny, nz, 3, halo=H)
    sc = fields.make_chain_scalars(3)
    st = {k: pkg.Storage(torch.from_numpy(v.astype(dtype)).to(dev), H, nx=nx if v.ndim == 3 else None)
          for k, v in x.items()}
    shape = x["u"].shape
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    outs = {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=nx) for n in chain.OUTPUTS}
    rng = np.random.default_rng(3)
    seeds = {n: pkg.Storage(torch.from_numpy(rng.normal(0.0, 1.0, size=shape).astype(dtype)).to(dev), H, nx=nx)
             for n in chain.OUTPUTS}
    grads = {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=nx) for n in ("u", "v")}
    plan = chain.ChainPlan(st["u"], (nx, ny, nz), chain.FORWARD | chain.ADJOINT)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.calls):
        plan.forward(st, sc, outs, stream=stream)
        plan.adjoint(st, sc, seeds, grads, stream=stream)
    torch.cuda.synchronize()
    plan.close()
    print(json.dumps({"profile_chain": True, "precision": args.precision, "shape": [nx, ny, nz],
                      "calls": args.calls}))


# A small uneven ensemble for ncu captures of the batched forms (nx, ny, nz, element size):
# about 0.4 M points a member, 1.2 GB on the device in all.
PROFILE_MEMBERS = [(96, 64, 40, 8), (64, 80, 60, 4), (128, 48, 40, 8), (48, 112, 60, 4), (80, 80, 40, 8),
                   (112, 64, 40, 4), (64, 64, 60, 8), (96, 96, 40, 4)]


def profile_batch(args):
    """`--profile-batch`: the chained step forward + adjoint of a small uneven ensemble
    (PROFILE_MEMBERS) as one run of the per-launch form, then `--calls` runs of the one-launch
    form (kb 4, `--ctas-per-sm` CTAs an SM), for an ncu capture of the step kernel."""
    import torch
    import importlib
    pkg = graft.load_package()
    fields = importlib.import_module("oeb_gb300.fields")
    chain = importlib.import_module("oeb_gb300.chain")
    dev = torch.device("cuda", 0)
    H = fields.CHAIN_HALO
    members = []
    for idx, (nx, ny, nz, item) in enumerate(PROFILE_MEMBERS):
        dt = np.float64 if item == 8 else np.float32
        x = fields.make_chain_inputs_device(nx, ny, nz, 4000 + idx, dev, dt, halo=H)
        shape = tuple(x["u"].shape)
        tdt = x["u"].dtype
        gen = torch.Generator(device=dev).manual_seed(idx)
        members.append({
            "fields": {k: pkg.Storage(v, H, nx=nx if v.dim() == 3 else None) for k, v in x.items()},
            "scalars": fields.make_chain_scalars(4), "domain": (nx, ny, nz),
            "outs": {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=nx) for n in chain.OUTPUTS},
            "seeds": {n: pkg.Storage(torch.randn(shape, generator=gen, device=dev, dtype=tdt), H, nx=nx)
                      for n in chain.OUTPUTS},
            "grads": {n: pkg.Storage(torch.zeros(shape, dtype=tdt, device=dev), H, nx=nx) for n in ("u", "v")}})
    plan = chain.BatchPlan(members, chain.FORWARD | chain.ADJOINT)
    stream = torch.cuda.current_stream(dev)
    plan.run(stream)
    plan.set_form(plan.ONE_LAUNCH, 4, args.ctas_per_sm)
    for _ in range(args.calls):
        plan.run(stream)
    torch.cuda.synchronize()
    status = plan.step_status()
    plan.close()
    print(json.dumps({"profile_batch": True, "members": len(members), "calls": args.calls,
                      "ctas_per_sm": args.ctas_per_sm, "status": list(status)}))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-f32", action="store_true", help="skip the FP32-storage leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the forward+adjoint leg")
    ap.add_argument("--no-chain", action="store_true", help="skip the chained-step leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble leg")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--kernels", nargs="*", default=None,
                    help="run only these stencils in the step (profiling); the default line uses all ten")
    ap.add_argument("--profile-one", default=None,
                    help="run only these stencils (comma-separated) --calls times each (for ncu captures)")
    ap.add_argument("--precision", choices=["f64", "f32"], default="f64")
    ap.add_argument("--shape", type=int, nargs=3, default=[NX, NY, NZ])
    ap.add_argument("--workload", choices=["physical", "fronts", "smooth"], default="physical")
    ap.add_argument("--calls", type=int, default=4)
    ap.add_argument("--adjoint-calls", action="store_true",
                    help="with --profile-one: run each stencil's adjoint instead of its forward")
    ap.add_argument("--probe-shuffles", action="store_true",
                    help="time i-neighbours through L1 against warp shuffles (FP32 probe stencils) and exit")
    ap.add_argument("--profile-chain", action="store_true",
                    help="run the chained step forward + adjoint --calls times at --shape (for ncu captures)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="run a small uneven ensemble's step in the one-launch form --calls times (for ncu captures)")
    ap.add_argument("--ctas-per-sm", type=int, default=4, help="with --profile-batch: the step kernel build (2, 3, 4)")
    ap.add_argument("--port-vs-reference", action="store_true",
                    help="time the oracle port against the reference build on this host's cores (needs the "
                         "reference source tree) and exit")
    args = ap.parse_args()
    if args.port_vs_reference:
        port_vs_reference(args)
        return
    if args.profile_one:
        profile_one(args)
        return
    if args.profile_chain:
        profile_chain(args)
        return
    if args.profile_batch:
        profile_batch(args)
        return
    if args.probe_shuffles:
        probe_shuffles()
        return
    if args.warmup < 3 and args.impl == "ours":
        sys.stderr.write("warning: fewer than 3 warm-up steps\n")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
