#!/usr/bin/env python
"""Benchmark of the GB300 render path: traced rays per second.

Workload (default): the response-matrix configuration, a 12 m Davies-Cotton
dish (380 hex facets, f = 15 m, 0.5 mrad tilt errors, 4 mast cylinders and a
camera box) with a 2048-pixel hexagonal camera, 4096 point sources on a
64 x 64 grid within +-3 deg and 256 Monte-Carlo samples per facet: one step
renders the dense 4096 x 2048 response matrix (3.99e8 rays). Inputs are
seeded synthetic scenes (iactrace_gb300.workloads), resident on the device.

  value     rays/s of the render step (device time, CUDA events, L2 flushed
            before every timed step by a 256 MiB write outside the events)
  e2e       rays/s through the public API with host buffers: pinned
            sources/values copied in, the matrix copied back, every step
  roofline  the render kernel's algorithmic FP32 flops per launch over its
            event-timed duration, against an FP32 FMA peak measured live on
            the same GPU by a probe kernel of the library
  cpu_baseline  the C++ FP32 restatement of the reference (OpenMP, all host
            cores) on a bounded sample of the same workload

`--impl reference` times the reference algorithm's CPU restatement instead
(the reference itself is JAX and cannot be installed here).
Multi-GPU: one process per GPU, each renders its own full workload
(replicas, weak scaling); rank 0 prints the max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "traced rays/s: fwd and fwd+adjoint vs plain fwd kernel, img err<=1e-5 vs FP64"
# algorithmic FP32 flops per ray (FMA = 2), reference evaluation without early-out:
# point primary 26 + 4 cylinders x 98 + box 29 + sensor plane 34 + hex bin 56
F_RAY = {"response": 537, "plain": 503, "cassegrain": 894, "batched": 537,
         # primary point source 26 + 271 cylinders x 98 + 2 spheres x 35 + box 29 + oriented box 47
         # (rotation 18 + slab 29) + triangle 40 (Moller-Trumbore) + plane 34 + hex bin 56
         "obstructed": 26 + 271 * 98 + 2 * 35 + 29 + 47 + 40 + 34 + 56}


# the render kernel each workload's `roofline` times (kernel events of the library)
KERNEL = {"response": "k_masks + k_render_hard", "plain": "k_masks + k_render_hard",
          "cassegrain": "k_render (later mirror stages)", "obstructed": "k_render (276 primitives)",
          "batched": "k_batch_masks + k_batch_render_hard"}


# Figures from one ncu capture of each workload's render kernel (summaries
# under profiles/, with the commands that made them): DRAM bytes (read +
# write) per launch, shared-memory atomic wavefronts as a fraction of their
# sustained peak (l1tex__data_pipe_lsu_wavefronts_mem_shared_op_atom.sum.
# pct_of_peak_sustained_elapsed: the atomic-bound fraction of the histogram
# adds), executed thread instructions per ray (smsp__inst_executed.sum x
# average active threads per instruction / rays) and the FMA pipe's share of
# its peak (sm__inst_executed_pipe_fma). Each records the digest of the
# kernel sources it was taken on (source_digest() below); when the sources
# have changed since, the figures are reported as stale and not used as the
# roofline's traffic.
CAPTURES = {
    "response": {"digest": "8f1912f64f179566", "profile": "profiles/k_render_hard_response_matrix_dc380_hex2048.md",
                 "dram_bytes": 13.51e6, "shared_atomic_frac": 0.097, "thread_inst_per_ray": 175,
                 "fma_pipe": 0.351, "issue_active": 0.850},
    "plain": {"digest": "8f1912f64f179566", "profile": "profiles/k_render_hard_plain_forward_dc380_square960.md",
              "dram_bytes": 12.21e6, "shared_atomic_frac": 0.082, "thread_inst_per_ray": 183,
              "fma_pipe": 0.249, "issue_active": 0.672},
    "cassegrain": {"digest": "8f1912f64f179566", "profile": "profiles/k_render_cassegrain_61seg_square1024.md",
                   "dram_bytes": 1.050e6, "shared_atomic_frac": 0.025, "thread_inst_per_ray": 945,
                   "fma_pipe": 0.389, "issue_active": 0.740},
    "batched": {"digest": "8f1912f64f179566", "profile": "profiles/k_batch_render_hard_ragged_batch64_hex960_2048.md",
                "dram_bytes": 383.5e6, "thread_inst_per_ray": 188, "fma_pipe": 0.309, "issue_active": 0.804},
}


def source_digest() -> str:
    """sha256 (16 hex digits) of the CUDA sources and the C ABI header."""
    import hashlib
    h = hashlib.sha256()
    csrc = os.path.join(ROOT, "iactrace_gb300", "csrc")
    files = sorted(os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".cu", ".cuh", ".h")))
    for path in files + [os.path.join(ROOT, "include", "iactrace_gb300.h")]:
        h.update(os.path.basename(path).encode())
        with open(path, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def capture_fields(workload):
    """The capture record of `workload` and whether it matches the sources."""
    cap = CAPTURES.get(workload)
    if cap is None:
        return None, None
    current = cap["digest"] == source_digest()
    rec = dict(cap, current=current)
    return rec, current


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_workload(name: str):
    from iactrace_gb300 import workloads as W
    if name == "response":
        return W.response_matrix(), "response"
    if name == "plain":
        return W.plain_forward(), "image"
    if name == "cassegrain":
        return W.cassegrain(), "image"
    if name == "obstructed":
        return W.obstructed(), "image"
    raise SystemExit(f"unknown workload {name}")


def workload_config(name, tel, S, mode, flush):
    F = sum(len(g) for g in tel.mirror_groups if g.optical_stage == 0)
    M = tel.mirror_groups[0].n_samples
    cfg = {"workload": {"response": "response_matrix_dc380_hex2048", "plain": "plain_forward_dc380_square960",
                        "cassegrain": "cassegrain_61seg_square1024",
                        "obstructed": "obstructed_dc380_struts271_hex960"}[name],
           "facets": F, "samples_per_facet": M, "sources": S,
           "pixels": int(math.prod(tel.sensors[0].get_accumulator_shape())),
           "output": "response matrix (S, P) fp32" if mode == "response" else "image fp32",
           "rays_per_step": F * M * S, "l2": flush}
    return cfg, F * M * S


def adjoint_kernel_seconds(tel, src, val, stype, mode, gout, flush_buf, steps, samples=False):
    """Event time of the adjoint kernel alone (iact_render_backward through
    the C ABI, gradients w.r.t. facet rotations and positions, sources and
    values, and with `samples` the per-sample sums that carry the primary
    surface's gradients), averaged over `steps` launches with the L2 flushed
    before each."""
    import ctypes
    from iactrace_gb300 import _native as N
    from iactrace_gb300.core.render import source_code
    from iactrace_gb300.core.scene import pack_scene
    dev = src.device
    lib = N.load()
    ps = pack_scene(tel, dev)
    sdesc, keep = tel.sensors[0].pack(dev)
    S = src.shape[0]
    ws = torch.empty(ps.workspace_bytes(sdesc, S, N.MODE_BACKWARD), dtype=torch.uint8, device=dev)
    g = [torch.empty((ps.F, 3), device=dev), torch.empty((ps.F, 3), device=dev),
         torch.empty((S, 3), device=dev), torch.empty(S, device=dev)]
    gsamp = torch.empty((ps.F * ps.M, 7), device=dev) if samples else None
    nm = N.MODE_RESPONSE if mode == "response" else N.MODE_IMAGE
    gout = gout.contiguous()
    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    stream = torch.cuda.current_stream(dev)
    ev[0].record(stream)
    ev[1].record(stream)
    o = N.IactOpts()
    o.kernel_events[0], o.kernel_events[1] = ev[0].cuda_event, ev[1].cuda_event
    code = source_code(stype)
    no_src = code == N.SRC_EXTENDED

    def call():
        N.check(lib.iact_render_backward(ctypes.byref(ps.desc), ctypes.byref(sdesc), code, src.data_ptr(),
                                         val.data_ptr(), S, nm, gout.data_ptr(), g[0].data_ptr(), g[1].data_ptr(),
                                         None, None if no_src else g[2].data_ptr(), g[3].data_ptr(), None, None,
                                         None, gsamp.data_ptr() if samples else None, ws.data_ptr(),
                                         ws.numel(), ctypes.byref(o), stream.cuda_stream))

    call()
    tot = 0.0
    for k in range(steps):
        flush_buf.fill_(float(k))
        call()
        ev[1].synchronize()
        tot += ev[0].elapsed_time(ev[1]) / 1e3
    del keep
    return tot / steps


def fp32_peak_tflops(dev) -> float:
    """FP32 throughput of an FMA-chain probe kernel on this GPU (TFLOP/s)."""
    from iactrace_gb300 import _native as N
    lib = N.load()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = sms * 16, 4096
    out = torch.empty(blocks * 256, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(3):
        N.check(lib.iact_probe_fma(out.data_ptr(), blocks, iters, stream.cuda_stream))
    best = float("inf")
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        N.check(lib.iact_probe_fma(out.data_ptr(), blocks, iters, stream.cuda_stream))
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b) / 1e3)
    flops = blocks * 256 * iters * 8 * 2
    return flops / best / 1e12


def cpu_baseline(name, tel, src, val, stype, mode, target_s=12.0):
    """C++ FP32 restatement on all host cores, bounded sample of the workload."""
    import oracle.oracle as O
    threads = os.cpu_count() or 1
    F = sum(len(g) for g in tel.mirror_groups if g.optical_stage == 0)
    M = tel.mirror_groups[0].n_samples
    omode = "response" if mode == "response" else "image"
    n = max(1, min(src.shape[0], threads))
    t = time.perf_counter()
    O.render(tel, src[:n], val[:n], stype, 0, mode=omode, dtype="f32", threads=threads)
    dt = time.perf_counter() - t
    rate = n * F * M / max(dt, 1e-9)
    n2 = int(max(n, min(src.shape[0], rate * target_s / (F * M))))
    t = time.perf_counter()
    O.render(tel, src[:n2], val[:n2], stype, 0, mode=omode, dtype="f32", threads=threads)
    dt = time.perf_counter() - t
    rays = n2 * F * M
    return {"value": rays / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": f"{n2} of {src.shape[0]} sources x {F} facets x {M} samples ({rays:.3g} rays, {dt:.1f} s)"}


def run_reference(args, rank, world):
    """CPU restatement of the reference algorithm, all host threads, bounded steps."""
    if rank != 0:
        return
    import oracle.oracle as O
    if args.workload == "batched":
        return run_reference_batched(args, world)
    (tel, src, val, stype), mode = build_workload(args.workload)
    cfg, rays_full = workload_config(args.workload, tel, src.shape[0], mode, "n/a (CPU)")
    threads = os.cpu_count() or 1
    F = cfg["facets"]
    M = cfg["samples_per_facet"]
    omode = "response" if mode == "response" else "image"
    n = max(1, min(src.shape[0], threads))
    t = time.perf_counter()
    O.render(tel, src[:n], val[:n], stype, 0, mode=omode, dtype="f32", threads=threads)
    rate = n * F * M / max(time.perf_counter() - t, 1e-9)
    budget = args.cpu_budget / max(1, args.steps + args.warmup)
    ns = int(max(1, min(src.shape[0], rate * budget / (F * M))))
    for _ in range(args.warmup):
        O.render(tel, src[:ns], val[:ns], stype, 0, mode=omode, dtype="f32", threads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        O.render(tel, src[:ns], val[:ns], stype, 0, mode=omode, dtype="f32", threads=threads)
    dt = time.perf_counter() - t
    rays = ns * F * M * args.steps
    value = rays / dt
    sample = f"{ns} of {src.shape[0]} sources x {F} facets x {M} samples per step"
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": cfg, "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "rays/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is JAX (not installable here); timed its C++ FP32 restatement (oracle/) on host cores",
    }), flush=True)


def run_reference_batched(args, world):
    """The ragged batch through the CPU restatement: instances in order, each
    a bounded number of sources, until the per-step time budget is spent."""
    import oracle.oracle as O
    from iactrace_gb300 import workloads as W
    tels, srcs, vals, st = W.ragged_batch()
    threads = os.cpu_count() or 1
    M = tels[0].mirror_groups[0].n_samples
    budget = args.cpu_budget / max(1, args.steps + args.warmup)

    def step():
        rays, t0, k = 0, time.perf_counter(), 0
        while k < len(tels) and time.perf_counter() - t0 < budget:
            n = min(srcs[k].shape[0], threads)
            O.render(tels[k], srcs[k][:n], vals[k][:n], st, 0, mode="image", dtype="f32", threads=threads)
            rays += n * len(tels[k].mirror_groups[0]) * M
            k += 1
        return rays, time.perf_counter() - t0, k

    for _ in range(args.warmup):
        step()
    tot_r, tot_t, ks = 0, 0.0, []
    for _ in range(args.steps):
        r, t, k = step()
        tot_r += r
        tot_t += t
        ks.append(k)
    value = tot_r / tot_t
    sample = (f"per step: instances 0..{min(ks) - 1} of 64 in order, up to {threads} sources each, "
              f"{M} samples per facet (~{budget:.0f} s budget)")
    print(json.dumps({
        "metric": METRIC + " [ragged batch: one persistent launch + CUDA graph]", "value": value, "unit": "rays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": {"workload": "ragged_batch_64_dc_variants_hex960_2048"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "rays/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is JAX (not installable here); timed its C++ FP32 restatement (oracle/) on host cores",
    }), flush=True)


def run_alignment(args, rank, world):
    """Mirror-alignment inverse problem: Adam steps of forward + adjoint."""
    import iactrace_gb300 as it  # noqa: F401
    from iactrace_gb300 import _native as N, alignment as A
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    N.load(build_if_missing=True)
    pb = A.problem(device=dev)
    F = pb["telescope"].mirror_groups[0].positions.shape[0]
    M = pb["telescope"].mirror_groups[0].n_samples
    S = pb["sources"].shape[0]
    rays = F * M * S
    A.run(pb, steps=args.warmup, graph=True)  # warm-up
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    steps = max(args.steps, 200)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    hist = A.run(pb, steps=steps, graph=True)
    torch.cuda.synchronize(dev)
    dt = (time.perf_counter() - t0) / steps
    clk = clocks.stop()
    # kernel time of one forward render and one adjoint of the same problem (CUDA events)
    import iactrace_gb300 as it
    from iactrace_gb300 import _native as N
    tel, src, val = pb["telescope"], pb["sources"], pb["values"]
    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    stream = torch.cuda.current_stream(dev)
    ev[0].record(stream)
    ev[1].record(stream)
    o = N.IactOpts()
    o.kernel_events[0], o.kernel_events[1] = ev[0].cuda_event, ev[1].cuda_event
    o.seed = pb["seed"]
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    fw = []
    for k in range(5):
        flush_buf.fill_(float(k))
        out = it.render(tel, src, val, "extended", opts=o, seed=pb["seed"])
        ev[1].synchronize()
        fw.append(ev[0].elapsed_time(ev[1]))
    adj_s = adjoint_kernel_seconds(tel, src, val, "extended", "image", torch.ones_like(out), flush_buf, 5)
    if rank == 0:
        print(json.dumps({
            "metric": METRIC + " [alignment: Adam step = fwd + adjoint]", "value": rays / dt, "unit": "rays/s",
            "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded dish, sources and misalignment)",
            "config": {"workload": "alignment_dish28m_876facets_hex2048_extended256", "facets": F,
                       "samples_per_facet": M, "sources": S, "parameters": 2 * F, "rays_per_step": rays,
                       "timing": "host wall clock per Adam step incl. synchronize (forward, adjoint, optimiser; "
                                 "3 eager steps, then the step replayed as one CUDA graph)"},
            "kernels": {"render_ms": sorted(fw)[2], "adjoint_ms": adj_s * 1e3,
                        "kernel_time_ratio_vs_fwd": (sorted(fw)[2] + adj_s * 1e3) / sorted(fw)[2]},
            "alignment": {"loss_first": hist["loss"][0], "loss_last": hist["loss"][-1],
                          "rms_tilt_error_mrad_first": hist["rms_mrad"][0],
                          "rms_tilt_error_mrad_last": hist["rms_mrad"][-1], "adam_steps": steps,
                          "note": "camera at the focus, where every facet's spot of a source falls on the "
                                  "same place: the image loss falls, the per-facet tilts are not identifiable "
                                  "from the summed image; with a defocused camera the same run recovers them "
                                  "(tests/test_gpu_extended.py)"},
            # the library's kernels per Adam step (counted by the library around the
            # captured step) times the timed steps
            "gpu_launches": hist["launches_per_step"] * steps,
            "clocks": clk,
        }), flush=True)


def run_batched(args, rank, world):
    """Ragged batch of 64 telescope variants: one CUDA-graph replay of the
    persistent batched kernel against per-instance render() launches."""
    import iactrace_gb300 as it
    from iactrace_gb300 import _native as N, workloads as W
    from iactrace_gb300.core import autotune as AT
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    N.load(build_if_missing=True)
    tels, srcs_h, vals_h, st = W.ragged_batch(n_instances=args.instances, max_sources=args.max_sources)
    srcs = [s.to(dev) for s in srcs_h]
    vals = [v.to(dev) for v in vals_h]
    F = [len(t.mirror_groups[0]) for t in tels]
    M = tels[0].mirror_groups[0].n_samples
    S = [s.shape[0] for s in srcs]
    rays = sum(f * s * M for f, s in zip(F, S))
    stream = torch.cuda.current_stream(dev)
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    t0 = time.perf_counter()
    b = it.BatchRenderer(tels, srcs, vals, st, tune=not args.no_tune)
    setup_s = time.perf_counter() - t0
    tune = AT.last_result(b)
    info = b.info()

    def timed(fn, steps):
        evs = []
        for k in range(steps):
            flush_buf.fill_(float(k))
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            e.record(stream)
            evs.append((a, e))
        torch.cuda.synchronize(dev)
        return sum(a.elapsed_time(e) for a, e in evs) / 1e3 / steps

    def per_instance():
        for t, s, v in zip(tels, srcs, vals):
            it.render(t, s, v, st)

    for _ in range(args.warmup):
        b()
        per_instance()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        import torch.distributed as tdist
        tdist.barrier()
    torch.cuda.synchronize(dev)
    batch_s = timed(b, args.steps)
    inst_s = timed(per_instance, args.steps)

    # kernel-only time of the persistent kernel (events inside the launch sequence)
    kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    kev[0].record(stream)
    kev[1].record(stream)
    o = N.IactOpts()
    if b.opts is not None:
        ctypes_memmove(o, b.opts)
    o.kernel_events[0], o.kernel_events[1] = kev[0].cuda_event, kev[1].cuda_event
    bk = it.BatchRenderer(tels, srcs, vals, st, opts=o, graph=False, tune=False)
    bk()
    ks = []
    for k in range(args.steps):
        flush_buf.fill_(float(k))
        bk()
        kev[1].synchronize()
        ks.append(kev[0].elapsed_time(kev[1]) / 1e3)
    kern_s = sum(ks) / len(ks)
    del bk

    # e2e: pinned host sources/values into the batch's tensors, replay, outputs back
    src_pin = [s.pin_memory() for s in srcs_h]
    val_pin = [v.pin_memory() for v in vals_h]
    out_pin = [torch.empty(x.shape, dtype=torch.float32).pin_memory() for x in b.outs]

    def e2e_step():
        for i in range(len(tels)):
            b.sources[i].copy_(src_pin[i], non_blocking=True)
            b.values[i].copy_(val_pin[i], non_blocking=True)
        outs = b()
        for i in range(len(tels)):
            out_pin[i].copy_(outs[i], non_blocking=True)

    e2e_step()
    e2e_s = timed(e2e_step, args.steps)

    # forward + adjoint per instance (facet tilts and positions, sources, values)
    def fwd_adj():
        for t, s, v in zip(tels, srcs, vals):
            g = t.mirror_groups[0]
            rot = g.rotations.to(dev).requires_grad_(True)
            t2 = t.set_mirror_rotations(0, rot)
            out = it.render(t2, s, v.clone().requires_grad_(True), st)
            out.sum().backward()

    fwd_adj()
    fa_steps = max(1, min(args.steps, 3))
    fa_s = timed(fwd_adj, fa_steps)

    # forward + adjoint of every instance as two graph replays (iact_batch_backward)
    bb = it.BatchRenderer(tels, srcs, vals, st, opts=b.opts, tune=False, backward=True,
                          grads=("rot", "pos", "src", "val"))
    gen = torch.Generator(device=dev).manual_seed(0)
    for go in bb.grad_outs:
        go.copy_(torch.randn(go.shape, device=dev, generator=gen))

    def fwd_adj_batched():
        bb()
        bb.backward()

    fwd_adj_batched()
    fab_s = timed(fwd_adj_batched, fa_steps)
    b_info = bb.info()
    del bb

    # the launch-bound regime: 64 small variants (1-64 sources, 100-300 facets)
    st_tels, st_src, st_val, _ = W.ragged_batch(n_instances=64, seed=11, max_sources=64, max_facets=300)
    st_src = [x.to(dev) for x in st_src]
    st_val = [x.to(dev) for x in st_val]
    st_rays = sum(len(t.mirror_groups[0]) * t.mirror_groups[0].n_samples * x.shape[0] for t, x in zip(st_tels, st_src))
    sb = it.BatchRenderer(st_tels, st_src, st_val, st, tune=True)

    def st_inst():
        for t, x, v in zip(st_tels, st_src, st_val):
            it.render(t, x, v, st)

    for _ in range(args.warmup):
        sb()
        st_inst()
    small = {"instances": 64, "sources_max": 64, "facets_min_max": [100, 300], "rays_per_step": st_rays}
    small["batched_ms"] = timed(sb, args.steps) * 1e3
    small["per_instance_ms"] = timed(st_inst, args.steps) * 1e3
    small["batched_vs_per_instance"] = small["per_instance_ms"] / small["batched_ms"]
    del sb
    clk = clocks.stop()
    peak = fp32_peak_tflops(dev)
    achieved = F_RAY["batched"] * rays / kern_s / 1e12
    h2d = sum(s.numel() * 4 + v.numel() * 4 for s, v in zip(srcs_h, vals_h))
    d2h = sum(x.numel() * 4 for x in b.outs)
    bcap, bcap_ok = capture_fields("batched")
    line = {
        "metric": METRIC + " [ragged batch: one persistent launch + CUDA graph]", "value": rays * world / batch_s,
        "unit": "rays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": batch_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded Davies-Cotton variants and sources)",
        "config": {"workload": f"ragged_batch_{len(tels)}_dc_variants_hex960_2048", "instances": len(tels),
                   "facets_min_max": [min(F), max(F)], "sources_min_max": [min(S), max(S)],
                   "samples_per_facet": M, "rays_per_step": rays, "output": "64 images fp32",
                   "l2": "flushed before each step (256 MiB write)"},
        "e2e": {"value": rays * world / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
        "per_instance": {"value": rays / inst_s, "unit": "rays/s", "ms_per_step": inst_s * 1e3,
                         "launches_per_step": 3 * len(tels), "path": "render() per telescope, same stream"},
        "batched_vs_per_instance": inst_s / batch_s,
        "small_instances": small,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": bcap["dram_bytes"] if bcap_ok else None,
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read + write)",
                     "kernel": KERNEL["batched"], "kernel_ms": kern_s * 1e3,
                     "flops_per_ray": F_RAY["batched"],
                     "flops_note": "algorithmic: the reference's full evaluation per ray without early-out "
                                   "(obstruction tests the bundle culling skips are counted)",
                     "peak_source": "measured live: FP32 FMA-chain probe kernel (iact_probe_fma)",
                     "executed": {k: bcap[k] for k in ("thread_inst_per_ray", "fma_pipe", "issue_active")
                                  if k in bcap} if bcap_ok else None,
                     "capture": bcap},
        "fwd_adjoint_per_instance": {"value": rays / fa_s, "unit": "rays/s", "ms_per_step": fa_s * 1e3,
                                     "time_ratio_vs_batched_fwd": fa_s / batch_s},
        "fwd_adjoint_batched": {"value": rays / fab_s, "unit": "rays/s", "ms_per_step": fab_s * 1e3,
                                "time_ratio_vs_batched_fwd": fab_s / batch_s,
                                "vs_per_instance": fa_s / fab_s, "launches": b_info["launches"] +
                                b_info["backward_launches"]},
        "autotune": {"knobs_block_tasks_hist": tune["knobs"] if tune else None,
                     "candidates_ms": tune["tried"] if tune else None, "setup_s": setup_s},
        "batch": info,
        "gpu_launches": info["launches"] * args.steps,
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline("batched", tels[0], srcs_h[0], vals_h[0], st, "image")
        line["cpu_baseline"]["sample"] = "instance 0 of 64: " + line["cpu_baseline"]["sample"]
    if rank == 0:
        print(json.dumps(line), flush=True)


def ctypes_memmove(dst, src):
    import ctypes
    ctypes.memmove(ctypes.addressof(dst), ctypes.addressof(src), ctypes.sizeof(dst))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="response",
                    choices=["response", "plain", "cassegrain", "obstructed", "alignment", "batched"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--instances", type=int, default=64, help="batched workload: telescope variants")
    ap.add_argument("--max-sources", type=int, default=4096, help="batched workload: largest source count")
    ap.add_argument("--no-tune", action="store_true", help="batched workload: library defaults, no autotuner")
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="--impl reference: seconds of CPU work over all steps")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = _env_rank()
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            tdist.destroy_process_group()
        return
    if args.workload == "batched":
        run_batched(args, rank, world)
        if dist:
            tdist.destroy_process_group()
        return
    if args.workload == "alignment":
        run_alignment(args, rank, world)
        if dist:
            tdist.destroy_process_group()
        return

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import iactrace_gb300 as it
    from iactrace_gb300 import _native as N
    N.load(build_if_missing=True)
    (tel, src_h, val_h, stype), mode = build_workload(args.workload)
    S = src_h.shape[0]
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    cfg, rays = workload_config(args.workload, tel, S, mode, "flushed before each step (256 MiB write)")
    fn = it.render_response_matrix if mode == "response" else it.render
    src = src_h.to(dev)
    val = val_h.to(dev)
    stream = torch.cuda.current_stream(dev)

    opts = N.IactOpts()
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in kev:  # torch creates the CUDA event at its first record()
        a.record(stream)
        b.record(stream)

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    # warm-up steps after the sampler's start (an idle pause before the timed
    # steps would make the first of them pay the wake-up), each the same
    # call as a timed step
    for k in range(args.warmup):
        flush_buf.fill_(float(k))
        opts.kernel_events[0] = kev[0][0].cuda_event
        opts.kernel_events[1] = kev[0][1].cuda_event
        out = fn(tel, src, val, stype, opts=opts)
    torch.cuda.synchronize(dev)
    if dist:
        tdist.barrier()
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    lib = N.load()
    n_launch0 = lib.iact_kernel_launches()
    for k in range(args.steps):
        flush_buf.fill_(float(k))
        opts.kernel_events[0] = kev[k][0].cuda_event
        opts.kernel_events[1] = kev[k][1].cuda_event
        ev[k][0].record(stream)
        out = fn(tel, src, val, stype, opts=opts)
        ev[k][1].record(stream)
    n_launch = lib.iact_kernel_launches() - n_launch0  # the library's kernels in the timed steps
    torch.cuda.synchronize(dev)
    if dist:
        tdist.barrier()
    step_s = sum(a.elapsed_time(b) for a, b in ev) / 1e3 / args.steps
    kern_s = sum(a.elapsed_time(b) for a, b in kev) / 1e3 / args.steps
    culling = None
    if args.workload == "obstructed":
        # the same launches with every primitive tested on every ray
        nc = N.IactOpts()
        nc.flags = N.FLAG_NO_CULL
        nev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in nev:
            a.record(stream)
            b.record(stream)
        fn(tel, src, val, stype, opts=nc)
        for k in range(args.steps):
            flush_buf.fill_(float(k))
            nc.kernel_events[0] = nev[k][0].cuda_event
            nc.kernel_events[1] = nev[k][1].cuda_event
            fn(tel, src, val, stype, opts=nc)
        torch.cuda.synchronize(dev)
        nc_s = sum(a.elapsed_time(b) for a, b in nev) / 1e3 / args.steps
        culling = {"kernel_ms": kern_s * 1e3, "no_cull_kernel_ms": nc_s * 1e3, "speedup": nc_s / kern_s,
                   "primitives": 276, "note": "exact warp-bundle culling vs every primitive on every ray"}

    # forward + adjoint through torch.autograd (recompute-based adjoint kernel)
    grp = tel.mirror_groups[0]
    rot = grp.rotations.clone().to(dev).requires_grad_(True)
    pos = grp.positions.clone().to(dev).requires_grad_(True)
    src_g = src.clone().requires_grad_(True)
    val_g = val.clone().requires_grad_(True)
    grads = "facet rotations and positions, sources, values"
    resample = args.workload == "cassegrain"
    if resample:
        # the two-mirror config's backward includes the primary's aspheric
        # coefficients: each step resamples the primary on the device with
        # the coefficients as autograd leaves (per-sample adjoint sums, mapped
        # to the surface by the sampler's differentiable restatement)
        asph = torch.as_tensor(grp.aspheric, dtype=torch.float32).clone().to(dev).requires_grad_(True)
        grp = grp.replace(offsets=grp.offsets.to(dev), vertices=grp.vertices.to(dev),
                          perturbation_scale=grp.perturbation_scale.to(dev))
        # fixed stage >= 1 mirrors with device-resident parameters (nothing is
        # copied from the host inside a captured step)
        dev_t = lambda x: (x if isinstance(x, torch.Tensor) else torch.tensor(float(x))).to(dev)
        later = [g.replace(**{n: dev_t(getattr(g, n)) for n in ("positions", "rotations", "offsets", "aspheric",
                                                                  "radii", "vertices", "curvature", "conic")
                              if getattr(g, n, None) is not None}) for g in tel.mirror_groups[1:]]
        integ = it.DeviceIntegrator(grp.n_samples, device=dev)
        grads += ", primary aspheric coefficients (resampling)"
    else:
        # the optimised facet transforms and the roughness scales on the device
        # (no host-to-device copy inside a step)
        grp = grp.replace(perturbation_scale=grp.perturbation_scale.to(dev))
        later = [g for g in tel.mirror_groups[1:]]

    def tel_for_step():
        if not resample:
            return it.Telescope([grp.replace(rotations=rot, positions=pos)] + later, tel.obstruction_groups,
                                tel.sensors, tel.name)
        gs = integ.sample_group(grp.replace(aspheric=asph), 0).replace(rotations=rot, positions=pos)
        return it.Telescope([gs] + later, tel.obstruction_groups, tel.sensors, tel.name)

    gout = torch.randn(out.shape, device=dev, generator=torch.Generator(device=dev).manual_seed(0))
    fwdadj = None
    try:
        for _ in range(2):
            fn(tel_for_step(), src_g, val_g, stype).backward(gout)
        torch.cuda.synchronize(dev)
        fa_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(args.steps)]
        for k in range(args.steps):
            flush_buf.fill_(float(k))
            fa_ev[k][0].record(stream)
            fn(tel_for_step(), src_g, val_g, stype).backward(gout)
            fa_ev[k][1].record(stream)
        torch.cuda.synchronize(dev)
        fa_s = sum(a.elapsed_time(b) for a, b in fa_ev) / 1e3 / args.steps
        adj_s = adjoint_kernel_seconds(tel, src, val, stype, mode, gout, flush_buf, args.steps, samples=resample)
        fwdadj = {"value": rays / fa_s, "unit": "rays/s", "ms_per_step": fa_s * 1e3,
                  "time_ratio_vs_fwd": fa_s / step_s,
                  "adjoint_kernel_ms": adj_s * 1e3,
                  "kernel_time_ratio_vs_fwd": (kern_s + adj_s) / kern_s,
                  "grads": grads}
        # the same step (with resampling: resample, render, adjoint,
        # sampler reverse) captured once in a CUDA graph and replayed: the
        # eager step of a small scene is bound by the host's Python and
        # torch dispatch, the graph replay by the GPU
        try:
            side = torch.cuda.Stream(dev)
            side.wait_stream(stream)
            with torch.cuda.stream(side):
                for _ in range(2):
                    fn(tel_for_step(), src_g, val_g, stype).backward(gout)
            stream.wait_stream(side)
            for t in (rot, pos, src_g, val_g) + ((asph,) if resample else ()):
                t.grad = None
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                fn(tel_for_step(), src_g, val_g, stype).backward(gout)
            graph.replay()
            torch.cuda.synchronize(dev)
            gr_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                     for _ in range(args.steps)]
            for k in range(args.steps):
                flush_buf.fill_(float(k))
                gr_ev[k][0].record(stream)
                graph.replay()
                gr_ev[k][1].record(stream)
            torch.cuda.synchronize(dev)
            gr_s = sum(a.elapsed_time(b) for a, b in gr_ev) / 1e3 / args.steps
            fwdadj["graph"] = {"value": rays / gr_s, "unit": "rays/s", "ms_per_step": gr_s * 1e3,
                               "time_ratio_vs_fwd": gr_s / step_s}
        except Exception as e:  # reported, not fatal: the eager numbers above stand
            torch.cuda.synchronize(dev)
            fwdadj["graph"] = {"unavailable": str(e).splitlines()[0][:200]}
    except NotImplementedError as e:
        fwdadj = {"unavailable": str(e)}

    # e2e through the public API with host buffers
    src_pin = src_h.pin_memory()
    val_pin = val_h.pin_memory()
    out_pin = torch.empty(out.shape, dtype=torch.float32).pin_memory()
    for _ in range(2):
        o = fn(tel, src_pin.to(dev, non_blocking=True), val_pin.to(dev, non_blocking=True), stype)
        out_pin.copy_(o, non_blocking=True)
    torch.cuda.synchronize(dev)
    # K steps back to back, each: sources and values copied in from pinned
    # memory, render, result copied back into pinned memory on a second
    # stream (two buffers), so step k's copy-back overlaps step k+1's render;
    # the L2-flush write before each step stays in the loop, its time (the
    # mean of K flushes timed alone) is subtracted: time per step = (the
    # loop's span from the first step's start to the last copy-back's end -
    # (K - 1) flushes) / K. No per-step events: on a short step their host
    # cost would pace the loop
    ev = lambda: torch.cuda.Event(enable_timing=True)
    fill_ev = [(ev(), ev()) for _ in range(args.steps)]
    for k in range(args.steps):
        fill_ev[k][0].record(stream)
        flush_buf.fill_(float(k))
        fill_ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    fill_s = sum(a.elapsed_time(b) for a, b in fill_ev) / 1e3 / args.steps
    cstream = torch.cuda.Stream(dev)
    out_pins = [out_pin, torch.empty(out.shape, dtype=torch.float32).pin_memory()]
    start, end = ev(), ev()
    for k in range(args.steps):
        flush_buf.fill_(float(k))
        if k == 0:
            start.record(stream)
        o = fn(tel, src_pin.to(dev, non_blocking=True), val_pin.to(dev, non_blocking=True), stype)
        cstream.wait_stream(stream)
        with torch.cuda.stream(cstream):
            out_pins[k % 2].copy_(o, non_blocking=True)
        o.record_stream(cstream)
    end.record(cstream)
    torch.cuda.synchronize(dev)
    e2e_s = (start.elapsed_time(end) / 1e3 - (args.steps - 1) * fill_s) / args.steps
    # the same call timed by the host clock, one call at a time: each step
    # ends with a synchronize, so the host's own overhead (argument checks,
    # the cached packing, launches, copies) and the synchronisation latency
    # are inside the time, as a caller waiting for each result sees them
    wall = []
    for k in range(args.steps):
        flush_buf.fill_(float(k))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        o = fn(tel, src_pin.to(dev, non_blocking=True), val_pin.to(dev, non_blocking=True), stype)
        out_pin.copy_(o, non_blocking=True)
        torch.cuda.synchronize(dev)
        wall.append(time.perf_counter() - t0)
    wall_s = sorted(wall)[len(wall) // 2]
    # the same call through a RenderPlan (copies in, render, copy out as one
    # CUDA graph per call), host clock, one call at a time; the result lands
    # in the plan's pinned buffer
    plan = it.RenderPlan(tel, S, stype, mode=mode, depth=2)
    for _ in range(2):
        plan(src_h, val_h, copy=False)
    pw = []
    for k in range(args.steps):
        flush_buf.fill_(float(k))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        plan(src_h, val_h, copy=False)
        pw.append(time.perf_counter() - t0)
    plan_s = sorted(pw)[len(pw) // 2]
    # pipelined through RenderPlan.submit: each step copies the sources and
    # values into the next of two slots, replays its graph (copies in,
    # render, copy out) and takes the previous step's result, so the host
    # prepares step k + 1 while the GPU runs step k; the L2-flush write
    # before each step is on the plan's stream, its mean time subtracted as
    # above; CUDA events on the plan's stream from the first step's start to
    # the last copy-back's end
    n_pipe = max(args.steps, 50)
    pstart, pend = ev(), ev()
    prev = None
    for k in range(n_pipe):
        with torch.cuda.stream(plan.stream):
            flush_buf.fill_(float(k))
            if k == 0:
                pstart.record(plan.stream)
        tk = plan.submit(src_h, val_h)
        if prev is not None:
            prev.result(copy=False)
        prev = tk
    pend.record(plan.stream)
    prev.result(copy=False)
    torch.cuda.synchronize(dev)
    pipe_s = (pstart.elapsed_time(pend) / 1e3 - (n_pipe - 1) * fill_s) / n_pipe
    del plan, prev, tk
    clk = clocks.stop()

    t = torch.tensor([step_s, kern_s, e2e_s], device=dev, dtype=torch.float64)
    if dist:
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    step_s, kern_s, e2e_s = t.tolist()

    peak = fp32_peak_tflops(dev)
    achieved = F_RAY[args.workload] * rays / kern_s / 1e12
    cap, cap_ok = capture_fields(args.workload)
    h2d = src_h.numel() * 4 + val_h.numel() * 4
    d2h = out.numel() * 4
    line = {
        "metric": METRIC, "value": rays * world / step_s, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes and sources)", "config": cfg,
        "e2e": {"value": rays * world / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                "timing": "K steps back to back (copy in, render, copy back on a second stream, so a "
                          "step's copy-back overlaps the next render); CUDA events around the loop, less "
                          "the L2-flush writes between steps (their mean time alone), over K",
                "host_wall": {"value": rays * world / wall_s, "unit": "rays/s", "ms_per_step": wall_s * 1e3,
                              "timing": "host clock around call + copies + synchronize, one step at a time "
                                        "(median)"},
                "plan_host_wall": {"value": rays * world / plan_s, "unit": "rays/s", "ms_per_step": plan_s * 1e3,
                                   "timing": "RenderPlan: copies in, render, copy out replayed as one CUDA graph "
                                             "per call; host clock, one call at a time (median)"},
                "plan_pipelined": {"value": rays * world / pipe_s, "unit": "rays/s", "ms_per_step": pipe_s * 1e3,
                                   "steps": n_pipe,
                                   "timing": "RenderPlan.submit with two slots, each step's result taken after "
                                             "the next step is queued; CUDA events on the plan's stream, less the "
                                             "L2-flush writes between steps"}},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": cap["dram_bytes"] if cap_ok else None,
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read + write)",
                     "kernel": KERNEL.get(args.workload, "k_render"), "kernel_ms": kern_s * 1e3,
                     "flops_per_ray": F_RAY[args.workload],
                     "flops_note": "algorithmic: the reference's full evaluation per ray without early-out "
                                   "(obstruction tests the bundle culling skips are counted)",
                     "peak_source": "measured live: FP32 FMA-chain probe kernel (iact_probe_fma)",
                     "executed": {k: cap[k] for k in ("thread_inst_per_ray", "fma_pipe", "issue_active",
                                                      "shared_atomic_frac") if k in cap} if cap_ok else None,
                     "capture": ({"profile": cap["profile"], "digest": cap["digest"], "current": cap_ok}
                                 if cap else None)},
        "fwd_adjoint": fwdadj,
        "gpu_launches": n_launch,
        **({"culling": culling} if culling else {}),
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, tel, src_h, val_h, stype, mode)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
