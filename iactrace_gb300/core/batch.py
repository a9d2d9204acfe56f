"""Batched persistent render of many telescope variants (iact_batch_* C ABI).

The reference renders variants one ``Telescope.__call__``
(telescope/telescope.py:56-83) at a time. ``BatchRenderer`` packs every
(telescope, sources, values) job once, plans one persistent kernel per
template class over a global tile queue, and replays the whole batch as one
CUDA graph. Per-job results equal ``render`` / ``render_response_matrix`` of
that job up to FP64 summation order.

Inputs stay bound to the batch: to render new parameters, write them into
the batch's own tensors (``sources[i]``, ``values[i]``, ``facet_rotations[i]``
...) in place and call the batch again.

With ``backward=True`` the batch also runs the adjoint of every job in one
persistent launch (``iact_batch_backward``): write dL/d(out) into
``grad_outs[i]`` and call ``backward()``; the gradients land in ``grads[i]``
(facet rotations and positions, roughness scales, sources, values, stage
mirrors, as requested).
"""
from __future__ import annotations

import ctypes
import math

import torch

from .. import _native as N
from .render import _device, _inputs, source_code
from .scene import pack_scene, primary_params, stages_of


class BatchRenderer:
    """Render jobs ``(telescopes[i], sources[i], values[i])`` in one launch.

    mode: "image" (out[i] has the sensor's accumulator shape) or "response"
    (out[i] is (S_i, P_i)). opts: an ``IactOpts`` (block_threads,
    tasks_per_warp, hist_mode); None runs the autotuner when ``tune`` is set,
    else the library defaults. graph: capture the launch in a CUDA graph.
    """

    GRADS = ("rot", "pos", "scale", "src", "val", "mrot", "mpos", "msurf")

    def __init__(self, telescopes, sources, values, source_type="point", mode="image", sensor_idx=0, opts=None,
                 seeds=None, graph=True, tune=True, device=None, backward=False, grads=("rot", "pos", "src", "val")):
        if not (len(telescopes) == len(sources) == len(values)):
            raise ValueError("telescopes, sources and values must have the same length")
        self.device = torch.device(device) if device is not None else _device()
        self.lib = N.load()
        self.code = source_code(source_type)
        self.mode = N.MODE_RESPONSE if mode == "response" else N.MODE_IMAGE
        n = len(telescopes)
        self.sources, self.values, self.outs = [], [], []
        self.facet_rotations, self.facet_positions, self.facet_scales = [], [], []
        self._keep = []
        self._jobs = (N.IactJob * max(n, 1))()
        self._descs = []
        shapes = []
        for i, tel in enumerate(telescopes):
            if 0 not in stages_of(tel):
                raise ValueError(f"job {i}: telescope has no primary mirror")
            sensor = tel.sensors[sensor_idx]
            src, val = _inputs(sources[i], values[i], self.device, source_type)
            S = int(src.shape[0])
            P = int(math.prod(sensor.get_accumulator_shape()))
            shape = (S, P) if self.mode == N.MODE_RESPONSE else tuple(sensor.get_accumulator_shape())
            out = torch.empty(shape, dtype=torch.float32, device=self.device)
            # the batch owns its facet transforms (written in place by callers)
            rot, pos, scale = (t.detach().clone().contiguous() for t in primary_params(tel, self.device))
            ps = pack_scene(tel, self.device, (rot, pos, scale))
            desc = N.IactScene()
            ctypes.memmove(ctypes.addressof(desc), ctypes.addressof(ps.desc), ctypes.sizeof(desc))
            sdesc, keep = sensor.pack(self.device)
            self._keep += [ps, keep, sdesc]
            self._descs.append(desc)
            self.sources.append(src)
            self.values.append(val)
            self.outs.append(out)
            self.facet_rotations.append(rot)
            self.facet_positions.append(pos)
            self.facet_scales.append(scale)
            shapes.append((ps.F, ps.M, S, P, int(sensor.kind), ps.n_mirrors))
            J = self._jobs[i]
            J.scene = ctypes.pointer(desc)
            J.sensor = ctypes.pointer(sdesc)
            J.sources, J.values, J.n_sources = src.data_ptr(), val.data_ptr(), S
            J.seed = int(seeds[i]) & 0xFFFFFFFF if seeds is not None else 0
            J.out = out.data_ptr()
        self.backward_enabled = bool(backward)
        self.grad_outs, self.grads = [], []
        if backward:
            unknown = set(grads) - set(self.GRADS)
            if unknown:
                raise ValueError(f"unknown gradient names {sorted(unknown)}")
            for i in range(n):
                F, M, S, P, kind, nm = shapes[i]
                go = torch.zeros_like(self.outs[i])
                shp = {"rot": (F, 3), "pos": (F, 3), "scale": (F,), "src": (S, 3), "val": (S,), "mrot": (nm, 3),
                       "mpos": (nm, 3), "msurf": (nm, 2 + N.IACT_MAX_ASPH)}
                gi = {k: torch.zeros(shp[k], device=self.device) for k in grads
                      if not (k == "src" and self.code == N.SRC_EXTENDED) and not (k[0] == "m" and nm == 0)}
                self.grad_outs.append(go)
                self.grads.append(gi)
                J = self._jobs[i]
                J.grad_out = go.data_ptr()
                ptr = lambda k: gi[k].data_ptr() if k in gi else None
                J.g_facet_rot, J.g_facet_pos, J.g_facet_scale = ptr("rot"), ptr("pos"), ptr("scale")
                J.g_sources, J.g_values = ptr("src"), ptr("val")
                J.g_mirror_rot, J.g_mirror_pos, J.g_mirror_surface = ptr("mrot"), ptr("mpos"), ptr("msurf")
        self.n_jobs = n
        self.rays = sum(F * M * S for F, M, S, *_ in shapes)
        self.signature = (self.mode, self.code, tuple(shapes))
        self._handle = None
        self._ws = None
        self._graph = None
        self._bgraph = None
        if opts is None and tune:
            from .autotune import tune_batch
            opts = tune_batch(self)
        self.opts = opts
        self._build(opts)
        if graph:
            self.capture()

    # ---------------------------------------------------------------- plumbing
    def _create(self, opts):
        h = ctypes.c_void_p()
        if self.backward_enabled:
            o = N.IactOpts()
            if opts is not None:
                ctypes.memmove(ctypes.addressof(o), ctypes.addressof(opts), ctypes.sizeof(o))
            o.flags |= N.FLAG_BATCH_BACKWARD
            opts = o
        N.check(self.lib.iact_batch_create(self._jobs, self.n_jobs, self.code, self.mode,
                                           ctypes.byref(opts) if opts is not None else None, ctypes.byref(h)))
        size = ctypes.c_size_t(0)
        N.check(self.lib.iact_batch_workspace_size(h, ctypes.byref(size)))
        ws = torch.empty(max(int(size.value), 256), dtype=torch.uint8, device=self.device)
        stream = torch.cuda.current_stream(self.device)
        N.check(self.lib.iact_batch_prepare(h, ws.data_ptr(), ws.numel(), stream.cuda_stream))
        return h, ws

    def _build(self, opts):
        self.release()
        self._handle, self._ws = self._create(opts)

    def launch(self, stream=None):
        """Queue one render of every job on `stream` (default: current stream)."""
        stream = stream or torch.cuda.current_stream(self.device)
        N.check(self.lib.iact_batch_render(self._handle, stream.cuda_stream))

    def launch_backward(self, stream=None):
        """Queue the adjoint of every job on `stream` (default: current stream)."""
        if not self.backward_enabled:
            raise RuntimeError("create the BatchRenderer with backward=True")
        stream = stream or torch.cuda.current_stream(self.device)
        N.check(self.lib.iact_batch_backward(self._handle, stream.cuda_stream))

    def _capture(self, fn):
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            fn(side)  # first launch outside the capture
        torch.cuda.current_stream(self.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn(None)
        return g

    def capture(self):
        """Capture the batch's launch sequences (forward, backward) in CUDA graphs."""
        self._graph = self._capture(self.launch)
        if self.backward_enabled:
            self._bgraph = self._capture(self.launch_backward)

    def backward(self, grad_outs=None):
        """Adjoint of every job: dL/d(out_i) from `grad_outs` (copied into the
        bound tensors) or from the bound ``grad_outs`` as they are; returns
        the list of gradient dicts (owned by the batch)."""
        if grad_outs is not None:
            for dst, src in zip(self.grad_outs, grad_outs):
                dst.copy_(src)
        if self._bgraph is not None:
            self._bgraph.replay()
        else:
            self.launch_backward()
        return self.grads

    def __call__(self):
        """Render every job; returns the list of outputs (owned by the batch)."""
        if self._graph is not None:
            self._graph.replay()
        else:
            self.launch()
        return self.outs

    def info(self) -> dict:
        v = (ctypes.c_int64 * 7)()
        N.check(self.lib.iact_batch_info(self._handle, v, 7))
        return {"jobs": v[0], "tiles": v[1], "rays": v[2], "launches": v[3], "classes": v[4],
                "adjoint_tiles": v[5], "backward_launches": v[6]}

    def release(self):
        if self._handle is not None:
            self._graph = None
            self._bgraph = None
            self.lib.iact_batch_destroy(self._handle)
            self._handle = None
            self._ws = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass
