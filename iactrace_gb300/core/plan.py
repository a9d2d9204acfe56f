"""Prepared renders for latency-bound callers: one CUDA graph per call.

A forward render of a small scene (the plain-forward configuration: 6e6
rays, ~90 us of GPU work) costs a caller who waits for each result more in
host-side issue and synchronisation than on the GPU: argument handling,
three kernel launches, the copies of the inputs and of the image. A
RenderPlan fixes what a sequence of such calls shares -- the telescope, the
sensor, the mode, the source type and the number of sources -- and captures
the whole call once in a CUDA graph: the copy of the sources and values
from pinned host staging buffers, the render (prep, render and finish
launches of iact_render) and the copy of the result back to a pinned host
buffer. Each call then fills the staging buffers on the host, replays the
graph and waits for it.

A caller that can take results a few calls late (an acquisition loop that
queues the next frame before it reads the last one) submits instead:
submit() fills the staging buffers of the next of `depth` slots, replays
that slot's graph on the plan's stream and returns a ticket at once;
ticket.result() waits for that replay alone. The host fills slot k + 1
while the GPU renders slot k, so the call rate is set by the GPU, not by
the host's issue and synchronisation. Each slot has its own staging and
device buffers and graph; the graphs share one memory pool, which their
replays, serialised on the plan's stream, never use at the same time.

The plan reads the telescope's device tables at the addresses it had when
the plan was made: edits of the telescope after that (new sample arrays,
moved facets, a different sensor) need a new plan.
"""
from __future__ import annotations

import math

import torch

from .. import _native as N
from .render import _launch


class RenderPlan:
    """telescope(sources, values) for a fixed shape, replayed as one CUDA graph.

    plan = RenderPlan(tel, n_sources, source_type="point", sensor_idx=0, mode="image")
    image = plan(sources, values)   # host tensors in, host tensor out
    ticket = plan.submit(sources, values)   # queued: returns at once
    image = ticket.result()                 # waits for that call alone

    mode: "image" (the sensor's accumulator shape) or "response"
    (n_sources x n_pixels). sources: (n_sources, 3) (4 for "extended"),
    values: (n_sources,), anything torch.as_tensor accepts; the result is a
    float32 CPU tensor of its own (not reused by the next call) unless
    `out` is given or copy=False (then the slot's pinned buffer, valid until
    the slot is submitted again). depth: slots of staging buffers and
    graphs; a ticket's result can be taken until `depth` further submits
    (the next submit into its slot waits for its replay and then reuses the
    slot: taking the result after that raises). A plan serves one caller at
    a time: two threads calling it at once race on its staging buffers.
    """

    def __init__(self, tel, n_sources: int, source_type: str = "point", sensor_idx: int = 0, mode: str = "image",
                 seed: int = 0, device=None, depth: int = 1):
        if not torch.cuda.is_available():
            raise RuntimeError("RenderPlan needs a CUDA device")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if mode not in ("image", "response"):
            raise ValueError("mode must be 'image' or 'response'")
        if int(depth) < 1:
            raise ValueError("depth must be at least 1")
        self.tel, self.source_type, self.sensor_idx, self.seed = tel, source_type, int(sensor_idx), int(seed)
        self.mode = N.MODE_RESPONSE if mode == "response" else N.MODE_IMAGE
        self.n_sources = S = int(n_sources)
        self.width = 4 if source_type == "extended" else 3
        sensor = tel.sensors[self.sensor_idx]
        P = int(math.prod(sensor.get_accumulator_shape()))
        self.shape = (S, P) if self.mode == N.MODE_RESPONSE else tuple(sensor.get_accumulator_shape())
        self.stream = torch.cuda.Stream(self.device)
        self.stream.wait_stream(torch.cuda.current_stream(self.device))
        self.slots = []
        pool = None
        for _ in range(int(depth)):
            slot = _Slot(self)
            with torch.cuda.device(self.device), torch.cuda.stream(self.stream), torch.no_grad():
                for _ in range(2):  # packs the scene, fills the launch caches, warms the allocator
                    self._body(slot)
            self.stream.synchronize()
            with torch.cuda.device(self.device), torch.no_grad(), \
                    torch.cuda.graph(slot.graph, stream=self.stream, pool=pool):
                slot.out_d = self._body(slot)
            pool = slot.graph.pool() if pool is None else pool
            self.slots.append(slot)
        self._next = 0

    def _body(self, slot):
        slot.src_d.copy_(slot.src_h, non_blocking=True)
        slot.val_d.copy_(slot.val_h, non_blocking=True)
        out = _launch(self.tel, slot.src_d, slot.val_d, self.source_type, self.sensor_idx, self.mode, None,
                      self.seed)
        slot.out_h.copy_(out, non_blocking=True)
        return out

    def submit(self, sources, values) -> "RenderTicket":
        """Queue a render of these sources; returns a ticket at once. Waits
        only when the next slot's previous replay is still running."""
        slot = self.slots[self._next]
        src = torch.as_tensor(sources, dtype=torch.float32).reshape(slot.src_h.shape)
        val = torch.as_tensor(values, dtype=torch.float32).reshape(slot.val_h.shape)
        self._next = (self._next + 1) % len(self.slots)
        slot.done.synchronize()  # its previous replay has read the staging buffers and written out_h
        slot.gen += 1
        slot.src_h.copy_(src)
        slot.val_h.copy_(val)
        with torch.cuda.stream(self.stream):
            slot.graph.replay()
            slot.done.record(self.stream)
        return RenderTicket(slot, slot.gen)

    def __call__(self, sources, values, out=None, copy=True):
        """Render these sources: copy them in, replay the graph, wait, return
        the result: a new CPU tensor, `out` if given, or with copy=False the
        slot's own pinned buffer, which the slot's next use overwrites."""
        return self.submit(sources, values).result(out=out, copy=copy)

    def h2d_bytes(self) -> int:
        return self.n_sources * self.width * 4 + self.n_sources * 4

    def d2h_bytes(self) -> int:
        return int(math.prod(self.shape)) * 4


class _Slot:
    """Staging buffers, device inputs, graph and completion event of one slot."""

    def __init__(self, plan):
        S, width, dev = plan.n_sources, plan.width, plan.device
        self.src_h = torch.zeros((S, width), dtype=torch.float32).pin_memory()
        self.val_h = torch.zeros((S,), dtype=torch.float32).pin_memory()
        self.out_h = torch.zeros(plan.shape, dtype=torch.float32).pin_memory()
        self.src_d = torch.zeros((S, width), dtype=torch.float32, device=dev)
        self.val_d = torch.zeros((S,), dtype=torch.float32, device=dev)
        self.graph = torch.cuda.CUDAGraph()
        self.done = torch.cuda.Event()
        self.gen = 0
        self.out_d = None


class RenderTicket:
    """A render queued by RenderPlan.submit."""

    def __init__(self, slot, gen):
        self._slot, self._gen = slot, gen

    def done(self) -> bool:
        """True once the render and the copy of its result have finished."""
        self._check()
        return self._slot.done.query()

    def result(self, out=None, copy=True):
        """Wait for this render and return its result (see RenderPlan)."""
        self._check()
        self._slot.done.synchronize()
        if out is not None:
            out.copy_(self._slot.out_h)
            return out
        return self._slot.out_h.clone() if copy else self._slot.out_h

    def _check(self):
        if self._slot.gen != self._gen:
            raise RuntimeError("RenderTicket: its slot has been submitted again; the result is gone "
                               "(take results within `depth` submits)")
