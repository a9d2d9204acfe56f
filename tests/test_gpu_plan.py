"""RenderPlan: a forward render of fixed shape replayed as one CUDA graph
(host-to-device copies, the library's launches, device-to-host copy). Its
results equal render()'s for every call, with new inputs each time, also
when calls are pipelined through submit() over several slots."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-6  # FP32 shared-memory atomics land in varying order between launches


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("mode", ["image", "response"])
def test_plan_equals_render_call_after_call(cuda, mode):
    tel, src, val, st = W.plain_forward(n_samples=64, n_sources=6)
    plan = it.RenderPlan(tel, 6, st, mode=mode)
    fn = it.render_response_matrix if mode == "response" else it.render
    g = torch.Generator().manual_seed(3)
    for call in range(3):
        s = W.point_sources_disk(6, 2.5, 10 + call)
        v = torch.rand(6, generator=g) + 0.5
        got = plan(s, v)
        want = fn(tel, s, v, st).cpu()
        assert got.shape == want.shape and got.device.type == "cpu"
        assert _rel(got, want) <= TOL, f"call {call}: {_rel(got, want):.3g}"


def test_plan_extended_sources_and_buffers(cuda):
    from iactrace_gb300 import alignment as A
    pb = A.problem(n_facets=37, n_samples=32, n_sources=8, n_pixels=400)
    tel, src, val = pb["telescope"], pb["sources"].cpu(), pb["values"].cpu()
    plan = it.RenderPlan(tel, 8, "extended", seed=pb["seed"])
    want = it.render(tel, src, val, "extended", seed=pb["seed"]).cpu()
    out = torch.empty(want.shape)
    assert plan(src, val, out=out) is out and _rel(out, want) <= TOL
    shared = plan(src, val, copy=False)
    assert shared.is_pinned() and _rel(shared, want) <= TOL
    with pytest.raises(RuntimeError):
        plan(src[:4], val[:4])  # the plan's source count is fixed


def test_plan_submit_pipelines_calls(cuda):
    """Three slots: up to three renders queued at once, each result taken
    before its slot is submitted again; every result equals render()'s for
    its own inputs, in order."""
    tel, src, val, st = W.plain_forward(n_samples=64, n_sources=6)
    plan = it.RenderPlan(tel, 6, st, depth=3)
    g = torch.Generator().manual_seed(5)
    inputs = [(W.point_sources_disk(6, 2.5, 20 + k), torch.rand(6, generator=g) + 0.5) for k in range(8)]
    pending, got = [], []
    for s, v in inputs:
        if len(pending) == 3:
            got.append(pending.pop(0).result())
        pending.append(plan.submit(s, v))
    got += [t.result() for t in pending]
    for k, (s, v) in enumerate(inputs):
        want = it.render(tel, s, v, st).cpu()
        assert _rel(got[k], want) <= TOL, f"call {k}: {_rel(got[k], want):.3g}"


def test_plan_ticket_of_a_reused_slot_raises(cuda):
    tel, src, val, st = W.plain_forward(n_samples=64, n_sources=6)
    plan = it.RenderPlan(tel, 6, st, depth=2)
    t = plan.submit(src, val)
    t.result(copy=False)
    assert t.done()
    plan.submit(src, val)
    plan.submit(src, val)  # two slots: the second submit after t goes back to t's slot
    with pytest.raises(RuntimeError):
        t.result()
    with pytest.raises(ValueError):
        it.RenderPlan(tel, 6, st, depth=0)
