"""Batched adjoint (iact_batch_backward through BatchRenderer.backward)
against the single-scene adjoint of every job (iact_render_backward through
torch.autograd, itself checked against the FP64 twin and finite
differences). Same rays, same buckets; only the FP64 summation order of the
warp flushes differs: relative L2 per gradient block <= SAME_TOL; the
stage-mirror blocks go through FP32 shared-memory partial sums whose
grouping follows the tiling (which differs between a batch and a single
launch), so they are held to the gradient tolerance MIRROR_TOL."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import workloads as W

from gradref import gpu_grads
from test_gpu_batch import _mixed_jobs

SAME_TOL = 1e-5
MIRROR_TOL = 1e-4

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64).reshape(-1), np.asarray(b, np.float64).reshape(-1)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb else np.linalg.norm(a)


@pytest.mark.parametrize("mode", ["image", "response"])
def test_batch_backward_equals_single_backward(cuda, mode):
    tels, srcs, vals = _mixed_jobs()
    grads = ("rot", "pos", "scale", "src", "val", "mrot", "mpos", "msurf")
    b = it.BatchRenderer(tels, srcs, vals, "point", mode=mode, tune=False, backward=True, grads=grads)
    assert b.info()["adjoint_tiles"] > 0
    outs = b()
    rng = np.random.default_rng(4)
    gouts = [torch.as_tensor(rng.standard_normal(tuple(o.shape)), dtype=torch.float32) for o in outs]
    for rep in range(2):  # graph replays of the backward
        res = b.backward([g.to(cuda) for g in gouts])
        for i, (t, s, v) in enumerate(zip(tels, srcs, vals)):
            if s.shape[0] == 0:
                for k, x in res[i].items():
                    assert float(x.abs().sum()) == 0.0, (i, k)
                continue
            ref = gpu_grads(t, s, v, "point", gouts[i].numpy(), mode)
            for k in ("rot", "pos", "scale", "src", "val"):
                e = _rel(res[i][k].cpu().numpy(), ref[k])
                assert e <= SAME_TOL, f"replay {rep} job {i} d/d{k}: relative L2 {e:.3g}"
            if "mrot0" in ref:
                assert _rel(res[i]["mrot"].cpu().numpy(), ref["mrot0"]) <= MIRROR_TOL
                assert _rel(res[i]["mpos"].cpu().numpy(), ref["mpos0"]) <= MIRROR_TOL
                ms = res[i]["msurf"].cpu().numpy()[0]
                assert _rel(ms[0], ref["mc0"]) <= MIRROR_TOL and _rel(ms[1], ref["mk0"]) <= MIRROR_TOL
                na = ref["masph0"].size
                assert _rel(ms[2:2 + na], ref["masph0"]) <= MIRROR_TOL


def test_batch_backward_extended_soft_hex(cuda):
    from iactrace_gb300 import alignment as A
    pb = A.problem(n_facets=37, n_samples=16, n_sources=12, n_pixels=400, device=cuda)
    tel, src, val = pb["telescope"], pb["sources"], pb["values"]
    b = it.BatchRenderer([tel, tel], [src, src[:5]], [val, val[:5]], "extended", seeds=[3, 9], tune=False,
                         backward=True, grads=("rot", "val"))
    outs = b()
    g = [torch.randn(o.shape, device=cuda, generator=torch.Generator(device=cuda).manual_seed(i))
         for i, o in enumerate(outs)]
    res = b.backward(g)
    for i, (n, seed) in enumerate(((12, 3), (5, 9))):
        rot = tel.mirror_groups[0].rotations.clone().to(cuda).requires_grad_(True)
        v = val[:n].clone().requires_grad_(True)
        out = it.render(tel.set_mirror_rotations(0, rot), src[:n], v, "extended", seed=seed)
        (out * g[i]).sum().backward()
        assert _rel(res[i]["rot"].cpu().numpy(), rot.grad.cpu().numpy()) <= SAME_TOL
        assert _rel(res[i]["val"].cpu().numpy(), v.grad.cpu().numpy()) <= SAME_TOL
