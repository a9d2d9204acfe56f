"""Batched persistent render (iact_batch_* through BatchRenderer) against the
single-job path and the FP64 oracle.

Every job of a batch must give what iact_render gives for it alone (same
rays, same bins; only the FP64 summation order of the tile flushes differs:
relative L2 <= SAME_TOL), through plain launches and CUDA-graph replays,
across template classes (hard / soft sensors, scenes with later mirror
stages), ragged sizes (1 source, empty jobs) and in-place input updates.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import Telescope, workloads as W
from iactrace_gb300.core import autotune as AT

from test_gpu_forward import check_image

SAME_TOL = 1e-6

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = a.double().cpu().reshape(-1), b.double().cpu().reshape(-1)
    nb = float(b.norm())
    return float((a - b).norm()) / nb if nb else float(a.norm())


def _mixed_jobs():
    """Ragged jobs over all four template classes."""
    from iactrace_gb300 import DifferentiableHexagonalSensor, SquareSensor
    tels, srcs, vals, _ = W.ragged_batch(n_instances=5, n_samples=48, seed=3, max_facets=300, min_facets=40,
                                         max_sources=64, pixels=(960, 2048))
    g0 = tels[0].mirror_groups[0]
    sq = SquareSensor([0, 0, 15.0], [0, 0, 0], 32, 30, (-0.672, 0.672, -0.63, 0.63))
    soft = DifferentiableHexagonalSensor([0, 0, 15.0], [0, 0, 0], W.hex_grid(960, 0.042), sigma=0.5)
    tels.append(Telescope([g0], tels[0].obstruction_groups, [sq]))
    srcs.append(W.point_sources_disk(1, 2.0, 41))  # a single source
    vals.append(torch.ones(1))
    tels.append(Telescope([g0], tels[0].obstruction_groups, [soft]))
    srcs.append(W.point_sources_disk(7, 2.0, 42))
    vals.append(torch.rand(7) + 0.5)
    tels.append(Telescope([g0], tels[0].obstruction_groups, [W.hex_camera(960)]))
    srcs.append(torch.zeros((0, 3)))  # an empty job
    vals.append(torch.zeros(0))
    ct, cs, cv, _ = W.cassegrain(n_samples=32, n_sources=9)  # later mirror stage
    tels.append(ct)
    srcs.append(cs)
    vals.append(cv)
    return tels, srcs, vals


@pytest.mark.parametrize("mode", ["image", "response"])
def test_batch_equals_single_renders(cuda, mode):
    tels, srcs, vals = _mixed_jobs()
    b = it.BatchRenderer(tels, srcs, vals, "point", mode=mode, tune=False)
    info = b.info()
    assert info["jobs"] == len(tels) and info["classes"] == 3
    fn = it.render_response_matrix if mode == "response" else it.render
    for rep in range(2):  # graph replays
        outs = b()
        for i, (t, s, v) in enumerate(zip(tels, srcs, vals)):
            ref = fn(t, s, v, "point")
            assert outs[i].shape == ref.shape
            if ref.numel() == 0 or float(ref.abs().sum()) == 0:
                assert float(outs[i].abs().sum()) == 0.0, f"job {i}"
                continue
            err = _rel(outs[i], ref)
            assert err <= SAME_TOL, f"replay {rep} job {i}: relative L2 {err:.3g} against render()"


def test_batch_job_against_oracle(cuda):
    """One batched job through the forward parity check of the oracle."""
    tel, src, val, st = W.plain_forward(n_samples=128, n_sources=8)
    b = it.BatchRenderer([tel, tel], [src, src[:3]], [val, val[:3]], st, tune=False)
    out = b()
    cont, raw, stats = check_image(tel, src, val, st)  # the single-job path against FP64
    assert _rel(out[0], it.render(tel, src, val, st)) <= SAME_TOL
    assert _rel(out[1], it.render(tel, src[:3], val[:3], st)) <= SAME_TOL
    print(f"batch job: cont {cont:.2e} raw {raw:.2e} {stats}")


def test_batch_inplace_updates_and_no_graph(cuda):
    tels, srcs, vals, st = W.ragged_batch(n_instances=4, n_samples=32, seed=5, max_facets=200, min_facets=50,
                                          max_sources=32)
    b = it.BatchRenderer(tels, srcs, vals, st, tune=False, graph=True)
    nog = it.BatchRenderer(tels, srcs, vals, st, tune=False, graph=False)
    first = [o.clone() for o in b()]
    for o, r in zip(nog(), first):
        assert _rel(o, r) <= SAME_TOL
    # new sources and facet tilts written in place, then one replay
    new_src = [W.point_sources_disk(s.shape[0], 1.0, 77 + i) for i, s in enumerate(srcs)]
    for i in range(len(tels)):
        b.sources[i].copy_(new_src[i])
        b.facet_rotations[i][:, 0] += 0.01
    outs = b()
    for i, t in enumerate(tels):
        rot = t.mirror_groups[0].rotations.clone()
        rot[:, 0] += 0.01
        ref = it.render(t.set_mirror_rotations(0, rot), new_src[i], vals[i], st)
        assert _rel(outs[i], ref) <= SAME_TOL, i
        assert _rel(outs[i], first[i]) > 1e-3  # the update took effect


def test_batch_extended_sources_soft_hex(cuda):
    from iactrace_gb300 import alignment as A
    pb = A.problem(n_facets=37, n_samples=16, n_sources=12, n_pixels=400, device=cuda)
    tel, src, val = pb["telescope"], pb["sources"], pb["values"]
    b = it.BatchRenderer([tel, tel], [src, src[:5]], [val, val[:5]], "extended", seeds=[3, 9], tune=False)
    out = b()
    assert _rel(out[0], it.render(tel, src, val, "extended", seed=3)) <= SAME_TOL
    assert _rel(out[1], it.render(tel, src[:5], val[:5], "extended", seed=9)) <= SAME_TOL


def test_autotuner_picks_and_caches(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("IACTRACE_TUNE_CACHE", str(tmp_path / "tune.json"))
    AT._mem.clear()
    tels, srcs, vals, st = W.ragged_batch(n_instances=6, n_samples=32, seed=7, max_facets=200, min_facets=50,
                                          max_sources=64)
    b = it.BatchRenderer(tels, srcs, vals, st, tune=True)
    rec = AT.last_result(b)
    assert rec is not None and len(rec["tried"]) >= 6
    assert (tmp_path / "tune.json").exists()
    assert list(rec["knobs"]) == [b.opts.block_threads, b.opts.tasks_per_warp, b.opts.hist_mode]
    ref = it.BatchRenderer(tels, srcs, vals, st, tune=False)()
    for o, r in zip(b(), ref):
        assert _rel(o, r) <= SAME_TOL
    AT._mem.clear()  # second batch of the same shape: served from the file
    b2 = it.BatchRenderer(tels, srcs, vals, st, tune=True, graph=False)
    assert [b2.opts.block_threads, b2.opts.tasks_per_warp, b2.opts.hist_mode] == list(rec["knobs"])
