"""A render's launches on the caller's stream.

A forward render queues k_prep (an ordinary launch), then the candidate-word
launch, the render kernel and k_finish, each after the first with
programmatic dependent launch: it may be scheduled while its predecessor
runs and waits for the predecessor's results before it reads them. These
tests check the order against the caller's own work on the same stream:
inputs written by the kernel queued right before the call and outputs read
by the kernel queued right after it, many calls deep without a synchronize.
They also check the library's launch counter (iact_kernel_launches).
"""
from __future__ import annotations

import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import _native as N, workloads as W

pytestmark = pytest.mark.gpu

TOL = 2e-6  # relative, per entry: a scaled copy of the same render (values are linear)


def _scene(n_samples=128, n_sources=8):
    tel, src, val, st = W.plain_forward(n_samples=n_samples, n_sources=n_sources)
    return tel, src.cuda(), val.cuda(), st


def _rel(a, b):
    return float((a.double() - b.double()).abs().max() / b.double().abs().max())


def test_forward_counts_its_launches(cuda):
    lib = N.load()
    tel, src, val, st = _scene()
    it.render(tel, src, val, st)
    torch.cuda.synchronize()
    n0 = lib.iact_kernel_launches()
    it.render(tel, src, val, st)
    # prep, candidate words, hard-pixel render, finish
    assert lib.iact_kernel_launches() - n0 == 4
    n0 = lib.iact_kernel_launches()
    it.render_response_matrix(tel, src, val, st)
    assert lib.iact_kernel_launches() - n0 == 4
    torch.cuda.synchronize()


def test_backward_counts_its_launches(cuda):
    lib = N.load()
    tel, src, val, st = _scene()
    v = val.clone().requires_grad_(True)
    out = it.render(tel, src, v, st)
    g = torch.ones_like(out)
    n0 = lib.iact_kernel_launches()
    out.backward(g)
    # prep, candidate words, hard-pixel adjoint, adjoint finish
    assert lib.iact_kernel_launches() - n0 == 4
    torch.cuda.synchronize()


def test_inputs_written_right_before_and_output_read_right_after(cuda):
    """Values scaled by k + 1 by a torch kernel queued just before call k;
    the output copied by a torch kernel just after it; a long fill before
    each write keeps the stream busy, so the host runs far ahead. A launch
    that read its inputs before the write, or a copy that read the output
    before the render finished, gives a wrongly scaled image."""
    tel, src, val, st = _scene(n_samples=256, n_sources=16)
    ref = it.render(tel, src, val, st).clone()
    torch.cuda.synchronize()
    busy = torch.empty(32 * 1024 * 1024, device="cuda")
    v = torch.empty_like(val)
    outs = []
    for k in range(6):
        busy.fill_(float(k))
        torch.mul(val, float(k + 1), out=v)
        o = it.render(tel, src, v, st)
        outs.append(o * 1.0)
    torch.cuda.synchronize()
    for k, o in enumerate(outs):
        assert _rel(o, ref * (k + 1)) < TOL, f"call {k}"


def test_back_to_back_calls_share_nothing(cuda):
    """Forward renders of different values, response matrices and an
    adjoint queued back to back on one stream without a synchronize each
    equal the same call made alone."""
    tel, src, val, st = _scene()
    alone_img = it.render(tel, src, val, st).clone()
    alone_rsp = it.render_response_matrix(tel, src, val, st).clone()
    vg = val.clone().requires_grad_(True)
    it.render(tel, src, vg, st).sum().backward()
    alone_g = vg.grad.clone()
    torch.cuda.synchronize()
    imgs, rsps, grads = [], [], []
    for k in range(4):
        imgs.append(it.render(tel, src, val * (k + 1), st))
        rsps.append(it.render_response_matrix(tel, src, val * (k + 1), st))
        vk = (val * (k + 1)).detach().requires_grad_(True)
        it.render(tel, src, vk, st).sum().backward()
        grads.append(vk.grad)
    torch.cuda.synchronize()
    for k in range(4):
        assert _rel(imgs[k], alone_img * (k + 1)) < TOL
        assert _rel(rsps[k], alone_rsp * (k + 1)) < TOL
        # dL/dv of L = sum(image) is R 1 / 1 per source: independent of the values
        assert _rel(grads[k], alone_g) < 1e-5
