"""Parity at the full sizes of the benchmark workloads.

The other GPU tests compare every ray of small scenes with the FP64 oracle.
These run the scenes at the sizes the bench measures and check what holds
at any size:

* plain forward (380 facets x 1000 samples x 16 point sources, 6.08e6 rays,
  32 x 30 square camera) and the two-mirror Cassegrain (61 segments x 500
  samples x 64 sources, 1.95e6 rays): every ray and the image against the
  FP64 oracle, with the forward tests' tolerances (the oracle runs these in
  seconds on the host cores);
* response matrix (4096 point sources x 380 facets x 256 samples, 3.98e8
  rays, 4096 x 2048):
  - the raw relative L2 error against the FP64 oracle's full matrix;
  - rows of a spread of sources against the FP64 ray values binned with the
    GPU's decisions (a point source's rays do not depend on the others);
  - rows sum to the image of the same rays;
  - a source subset, or the sources in reverse order, gives the same rows
    through other tiles;
  - doubling the values doubles the matrix;
  - the adjoint's value gradient of sum(g * R) equals (R * g).sum(1) / v;
* ragged batch (64 variants, 5.2e9 rays): one batched launch gives each
  variant's single render;
* alignment (876 facets x 128 samples x 256 extended sources, 2048 soft
  hexagons, 2.87e7 rays): the image against the FP64 oracle's replay of the
  same jitter stream, and the value-gradient identity through the soft
  response matrix.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import alignment as A
from iactrace_gb300 import workloads as W

from test_gpu_forward import IMG_TOL, RAW_TOL, check_image, check_rays, cont_values, rebin

SAME_TOL = 1e-6  # same rays and bins, other summation order (tiles, batch)
GRAD_TOL = 1e-4  # gradients against their linear identity
SOFT_TOL = 1e-5  # soft-sensor images against the FP64 oracle (the image gate: 1e-5 against FP64)

pytestmark = pytest.mark.gpu


def _oracle():
    import oracle.oracle as O
    return O


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_full_plain_forward_every_ray(cuda):
    tel, src, val, st = W.plain_forward()
    assert tel.mirror_groups[0].n_samples == 1000 and src.shape[0] == 16
    cont, raw, stats = check_image(tel, src, val, st)
    assert stats["rays"] == 380 * 16 * 1000
    print(f"plain full: cont {cont:.2e} raw {raw:.2e} {stats}")


def test_full_cassegrain_every_ray(cuda):
    tel, src, val, st = W.cassegrain()
    assert src.shape[0] == 64 and tel.mirror_groups[0].n_samples == 500
    cont, raw, stats = check_image(tel, src, val, st)
    print(f"cassegrain full: cont {cont:.2e} raw {raw:.2e} {stats}")


@pytest.fixture(scope="module")
def response_full(cuda):
    tel, src, val, st = W.response_matrix()
    assert src.shape[0] == 4096 and tel.sensors[0].n_pixels == 2048
    R = it.render_response_matrix(tel, src, val, st)
    return tel, src, val, st, R


def test_full_response_against_oracle(response_full):
    O = _oracle()
    tel, src, val, st, R = response_full
    ref = O.render(tel, src, val, st, 0, mode="response", threads=O.max_threads())
    raw = _rel(R.cpu().numpy(), ref)
    assert raw <= RAW_TOL, f"raw error {raw:.3g} of the full response matrix"
    # rows of sources spread over the grid, against the FP64 ray values
    # binned with the GPU's own decisions for those sources
    idx = torch.arange(0, 4096, 585)
    sub_src, sub_val = src[idx], val[idx]
    g, o, stats = check_rays(tel, sub_src, sub_val, st)
    M = tel.mirror_groups[0].n_samples
    ref_cont = rebin(g["pix"], cont_values(g, o), R.shape[1], len(idx), M)
    cont = _rel(R[idx.to(R.device)].cpu().numpy(), ref_cont)
    assert cont <= IMG_TOL, f"rows {idx.tolist()}: image error {cont:.3g} ({stats})"
    print(f"response full: raw {raw:.2e}, rows cont {cont:.2e} {stats}")


def test_full_response_properties(response_full):
    tel, src, val, st, R = response_full
    Rd = R.double()
    img = it.render(tel, src, val, st).double()
    assert _rel(Rd.sum(0).cpu(), img.cpu()) <= SAME_TOL
    sub = slice(1000, 1500)  # not aligned to any tile's source block
    Rs = it.render_response_matrix(tel, src[sub], val[sub], st).double()
    assert _rel(Rs.cpu(), Rd[sub].cpu()) <= SAME_TOL
    Rr = it.render_response_matrix(tel, src.flip(0), val.flip(0), st).double()
    assert _rel(Rr.flip(0).cpu(), Rd.cpu()) <= SAME_TOL
    R2 = it.render_response_matrix(tel, src, 2.0 * val, st).double()
    assert _rel(R2.cpu(), (2.0 * Rd).cpu()) <= SAME_TOL


def test_full_response_value_gradient(response_full):
    tel, src, val, st, R = response_full
    gen = torch.Generator(device=R.device).manual_seed(0)
    g = torch.randn(R.shape, device=R.device, generator=gen)
    v = val.clone().to(R.device).requires_grad_(True)
    (it.render_response_matrix(tel, src, v, st) * g).sum().backward()
    want = (R.double() * g.double()).sum(1) / val.to(R.device).double()
    err = _rel(v.grad.double().cpu(), want.cpu())
    assert err <= GRAD_TOL, f"dL/dvalues vs (R g)/v: {err:.3g}"


def test_full_ragged_batch_equals_single_renders(cuda):
    tels, srcs, vals, st = W.ragged_batch()
    assert len(tels) == 64
    b = it.BatchRenderer(tels, srcs, vals, st, tune=False)
    outs = b()
    worst = 0.0
    for i in range(len(tels)):
        one = it.render(tels[i], srcs[i], vals[i], st).double().cpu()
        if float(one.abs().sum()) == 0.0:
            assert float(outs[i].abs().sum()) == 0.0, f"instance {i}"
            continue
        worst = max(worst, _rel(outs[i].double().cpu(), one))
    assert worst <= SAME_TOL, f"batched vs single renders: {worst:.3g}"


def test_full_alignment_image_and_value_gradient(cuda):
    O = _oracle()
    pb = A.problem()
    tel, src, val, seed = pb["telescope"], pb["sources"], pb["values"], pb["seed"]
    assert tel.mirror_groups[0].n_samples == 128 and src.shape[0] == 256
    img = it.render(tel, src, val, "extended", seed=seed).double().cpu().numpy()
    ref = O.render(tel, src.cpu(), val.cpu(), "extended", 0, seed=seed, threads=O.max_threads())
    err = _rel(img, ref)
    assert err <= SOFT_TOL, f"alignment image vs FP64 oracle: {err:.3g}"
    R = it.render_response_matrix(tel, src, val, "extended", seed=seed)
    assert _rel(R.double().sum(0).cpu(), img) <= SAME_TOL
    gen = torch.Generator(device=R.device).manual_seed(1)
    g = torch.randn(R.shape, device=R.device, generator=gen)
    v = val.clone().requires_grad_(True)
    (it.render_response_matrix(tel, src, v, "extended", seed=seed) * g).sum().backward()
    want = (R.double() * g.double()).sum(1) / val.double()
    gerr = _rel(v.grad.double().cpu(), want.cpu())
    assert gerr <= GRAD_TOL, f"dL/dvalues vs (R g)/v: {gerr:.3g}"
    print(f"alignment full: image {err:.2e}, value gradient {gerr:.2e}")
