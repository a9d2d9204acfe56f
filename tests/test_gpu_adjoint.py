"""The adjoint kernel (iact_render_backward behind torch.autograd) against
central finite differences of the FP64 oracle.

jax.grad of the reference's render sees pixel ids and shadow masks as
constants. The finite differences here therefore hold each ray's FP64 pixel
id fixed (hard sensors: L(theta) = sum_rays g[pix_ray] val_ray(theta)) and
drop rays whose shadow state changes inside +-h. Soft sensors are
differentiated through the full FP64 image. Tolerance: relative L2 error of
each gradient block <= GRAD_TOL.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import Telescope, workloads as W

GRAD_TOL = 1e-4

pytestmark = pytest.mark.gpu


def _oracle():
    import oracle.oracle as O
    return O


def small_dish(camera, seed=2, n_samples=48, roughness=24.0):
    groups, obst = W.davies_cotton(n_facets=19, n_samples=n_samples, seed=seed)
    # a mast and the camera box that shadow part of this small dish
    from iactrace_gb300.core import Box, Cylinder, group_obstructions
    obst = group_obstructions([Cylinder([1.6, 0.4, 0.2], [0.3, 0.1, 15.4], 0.05),
                               Box([-0.3, -0.3, 15.0], [0.3, 0.3, 16.0])])
    tel = Telescope(groups, obst, [camera])
    return tel.apply_roughness(roughness) if roughness else tel


def grads_gpu(tel, src, val, st, g, mode="image"):
    grp = tel.mirror_groups[0]
    rot = grp.rotations.clone().cuda().requires_grad_(True)
    pos = grp.positions.clone().cuda().requires_grad_(True)
    sc = grp.perturbation_scale.clone().cuda().requires_grad_(True)
    t2 = tel.set_mirror_rotations(0, rot).set_mirror_positions(0, pos)
    t2.mirror_groups[0] = t2.mirror_groups[0].replace(perturbation_scale=sc)
    s = src.clone().cuda().requires_grad_(True)
    v = val.clone().cuda().requires_grad_(True)
    fn = it.render_response_matrix if mode == "response" else it.render
    out = fn(t2, s, v, st)
    (out.double() * torch.as_tensor(g, device="cuda").reshape(out.shape)).sum().backward()
    return {k: x.grad.double().cpu().numpy() for k, x in
            (("rot", rot), ("pos", pos), ("scale", sc), ("src", s), ("val", v))}


class FD:
    """Central differences of the FP64 oracle with the unperturbed discrete decisions."""

    def __init__(self, tel, src, val, st, g, mode="image", soft=False):
        self.O = _oracle()
        self.tel, self.src, self.val, self.st, self.mode, self.soft = tel, src, val, st, mode, soft
        self.g = np.asarray(g, np.float64)
        d = self.O.render_debug(tel, src, val, st, 0, "f64")
        self.pix0, self.zero0 = d["pix"], d["vals"] == 0
        S, M = src.shape[0], tel.mirror_groups[0].n_samples
        self.s_idx = (np.arange(self.pix0.size) // M) % S
        P = self.g.size // (S if mode == "response" else 1)
        self.P = P

    def loss(self, tel, src, val):
        if self.soft:
            img = self.O.render(tel, src, val, self.st, 0, mode=self.mode)
            return float((img.reshape(-1) * self.g).sum()), None
        d = self.O.render_debug(tel, src, val, self.st, 0, "f64")
        gv = np.where(self.pix0 >= 0, self.g[np.where(self.pix0 >= 0, self.pix0, 0) +
                                                (self.s_idx * self.P if self.mode == "response" else 0)], 0.0)
        return d["vals"], gv

    def diff(self, tel_p, src_p, val_p, tel_m, src_m, val_m):
        lp, gp = self.loss(tel_p, src_p, val_p)
        lm, _ = self.loss(tel_m, src_m, val_m)
        if self.soft:
            return lp - lm
        ok = ((lp == 0) == self.zero0) & ((lm == 0) == self.zero0)  # no shadow flip within +-h
        return float(((lp - lm) * gp * ok).sum())

    def grad(self, which, idx_list, h):
        out = []
        grp = self.tel.mirror_groups[0]
        for idx in idx_list:
            def moved(sign):
                if which in ("rot", "pos", "scale"):
                    base = {"rot": grp.rotations, "pos": grp.positions, "scale": grp.perturbation_scale}[which]
                    t = base.clone()
                    t.view(-1)[idx] = float(t.view(-1)[idx]) + sign * h
                    actual = float(t.view(-1)[idx])
                    if which == "rot":
                        tel = self.tel.set_mirror_rotations(0, t)
                    elif which == "pos":
                        tel = self.tel.set_mirror_positions(0, t)
                    else:
                        tel = Telescope([grp.replace(perturbation_scale=t)], self.tel.obstruction_groups,
                                        self.tel.sensors)
                    return tel, self.src, self.val, actual
                t = (self.src if which == "src" else self.val).clone()
                t.view(-1)[idx] = float(t.view(-1)[idx]) + sign * h
                actual = float(t.view(-1)[idx])
                return (self.tel, t, self.val, actual) if which == "src" else (self.tel, self.src, t, actual)
            tp, sp, vp, ap = moved(+1)
            tm, sm, vm, am = moved(-1)
            out.append(self.diff(tp, sp, vp, tm, sm, vm) / (ap - am))
        return np.array(out)


def check(gpu, fd, which, n, h, rng, k=None):
    idx = np.arange(n) if k is None or k >= n else np.sort(rng.choice(n, k, replace=False))
    ref = fd.grad(which, idx, h)
    got = gpu[which].reshape(-1)[idx]
    err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)
    assert err <= GRAD_TOL, f"{which}: relative error {err:.3g} (|ref| {np.linalg.norm(ref):.3g})"
    return err


@pytest.mark.parametrize("mode", ["image", "response"])
def test_adjoint_hard_square_point_sources(cuda, mode):
    from iactrace_gb300 import SquareSensor
    tel = small_dish(SquareSensor([0, 0, 15.0], [0, 0, 0], 16, 16, (-0.336, 0.336, -0.336, 0.336)))
    src = torch.tensor([[3.0, -2.0, 2000.0], [-20.0, 10.0, 2000.0], [35.0, 25.0, 2000.0]])
    val = torch.tensor([1.0, 0.7, 1.3])
    rng = np.random.default_rng(0)
    P = 256
    g = rng.standard_normal((3, P) if mode == "response" else P)
    gpu = grads_gpu(tel, src, val, "point", g, mode)
    fd = FD(tel, src, val, "point", g.reshape(-1), mode)
    errs = {w: check(gpu, fd, w, n, h, rng, k) for w, n, h, k in
            (("rot", 57, 2e-3, 24), ("pos", 57, 1e-4, 24), ("scale", 19, 2e-6, 8), ("src", 9, 1e-2, None),
             ("val", 3, 1e-3, None))}
    print(mode, errs)


def test_adjoint_hard_hex_parallel_sources(cuda):
    tel = small_dish(W.hex_camera(400, 0.042))
    d = torch.tensor([[0.01, -0.02, -1.0], [-0.03, 0.015, -1.0]])
    d = d / d.norm(dim=1, keepdim=True)
    val = torch.tensor([1.0, 2.0])
    rng = np.random.default_rng(1)
    g = rng.standard_normal(400)
    gpu = grads_gpu(tel, d, val, "parallel", g)
    fd = FD(tel, d, val, "parallel", g)
    for w, n, h, k in (("rot", 57, 2e-3, 20), ("pos", 57, 1e-4, 12), ("src", 6, 1e-5, None), ("val", 2, 1e-3, None)):
        check(gpu, fd, w, n, h, rng, k)


@pytest.mark.parametrize("kind", ["square", "hex"])
def test_adjoint_soft_sensors_position_path(cuda, kind):
    from iactrace_gb300 import DifferentiableHexagonalSensor, DifferentiableSquareSensor
    if kind == "square":
        cam = DifferentiableSquareSensor([0, 0, 15.0], [0, 0, 0], 16, 16, (-0.336, 0.336, -0.336, 0.336), sigma=0.4)
        P = 256
    else:
        cam = DifferentiableHexagonalSensor([0, 0, 15.0], [0, 0, 0], W.hex_grid(400, 0.042), sigma=0.35)
        P = 400
    tel = small_dish(cam, roughness=0.0)
    d = torch.tensor([[0.01, -0.02, -1.0], [-0.03, 0.015, -1.0]])
    d = d / d.norm(dim=1, keepdim=True)
    val = torch.tensor([1.0, 2.0])
    rng = np.random.default_rng(2)
    g = rng.standard_normal(P)
    gpu = grads_gpu(tel, d, val, "parallel", g)
    fd = FD(tel, d, val, "parallel", g, soft=True)
    for w, n, h, k in (("rot", 57, 1e-3, 20), ("pos", 57, 1e-4, 12), ("src", 6, 1e-5, None), ("val", 2, 1e-3, None)):
        check(gpu, fd, w, n, h, rng, k)


def test_backward_of_multistage_scene_is_refused(cuda):
    tel, src, val, st = W.cassegrain(n_samples=8, n_sources=2)
    rot = tel.mirror_groups[0].rotations.clone().requires_grad_(True)
    with pytest.raises(NotImplementedError):
        it.render(tel.set_mirror_rotations(0, rot), src, val, st)
