"""The torch FP64 autograd twin (tests/twin.py, the stand-in for jax.grad)
against central finite differences of the FP64 oracle, with the oracle's
discrete decisions held fixed. CPU only."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from iactrace_gb300 import Telescope, workloads as W

import twin


def _oracle(built):
    import oracle.oracle as O
    return O


def _tel(camera):
    groups, _ = W.davies_cotton(n_facets=7, n_samples=16, seed=5)
    from iactrace_gb300.core import Box, Cylinder, group_obstructions
    obst = group_obstructions([Cylinder([1.0, 0.3, 0.2], [0.3, 0.1, 15.4], 0.05),
                               Box([-0.2, -0.2, 15.0], [0.2, 0.2, 16.0])])
    return Telescope(groups, obst, [camera]).apply_roughness(24.0)


def _fd(O, tel, src, val, st, g, dec0, which, idx, h, soft):
    grp = tel.mirror_groups[0]

    def loss(sign):
        if which in ("rot", "pos"):
            t = (grp.rotations if which == "rot" else grp.positions).clone()
            t.view(-1)[idx] += sign * h
            tl = tel.set_mirror_rotations(0, t) if which == "rot" else tel.set_mirror_positions(0, t)
            s = src
            moved = float(t.view(-1)[idx])
        else:
            s = src.clone()
            s.view(-1)[idx] += sign * h
            tl = tel
            moved = float(s.view(-1)[idx])
        if soft:
            return float((O.render(tel=tl, sources=s, values=val, source_type=st).reshape(-1) * g).sum()), moved
        d = O.render_debug(tl, s, val, st, 0, "f64")
        ok = (d["vals"] != 0) == dec0["alive"]
        pix = dec0["pix"]
        gv = np.where(pix >= 0, g[np.maximum(pix, 0)], 0.0)
        return float((d["vals"] * gv * ok).sum()), moved

    lp, ap = loss(+1)
    lm, am = loss(-1)
    return (lp - lm) / (ap - am)


@pytest.mark.parametrize("kind", ["square", "soft_hex"])
def test_twin_matches_oracle_finite_differences(built, kind):
    O = _oracle(built)
    from iactrace_gb300 import DifferentiableHexagonalSensor, SquareSensor
    if kind == "square":
        cam = SquareSensor([0, 0, 15.0], [0, 0, 0], 12, 12, (-0.252, 0.252, -0.252, 0.252))
        src, st, P = torch.tensor([[3.0, -2.0, 2000.0], [-20.0, 10.0, 2000.0]]), "point", 144
    else:
        cam = DifferentiableHexagonalSensor([0, 0, 15.0], [0, 0, 0], W.hex_grid(200, 0.042), sigma=0.35)
        d = torch.tensor([[0.01, -0.02, -1.0], [-0.03, 0.015, -1.0]])
        src, st, P = d / d.norm(dim=1, keepdim=True), "parallel", 200
    tel = _tel(cam)
    val = torch.tensor([1.0, 0.7])
    g = np.random.default_rng(0).standard_normal(P)
    dd = O.render_debug(tel, src, val, st, 0, "f64")
    sc, sn = twin.scene_of(tel, 0, st)
    dec = {"pix": dd["pix"], "alive": dd["vals"] != 0}
    dec.update(twin.soft_base(sn, dd["pts"]))
    grp = tel.mirror_groups[0]
    params = {"rot": grp.rotations, "pos": grp.positions, "scale": grp.perturbation_scale, "src": src, "val": val}
    params = {k: v.detach().double().clone().requires_grad_(True) for k, v in params.items()}
    out = twin.render(sc, params, dec, sn)
    (out * torch.as_tensor(g)).sum().backward()
    rng = np.random.default_rng(1)
    # soft hex weights have kinks (|.| and max in the hex norm): small steps keep
    # the central difference on one side of them for almost every ray
    soft = kind != "square"
    steps = (("rot", 21, 2e-5 if soft else 1e-3), ("pos", 21, 2e-6 if soft else 1e-4),
             ("src", 6, 1e-6 if soft else 1e-2))
    for which, n, h in steps:
        for idx in rng.choice(n, 4, replace=False):
            fd = _fd(O, tel, src, val, st, g, dec, which, int(idx), h, kind != "square")
            ad = float(params[which].grad.reshape(-1)[idx])
            scale = float(params[which].grad.abs().max())
            assert abs(fd - ad) <= 2e-4 * scale + 1e-12, f"{which}[{idx}]: twin {ad:.6g} vs FD {fd:.6g}"
