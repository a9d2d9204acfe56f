"""Gradient helpers shared by the adjoint tests.

gpu_grads:   dL/dparameter of L = sum(g * out) from the CUDA adjoint
             (iact_render_backward behind torch.autograd), per parameter block.
twin_grads:  the same from the torch FP64 autograd twin (tests/twin.py), on
             given discrete decisions (pixel ids, shadow / hit masks,
             soft-splat base cells: constants under jax.grad).
fixture_grads: the same from a reference-held Jacobian (tests/golden/
             *_grad_f64.npz, central differences of the reference's own
             float64 render).
compare:     per-block relative L2 errors, asserted below a tolerance.

Block names: rot, pos, scale (stage-0 facets), src, val, and per later-stage
mirror i: mrot<i>, mpos<i>, mc<i> (curvature), mk<i> (conic), masph<i>.
"""
from __future__ import annotations

import json

import numpy as np
import torch

import twin


def stage_groups(tel):
    return [g for g in tel.mirror_groups if g.optical_stage != 0]


def gpu_grads(tel, src, val, st, g, mode="image", sensor_idx=0):
    """GPU gradients of L = sum(g * out) w.r.t. every parameter block."""
    import iactrace_gb300 as it
    from iactrace_gb300 import Telescope
    grp = tel.mirror_groups[0]
    leaves = {"rot": grp.rotations.clone().cuda().requires_grad_(True),
              "pos": grp.positions.clone().cuda().requires_grad_(True),
              "scale": grp.perturbation_scale.clone().cuda().requires_grad_(True),
              "src": src.clone().cuda().requires_grad_(True), "val": val.clone().cuda().requires_grad_(True)}
    groups = [grp.replace(rotations=leaves["rot"], positions=leaves["pos"], perturbation_scale=leaves["scale"])]
    for i, sg in enumerate(stage_groups(tel)):
        lv = {"mrot": sg.rotations.clone().cuda().requires_grad_(True),
              "mpos": sg.positions.clone().cuda().requires_grad_(True),
              "mc": torch.tensor(float(sg.curvature), device="cuda", requires_grad=True),
              "mk": torch.tensor(float(sg.conic), device="cuda", requires_grad=True),
              "masph": sg.aspheric.clone().cuda().requires_grad_(True)}
        leaves.update({f"{k}{i}": v for k, v in lv.items()})
        groups.append(sg.replace(rotations=lv["mrot"], positions=lv["mpos"], curvature=lv["mc"], conic=lv["mk"],
                                 aspheric=lv["masph"]))
    t2 = Telescope(groups, tel.obstruction_groups, tel.sensors)
    fn = it.render_response_matrix if mode == "response" else it.render
    out = fn(t2, leaves["src"], leaves["val"], st, sensor_idx)
    (out.double() * torch.as_tensor(g, device="cuda").reshape(out.shape)).sum().backward()
    return {k: (v.grad.double().cpu().numpy() if v.grad is not None else np.zeros(v.shape)) for k, v in leaves.items()}


def gpu_debug(tel, src, val, st, sensor_idx=0):
    """The GPU's per-ray decisions: plane hits, values, hard pixel ids."""
    import iactrace_gb300 as it
    pts, vals, pix, _ = it.render_debug(tel, src, val, st, sensor_idx, extras=True)
    return {"pts": pts.cpu().numpy(), "vals": vals.cpu().numpy(), "pix": pix.cpu().numpy()}


def twin_grads(tel, src, val, st, g, debug, mode="image", sensor_idx=0, dtype=torch.float64):
    """Twin (FP64 autograd) gradients on the decisions of `debug` (a dict
    with the per-ray pts, vals and hard pixel ids pix, in ray order
    (facet, source, sample)). dtype=torch.float32 runs the same chain and
    its autograd in float32 (the reference's default precision)."""
    sc, sn = twin.scene_of(tel, sensor_idx, st)
    dec = {"pix": np.asarray(debug["pix"]), "alive": np.asarray(debug["vals"]) != 0}
    dec.update(twin.soft_base(sn, np.asarray(debug["pts"])))
    grp = tel.mirror_groups[0]
    params = {"rot": grp.rotations, "pos": grp.positions, "scale": grp.perturbation_scale, "src": src, "val": val}
    params = {k: v.detach().to(dtype).clone().requires_grad_(True) for k, v in params.items()}
    leaves = dict(params)
    mirrors = []
    for i, sg in enumerate(stage_groups(tel)):
        m = {"rot": sg.rotations.to(dtype)[0].clone().requires_grad_(True),
             "pos": sg.positions.to(dtype)[0].clone().requires_grad_(True),
             "c": torch.tensor(float(sg.curvature), dtype=dtype, requires_grad=True),
             "k": torch.tensor(float(sg.conic), dtype=dtype, requires_grad=True),
             "asph": sg.aspheric.to(dtype).clone().requires_grad_(True),
             "off": sg.offsets.to(dtype)[0]}
        mirrors.append(m)
        leaves.update({f"mrot{i}": m["rot"], f"mpos{i}": m["pos"], f"mc{i}": m["c"], f"mk{i}": m["k"],
                       f"masph{i}": m["asph"]})
    params["mirrors"] = mirrors
    out = twin.render(sc, params, dec, sn, mode)
    (out.reshape(-1) * torch.as_tensor(g, dtype=dtype).reshape(-1)).sum().backward()
    return {k: v.grad.double().numpy() if v.grad is not None else np.zeros(v.shape) for k, v in leaves.items()}


def fixture_grads(fx, sensor_idx, g, shapes):
    """dL/dparameter = J @ g per block from a reference-held Jacobian
    fixture, shaped like `shapes[block]`."""
    out = {}
    for b in json.loads(str(fx["jac_blocks"])):
        J = fx[f"jac_{b}_{sensor_idx}"]
        out[b] = (J @ np.asarray(g, dtype=np.float64).reshape(-1)).reshape(shapes[b])
    return out


def kink_pixels(tel, st, pts, sensor_idx=0):
    """Soft-hexagon pixels fed by rays on a kink of the hexagonal norm."""
    _, sn = twin.scene_of(tel, sensor_idx, st)
    return twin.soft_hex_kink_pixels(sn, np.asarray(pts))


def compare(got, ref, tol, skip=()):
    errs = {}
    for k in ref:
        if k in skip:
            continue
        a, b = np.asarray(got[k]).reshape(-1), np.asarray(ref[k]).reshape(-1)
        nb = np.linalg.norm(b)
        if nb == 0:
            assert np.linalg.norm(a) == 0, k
            continue
        errs[k] = float(np.linalg.norm(a - b) / nb)
    bad = {k: e for k, e in errs.items() if e > tol}
    assert not bad, f"relative errors above {tol}: {bad} (all: {errs})"
    return errs
