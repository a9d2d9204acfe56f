#!/usr/bin/env python
"""Gradient fixtures of the render path from the reference itself.

Runs GerritRo/iactrace's own Python source (a checkout named by the
IACTRACE_REFERENCE environment variable) in float64 on the numpy stand-in
for jax/equinox (tests/golden/jaxshim) and takes central finite
differences of its `render` (core/render.py:174-220) with respect to the
parameters jax.grad differentiates: primary facet rotations, positions and
roughness scales, the later-stage mirror's pose, curvature, conic and
aspheric coefficient, source positions / directions and values. The
sensors are the soft-splat ones (sensors/square.py:144-172,
sensors/hexagonal.py:264-315), whose images are smooth in those parameters.

Per case and soft sensor the fixture stores the Jacobian of the whole
image, J[parameter, pixel] = d image[pixel] / d parameter, so a test can
weight pixels freely (L = sum g * image gives dL/dparameter = J @ g).

Each column is Richardson-extrapolated from central differences at steps h
and h/2; the two must agree to 1e-6 relative (or to the rounding noise of
the difference quotient, for a column that is zero), otherwise a ray crossed a
discontinuity (a shadow edge, an aperture edge, a soft-hexagon base-cell
change) inside the step, and the column is taken again with an eight times
smaller step (at most three times).

The scene is rounded to float32 values before differencing (the CUDA path
reads float32 tables), so both evaluate the same function at the same
point.

  dc_soft_grad    19-facet Davies-Cotton dish (the dc_mixed scene of
                  make_golden.py: cylinders, box, sphere, oriented box,
                  triangle), roughness 24", 3 point sources at 1 km,
                  soft square (sigma 0.4 px, 5x5 taps) and soft hexagonal
                  (sigma 0.5 inradius, 7 taps) cameras
  cass_soft_grad  the two-mirror Cassegrain of make_golden.py (aspheric
                  primary and secondary) with a 1.45 m secondary,
                  roughness 10", 4 parallel sources within 0.5 deg, soft
                  square camera (sigma 0.5 px)

Every ray of these scenes reaches the sensor plane. A ray that does not
gets the plane's sentinel hit (1e10, 1e10; core/intersections.py:6-41),
and the reference's soft sensors turn it into NaN: the float-to-int32 cast
of its pixel coordinate overflows, all tap weights underflow to zero, the
normalisation divides 0 by 0, and the NaN survives the `* valid` mask
(sensors/square.py:156-168). The CUDA path drops such rays instead.

Usage: IACTRACE_REFERENCE=<checkout> python tests/golden/make_grad_golden.py [case ...] [-j N]
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
import time

os.environ["JAXSHIM_X64"] = "1"
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import make_golden as MG  # noqa: E402  (imports the reference on the stand-in, x64)

eqx, jnp = MG.eqx, MG.jnp

# central-difference steps per parameter kind (units of the parameter)
STEPS = {"rot": 2e-6, "pos": 2e-7, "scale": 2e-8, "src_point": 2e-4, "src_parallel": 2e-7, "val": 1e-3,
         "mrot": 2e-6, "mpos": 2e-7, "mc": 2e-9, "mk": 2e-5, "masph": 2e-9}


def _f32(x):
    return jnp.array(np.asarray(x, dtype=np.float64).astype(np.float32).astype(np.float64))


def _round_scene(tel, src, val):
    """Every float the render reads, as the float32 value it has on the device."""
    groups = []
    for g in tel.mirror_groups:
        names = ["positions", "rotations", "points", "normals", "perturbation_delta", "weights",
                 "perturbation_scale"]
        if g.optical_stage != 0:
            names += ["offsets", "aspheric"] + (["radii"] if hasattr(g, "radii") else ["vertices"])
        g = eqx.tree_at(lambda q: tuple(getattr(q, n) for n in names), g, tuple(_f32(getattr(g, n)) for n in names))
        if g.optical_stage != 0:
            g = eqx.tree_at(lambda q: (q.curvature, q.conic), g,
                            (float(np.float32(g.curvature)), float(np.float32(g.conic))))
        groups.append(g)
    return eqx.tree_at(lambda t: t.mirror_groups, tel, groups), _f32(src), _f32(val)


def scene_dc_soft():
    tel, src, val, st, _ = MG.scene_dc_mixed()
    tel = eqx.tree_at(lambda t: t.sensors, tel, [tel.sensors[2], tel.sensors[3]]).apply_roughness(24.0)
    tel, src, val = _round_scene(tel, src, val)
    return tel, src, val, st


def scene_cass_soft():
    # a wider secondary and sources closer to the axis than cass_parallel, so
    # that every ray reaches the sensor plane (see _check_finite)
    tel, src, val, st, _ = MG.scene_cassegrain(sec_radius=1.45, theta_deg=(0.0, 0.2, 0.35, 0.5))
    cam = MG.DifferentiableSquareSensor(position=[0.0, 0.0, -0.5], rotation=[0.0, 0.0, 0.0], width=24, height=24,
                                        bounds=(-0.3, 0.3, -0.3, 0.3), sigma=0.5, kernel_size=2)
    tel = eqx.tree_at(lambda t: t.sensors, tel, [cam]).apply_roughness(10.0)
    tel, src, val = _round_scene(tel, src, val)
    return tel, src, val, st


CASES = {"dc_soft_grad": scene_dc_soft, "cass_soft_grad": scene_cass_soft}


def parameters(tel, src, st):
    """(block, index, step) for every differentiated parameter."""
    out = []
    prim = [g for g in tel.mirror_groups if g.optical_stage == 0]
    assert len(prim) == 1
    F = len(prim[0])
    for blk in ("rot", "pos"):
        out += [(blk, (f, j), STEPS[blk]) for f in range(F) for j in range(3)]
    out += [("scale", (f,), STEPS["scale"]) for f in range(F)]
    S = np.asarray(src).shape[0]
    skind = "src_point" if st == "point" else "src_parallel"
    out += [("src", (s, j), STEPS[skind]) for s in range(S) for j in range(3)]
    out += [("val", (s,), STEPS["val"]) for s in range(S)]
    later = [g for g in tel.mirror_groups if g.optical_stage != 0]
    for i, g in enumerate(later):
        assert len(g) == 1
        out += [(f"mrot{i}", (0, j), STEPS["mrot"]) for j in range(3)]
        out += [(f"mpos{i}", (0, j), STEPS["mpos"]) for j in range(3)]
        out += [(f"mc{i}", (), STEPS["mc"]), (f"mk{i}", (), STEPS["mk"])]
        out += [(f"masph{i}", (k,), STEPS["masph"]) for k in range(np.asarray(g.aspheric).shape[0])]
    return out


def _bump(arr, idx, d):
    a = np.array(np.asarray(arr), dtype=np.float64, copy=True)
    a[idx] += d
    return jnp.array(a)


def perturbed(tel, src, val, block, idx, d):
    if block == "src":
        return tel, _bump(src, idx, d), val
    if block == "val":
        return tel, src, _bump(val, idx, d)
    groups = list(tel.mirror_groups)
    if block in ("rot", "pos", "scale"):
        gi = [i for i, g in enumerate(groups) if g.optical_stage == 0][0]
        name = {"rot": "rotations", "pos": "positions", "scale": "perturbation_scale"}[block]
    else:
        gi = [i for i, g in enumerate(groups) if g.optical_stage != 0][int(block[-1])]
        name = {"mrot": "rotations", "mpos": "positions", "mc": "curvature", "mk": "conic",
                "masph": "aspheric"}[block[:-1]]
    g = groups[gi]
    cur = getattr(g, name)
    new = float(cur) + d if name in ("curvature", "conic") else _bump(cur, idx, d)
    groups[gi] = eqx.tree_at(lambda q: getattr(q, name), g, new)
    return eqx.tree_at(lambda t: t.mirror_groups, tel, groups), src, val


def images(tel, src, val, st):
    return np.concatenate([np.asarray(MG.render(tel, src, val, st, si), dtype=np.float64).reshape(-1)
                           for si in range(len(tel.sensors))])


_SCENE = {}


def column(args):
    """Richardson-extrapolated central difference of all images for one parameter."""
    case, block, idx, h = args
    if case not in _SCENE:
        tel, src, val, st = CASES[case]()
        _SCENE[case] = tel, src, val, st, np.linalg.norm(images(tel, src, val, st))
    tel, src, val, st, base_norm = _SCENE[case]

    def cd(step):
        up = images(*perturbed(tel, src, val, block, idx, step), st)
        dn = images(*perturbed(tel, src, val, block, idx, -step), st)
        return (up - dn) / (2 * step)

    for attempt in range(4):
        j1, j2 = cd(h), cd(h / 2)
        # rounding noise of a difference quotient is ~ eps |image| / h: a
        # parameter the image does not depend on (the roll of a rotationally
        # symmetric mirror) has a column of that size only
        noise = 1e3 * np.finfo(np.float64).eps * base_norm / h
        if np.linalg.norm(j1 - j2) <= 1e-6 * np.linalg.norm(j2) + noise:
            return block, idx, h, attempt, (4 * j2 - j1) / 3
        h /= 8
    return block, idx, h, -1, (4 * j2 - j1) / 3


def _check_finite(name, tel, src, val, st, base):
    pts, _ = MG.render_debug(tel, src, val, st, 0)
    if not (np.isfinite(base).all() and (np.abs(np.asarray(pts)) < 1e9).all()):
        sys.exit(f"{name}: some rays miss the sensor plane; the reference's soft sensors give NaN for them")


def run_case(name, jobs):
    t0 = time.time()
    tel, src, val, st = CASES[name]()
    rec = MG.scene_arrays(tel)
    rec["sources"], rec["values"], rec["source_type"] = np.asarray(src), np.asarray(val), np.array(st)
    base = images(tel, src, val, st)
    _check_finite(name, tel, src, val, st, base)
    sizes = [int(np.prod(s.get_accumulator_shape())) for s in tel.sensors]
    params = parameters(tel, src, st)
    with mp.get_context("spawn").Pool(jobs) as pool:
        cols = pool.map(column, [(name, b, i, h) for (b, i, h) in params], chunksize=1)
    bad = [(b, i) for b, i, _, att, _ in cols if att < 0]
    if bad:
        sys.exit(f"{name}: no consistent finite difference for {bad}")
    blocks = {}
    for b, i, h, att, col in cols:
        blocks.setdefault(b, []).append((i, h, col))
    off = np.cumsum([0] + sizes)
    for si in range(len(sizes)):
        rec[f"image_{si}_shape"] = np.array(tel.sensors[si].get_accumulator_shape())
        rec[f"image_{si}"] = base[off[si]:off[si + 1]]
    for b, items in blocks.items():
        J = np.stack([c for _, _, c in items])  # [n_params_in_block, sum of pixels]
        for si in range(len(sizes)):
            rec[f"jac_{b}_{si}"] = J[:, off[si]:off[si + 1]]
        rec[f"jac_{b}_index"] = np.array([list(i) for i, _, _ in items], dtype=np.int32).reshape(len(items), -1)
        rec[f"jac_{b}_step"] = np.array([h for _, h, _ in items])
    rec["jac_blocks"] = np.array(json.dumps(sorted(blocks)))
    retried = sum(1 for *_, att, _ in cols if att > 0)
    out = os.path.join(HERE, f"{name}_f64.npz")
    np.savez_compressed(out, **rec)
    print(f"{name}: {len(params)} parameters ({retried} with a smaller step), {time.time() - t0:.0f} s -> "
          f"{os.path.basename(out)} ({os.path.getsize(out) / 1024:.0f} KiB)", flush=True)


def main():
    args = sys.argv[1:]
    jobs = os.cpu_count() or 1
    if "-j" in args:
        k = args.index("-j")
        jobs = int(args[k + 1])
        del args[k:k + 2]
    for n in [a for a in args if not a.startswith("-")] or list(CASES):
        run_case(n, jobs)


if __name__ == "__main__":
    main()
