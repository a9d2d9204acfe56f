"""A torch FP64 restatement of the render chain with autograd: the stand-in
for jax.grad of the reference (JAX is not installable here). Test
infrastructure only.

Discrete decisions (pixel ids, shadow and hit masks, soft-splat base pixels)
are inputs, as they are constants under jax.grad: pass the ones the path
under test took. The chain follows the reference:
  telescope/mirrors.py:64-79, core/render.py:118-171, core/reflection.py:5-20,
  core/intersections.py:6-41 and :229-367 (10 unrolled Newton steps, as the
  reference's lax.scan), core/surfaces.py:25-108, sensors/square.py:144-172,
  sensors/hexagonal.py:174-315.
"""
from __future__ import annotations

import math

import numpy as np
import torch

D = torch.float64
SQRT3_3, SQRT3_2 = 0.5773502691896257, 0.8660254037844386


def euler(a):
    """core/transforms.py:72-107 (a in degrees, (..., 3))."""
    r = a * (math.pi / 180.0)
    cx, cy, cz = torch.cos(r[..., 0]), torch.cos(r[..., 1]), torch.cos(r[..., 2])
    sx, sy, sz = torch.sin(r[..., 0]), torch.sin(r[..., 1]), torch.sin(r[..., 2])
    o, z = torch.ones_like(cx), torch.zeros_like(cx)
    Rx = torch.stack([o, z, z, z, cx, -sx, z, sx, cx], -1).reshape(*cx.shape, 3, 3)
    Ry = torch.stack([cy, z, sy, z, o, z, -sy, z, cy], -1).reshape(*cx.shape, 3, 3)
    Rz = torch.stack([cz, -sz, z, sz, cz, z, z, z, o], -1).reshape(*cx.shape, 3, 3)
    return Rz @ Ry @ Rx


def sag_raw(x, y, c, k, asph):
    r2 = x * x + y * y
    z = r2 * c / (1 + torch.sqrt(1 - (1 + k) * c * c * r2))
    for i in range(asph.shape[0]):
        z = z + asph[i] * r2 ** (2 * (i + 1))
    return z


def mirror_hit(o, d, m):
    """core/surfaces.py:67-108 for one mirror (local frame), Newton unrolled."""
    c, k, asph, off = m["c"], m["k"], m["asph"], m["off"]
    x0, y0 = off[0], off[1]
    z0 = sag_raw(x0, y0, c, k, asph)
    ox, oy, oz = o[..., 0], o[..., 1], o[..., 2]
    dx, dy, dz = d[..., 0], d[..., 1], d[..., 2]
    # conic initial guess (detached: the reference's iteration reaches the same root)
    with torch.no_grad():
        A = c * (dx * dx + dy * dy + (1 + k) * dz * dz)
        oxr, oyr, ozr = ox + x0, oy + y0, oz + z0
        B = 2 * (c * (oxr * dx + oyr * dy + (1 + k) * ozr * dz) - dz)
        C = c * (oxr * oxr + oyr * oyr + (1 + k) * ozr * ozr) - 2 * ozr
        disc = B * B - 4 * A * C
        sq = torch.sqrt(torch.clamp(disc, min=0))
        t1, t2 = (-B - sq) / (2 * A + 1e-30), (-B + sq) / (2 * A + 1e-30)
        t = torch.where((t1 > 1e-8) & (t2 > 1e-8), torch.minimum(t1, t2), torch.where(t1 > 1e-8, t1, t2))
    t = t.detach()

    def g(tt):
        return (oz + tt * dz) - (sag_raw(ox + tt * dx + x0, oy + tt * dy + y0, c, k, asph) - z0)

    for _ in range(10):  # core/intersections.py:332-354, unrolled as the reference's lax.scan
        t = t - g(t) / _gprime(t, ox, oy, oz, dx, dy, dz, x0, y0, c, k, asph)
    xh, yh = ox + t * dx, oy + t * dy
    xs, ys = xh + x0, yh + y0
    zs = sag_raw(xs, ys, c, k, asph) - z0
    r2 = xs * xs + ys * ys
    q = torch.sqrt(1 - (1 + k) * c * c * r2)
    sr = c / (2 * q)
    for i in range(asph.shape[0]):
        p = 2 * (i + 1)
        sr = sr + asph[i] * p * r2 ** (p - 1)
    n = torch.stack([-(sr * 2 * xs), -(sr * 2 * ys), torch.ones_like(xs)], -1)
    n = n / torch.linalg.norm(n, dim=-1, keepdim=True)
    return t, torch.stack([xh, yh, zs], -1), n


def _gprime(t, ox, oy, oz, dx, dy, dz, x0, y0, c, k, asph):
    xs, ys = ox + t * dx + x0, oy + t * dy + y0
    r2 = xs * xs + ys * ys
    q = torch.sqrt(1 - (1 + k) * c * c * r2)
    sr = c / (2 * q)
    for i in range(asph.shape[0]):
        p = 2 * (i + 1)
        sr = sr + asph[i] * p * r2 ** (p - 1)
    return dz - (sr * 2 * xs * dx + sr * 2 * ys * dy)


def philox_normals(seed, F, S, M):
    """N(0,1) pairs of every ray (f, s, m) from Philox4x32-10 (the extended-
    source jitter stream), Box-Muller in float64: arrays (F, S, M)."""
    m = np.arange(M, dtype=np.uint64)[None, None, :]
    f = np.arange(F, dtype=np.uint64)[:, None, None]
    s = np.arange(S, dtype=np.uint64)[None, :, None]
    shape = (F, S, M)
    c0 = np.broadcast_to(m, shape).astype(np.uint64)
    c1 = np.broadcast_to(f, shape).astype(np.uint64)
    c2 = np.broadcast_to(s, shape).astype(np.uint64)
    c3 = np.full(shape, 0x1ACE7, np.uint64)
    k0, k1 = np.uint64(seed & 0xFFFFFFFF), np.uint64(0x5EED)
    M0, M1, W0, W1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57), np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
    mask = np.uint64(0xFFFFFFFF)
    for _ in range(10):
        p0, p1 = M0 * c0, M1 * c2
        n0 = ((p1 >> np.uint64(32)) ^ c1 ^ k0) & mask
        n2 = ((p0 >> np.uint64(32)) ^ c3 ^ k1) & mask
        c1, c3 = p1 & mask, p0 & mask
        c0, c2 = n0, n2
        k0, k1 = (k0 + W0) & mask, (k1 + W1) & mask
    u1 = ((c0 >> np.uint64(8)) + np.uint64(1)).astype(np.float64) / 16777216.0
    u2 = (c1 >> np.uint64(8)).astype(np.float64) / 16777216.0
    rad = np.sqrt(-2.0 * np.log(u1))
    return rad * np.cos(2 * np.pi * u2), rad * np.sin(2 * np.pi * u2)


def jitter_dirs(src, z0, z1):
    """Extended sources (S, 4): unit direction tilted by sigma (z0 t1 + z1 t2)."""
    dh = src[:, :3] / torch.linalg.norm(src[:, :3], dim=-1, keepdim=True)
    ex = torch.tensor([1.0, 0.0, 0.0], dtype=D).expand_as(dh)
    ez = torch.tensor([0.0, 0.0, 1.0], dtype=D).expand_as(dh)
    ref = torch.where((torch.abs(dh[:, 2:3]) > 0.9), ex, ez)
    t1 = torch.linalg.cross(dh, ref)
    t1 = t1 / torch.linalg.norm(t1, dim=-1, keepdim=True)
    t2 = torch.linalg.cross(dh, t1)
    z0, z1 = torch.as_tensor(z0, dtype=D), torch.as_tensor(z1, dtype=D)
    sig = src[:, 3][None, :, None, None]
    d = dh[None, :, None, :] + sig * (z0[..., None] * t1[None, :, None, :] + z1[..., None] * t2[None, :, None, :])
    return d / torch.linalg.norm(d, dim=-1, keepdim=True)


def render(scene, params, decisions, sensor, mode="image"):
    """Image (P,) or response (S, P) as a differentiable function of params.

    scene: dict of fixed float64 tensors: points, normals, delta (F,M,3), weights (F,M),
      sensor plane R (3,3), position (3,), and the sensor constants.
    params: dict of tensors: rot (F,3), pos (F,3), scale (F,), src (S,3), val (S,),
      optional mirrors: list of dicts (rot, pos, c, k, asph, off). The chain
      runs in the parameters' dtype: float64 for the twin proper, float32
      for the same chain at the reference's default precision (what
      jax.grad computes with x64 off).
    decisions: dict of numpy arrays over rays (f, s, m): pix (hard id or -1),
      alive (bool: unshadowed and every stage hit), base (soft: base pixel / hex (q, r)).
    """
    dt = params["val"].dtype  # float64 parameters: the FP64 twin; float32: the same chain in float32
    p, n, dl, w = (scene[k].to(dt) for k in ("points", "normals", "delta", "weights"))
    F, M = w.shape
    S = params["src"].shape[0]
    R = euler(params["rot"])
    tp = torch.einsum("fij,fmj->fmi", R, p) + params["pos"][:, None, :]
    nw = torch.einsum("fij,fmj->fmi", R, n)
    dw = torch.einsum("fij,fmj->fmi", R, dl)
    pe = nw + params["scale"][:, None, None] * dw
    nn = pe / torch.linalg.norm(pe, dim=-1, keepdim=True)
    tp4, nn4 = tp[:, None], nn[:, None]  # (F,1,M,3)
    if scene["source_type"] == "point":
        wv = tp4 - params["src"][None, :, None, :]
        d = wv / torch.linalg.norm(wv, dim=-1, keepdim=True)
    elif scene["source_type"] == "extended":
        z0, z1 = philox_normals(scene.get("seed", 0), F, S, M)
        d = jitter_dirs(params["src"], z0, z1)
    else:
        d = params["src"][None, :, None, :].expand(F, S, M, 3)
    c = (d * nn4).sum(-1)
    r = d - 2 * c[..., None] * nn4
    val = params["val"][None, :, None] * (-c) / w[:, None, :]
    alive = torch.as_tensor(decisions["alive"].reshape(F, S, M))
    val = torch.where(alive, val, torch.zeros_like(val))
    o = tp4.expand(F, S, M, 3)
    if params.get("mirrors") and bool(alive.any()):
        # dead rays (shadowed or missing a mirror) carry no gradient; give them a
        # live ray's geometry so that no NaN reaches the backward pass
        i0 = tuple(int(v) for v in torch.nonzero(alive)[0])
        o = torch.where(alive[..., None], o, o[i0].detach())
        r = torch.where(alive[..., None], r, r[i0].detach())
    for m in params.get("mirrors", []):
        Rm = euler(m["rot"])
        ol = torch.einsum("ji,fsmj->fsmi", Rm, o - m["pos"])
        dlc = torch.einsum("ji,fsmj->fsmi", Rm, r)
        t, pl, nl = mirror_hit(ol, dlc, m)
        pwld = torch.einsum("ij,fsmj->fsmi", Rm, pl) + m["pos"]
        nwld = torch.einsum("ij,fsmj->fsmi", Rm, nl)
        c2 = (r * nwld).sum(-1)
        val = val * torch.abs(c2)
        r = r - 2 * c2[..., None] * nwld
        o = pwld
    Rs, C = scene["sensor_R"].to(dt), scene["sensor_pos"].to(dt)
    u1, u2, ns = Rs[:, 0], Rs[:, 1], Rs[:, 2]
    t = ((ns * C).sum() - (o * ns).sum(-1)) / (r * ns).sum(-1)
    op = o + t[..., None] * r - C
    x, y = (op * u1).sum(-1), (op * u2).sum(-1)
    P = sensor["n_pixels"]
    rows = S if mode == "response" else 1
    out = torch.zeros(rows * P, dtype=dt)
    s_idx = torch.arange(S)[None, :, None].expand(F, S, M).reshape(-1) if mode == "response" else None
    kind = sensor["kind"]
    if kind in ("square", "hex"):
        pix = torch.as_tensor(decisions["pix"].reshape(-1)).long()
        ok = pix >= 0
        idx = pix + (s_idx * P if s_idx is not None else 0)
        out = out.index_add(0, idx[ok], val.reshape(-1)[ok])
    elif kind == "soft_square":
        xp = (x - sensor["x0"]) / sensor["dx"]
        yp = (y - sensor["y0"]) / sensor["dy"]
        xb = torch.floor(xp).detach()
        yb = torch.floor(yp).detach()
        xf, yf = xp - xb, yp - yb
        K = sensor["kernel_size"]
        taps = [(i, j) for i in range(-K, K + 1) for j in range(-K, K + 1)]
        ws = [torch.exp(-0.5 * ((xf - j) ** 2 + (yf - i) ** 2) / sensor["sigma"] ** 2) for i, j in taps]
        W = sum(ws)
        for (i, j), wk in zip(taps, ws):
            xi, yi = (xb + j).long().reshape(-1), (yb + i).long().reshape(-1)
            ok = (xi >= 0) & (xi < sensor["width"]) & (yi >= 0) & (yi < sensor["height"]) & \
                 (x.reshape(-1) < 1e9).detach()
            idx = yi * sensor["width"] + xi + (s_idx * P if s_idx is not None else 0)
            out = out.index_add(0, idx[ok], (val * wk / W).reshape(-1)[ok])
    else:  # soft hex
        gc, gs = sensor["gc"], sensor["gs"]
        xs, ys = x - sensor["off_x"], y - sensor["off_y"]
        xg, yg = gc * xs - gs * ys, gs * xs + gc * ys
        q0 = torch.as_tensor(decisions["base_q"].reshape(F, S, M), dtype=dt)
        r0 = torch.as_tensor(decisions["base_r"].reshape(F, S, M), dtype=dt)
        ddx = xg - sensor["hex_sx"] * (q0 + r0 / 2)
        ddy = yg - sensor["hex_sy"] * r0
        K = sensor["kernel_size"]
        taps = [(q, rr) for q in range(-K, K + 1) for rr in range(-K, K + 1) if max(abs(q), abs(rr), abs(q + rr)) <= K]
        ws = []
        for q, rr in taps:
            ux = ddx - sensor["hex_sx"] * (q + rr / 2)
            uy = ddy - sensor["hex_sy"] * rr
            hd = torch.maximum(torch.abs(ux), 0.5 * torch.abs(ux) + SQRT3_2 * torch.abs(uy)) / sensor["inradius"]
            ws.append(torch.exp(-0.5 * (hd / sensor["sigma"]) ** 2))
        W = sum(ws)
        table = sensor["table"]
        for (q, rr), wk in zip(taps, ws):
            qi = (q0 + q).long().reshape(-1) - sensor["q_min"]
            ri = (r0 + rr).long().reshape(-1) - sensor["r_min"]
            ok = (qi >= 0) & (qi < table.shape[0]) & (ri >= 0) & (ri < table.shape[1])
            pid = torch.full_like(qi, -1)
            pid[ok] = torch.as_tensor(table)[qi[ok], ri[ok]].long()
            ok = ok & (pid >= 0) & (x.reshape(-1) < 1e9).detach()
            idx = pid + (s_idx * P if s_idx is not None else 0)
            out = out.index_add(0, idx[ok], (val * wk / W).reshape(-1)[ok])
    return out.reshape(rows, P) if mode == "response" else out


def scene_of(tel, sensor_idx, source_type):
    """Fixed tensors of a single-group telescope for `render`."""
    g = tel.mirror_groups[0]
    sn = tel.sensors[sensor_idx]
    from iactrace_gb300.core.transforms import euler_to_matrix
    sc = {"points": g.points.double(), "normals": g.normals.double(), "delta": g.perturbation_delta.double(),
          "weights": g.weights.double().reshape(len(g), -1), "source_type": source_type,
          "sensor_R": euler(sn.rotation.double()), "sensor_pos": sn.position.double()}
    del euler_to_matrix
    kind = type(sn).__name__
    if "Square" in kind:
        s = {"kind": "soft_square" if "Differentiable" in kind else "square", "n_pixels": sn.width * sn.height,
             "x0": sn.x0, "y0": sn.y0, "dx": sn.dx, "dy": sn.dy, "width": sn.width, "height": sn.height,
             "sigma": getattr(sn, "sigma", 0.0), "kernel_size": getattr(sn, "kernel_size", 0)}
    else:
        a = np.float32(-sn.grid_rotation)
        s = {"kind": "soft_hex" if "Differentiable" in kind else "hex", "n_pixels": sn.n_pixels,
             "gc": float(np.cos(a)), "gs": float(np.sin(a)), "off_x": sn.grid_offset[0], "off_y": sn.grid_offset[1],
             "hex_sx": sn.hex_size * 1.7320508075688772, "hex_sy": sn.hex_size * 1.5, "inradius": sn.hex_inradius,
             "sigma": getattr(sn, "sigma", 0.0), "kernel_size": getattr(sn, "kernel_size", 0),
             "table": sn.lookup_table.numpy(), "q_min": sn.q_min, "r_min": sn.r_min, "hex_size": sn.hex_size}
    return sc, s


def soft_base(sensor, pts):
    """Base pixel (square) or base hex (q, r) of each ray's plane hit."""
    x, y = pts[:, 0].astype(np.float64), pts[:, 1].astype(np.float64)
    if sensor["kind"] != "soft_hex":
        return {}
    xs, ys = x - sensor["off_x"], y - sensor["off_y"]
    xg, yg = sensor["gc"] * xs - sensor["gs"] * ys, sensor["gs"] * xs + sensor["gc"] * ys
    q = (SQRT3_3 * xg - yg / 3) / sensor["hex_size"]
    r = (2 * yg / 3) / sensor["hex_size"]
    s = -q - r
    qi, ri, si = np.round(q), np.round(r), np.round(s)
    dq, dr, ds = np.abs(qi - q), np.abs(ri - r), np.abs(si - s)
    qi = np.where((dq > dr) & (dq > ds), -ri - si, qi)
    ri = np.where((dr > dq) & (dr > ds), -qi - si, ri)
    big = ~(x < 1e9)
    return {"base_q": np.where(big, 0, qi), "base_r": np.where(big, 0, ri)}


def soft_hex_kink_pixels(sensor, pts, band=1e-6, wmin=1e-6):
    """Pixel ids fed by rays whose soft-hex weights sit within `band` metres
    of a kink of the hexagonal norm (|ux| = 0, |uy| = 0 or the two branches
    of the max equal) on a tap of relative weight > wmin. The weights are not
    differentiable there: float32 and float64 evaluations of the same ray
    take opposite one-sided derivatives, so a gradient comparison must not
    weight those pixels."""
    if sensor["kind"] != "soft_hex":
        return np.zeros(0, dtype=np.int64)
    x, y = pts[:, 0].astype(np.float64), pts[:, 1].astype(np.float64)
    ok = x < 1e9
    base = soft_base(sensor, pts)
    xs, ys = x - sensor["off_x"], y - sensor["off_y"]
    xg, yg = sensor["gc"] * xs - sensor["gs"] * ys, sensor["gs"] * xs + sensor["gc"] * ys
    ddx = xg - sensor["hex_sx"] * (base["base_q"] + base["base_r"] / 2)
    ddy = yg - sensor["hex_sy"] * base["base_r"]
    K = sensor["kernel_size"]
    taps = [(q, rr) for q in range(-K, K + 1) for rr in range(-K, K + 1) if max(abs(q), abs(rr), abs(q + rr)) <= K]
    table = np.asarray(sensor["table"])
    near = np.zeros(x.shape, dtype=bool)
    ws = []
    for q, rr in taps:
        ux = ddx - sensor["hex_sx"] * (q + rr / 2)
        uy = ddy - sensor["hex_sy"] * rr
        ax, ay = np.abs(ux), np.abs(uy)
        hd = np.maximum(ax, 0.5 * ax + SQRT3_2 * ay) / sensor["inradius"]
        w = np.exp(-0.5 * (hd / sensor["sigma"]) ** 2)
        ws.append(w)
        kink = np.minimum(np.minimum(ax, ay), np.abs(ax - (0.5 * ax + SQRT3_2 * ay)))
        near |= ok & (kink < band) & (w > wmin * 1.0)
    bad = []
    for i in np.nonzero(near)[0]:
        for q, rr in taps:
            qi, ri = int(base["base_q"][i] + q) - sensor["q_min"], int(base["base_r"][i] + rr) - sensor["r_min"]
            if 0 <= qi < table.shape[0] and 0 <= ri < table.shape[1] and table[qi, ri] >= 0:
                bad.append(int(table[qi, ri]))
    return np.unique(np.array(bad, dtype=np.int64))


def resample_mapping(group, surf, pts, nrm, dlt, w, n_samples):
    """The sampled arrays as functions of the surface parameters, FP64 torch
    autograd (core/surfaces.py:41-65, core/reflection.py:22-49,
    core/integrators.py:124-127): the aperture positions and the roughness
    coefficients of drawn samples do not depend on the surface; points,
    normals, deltas and weights do. Reference for the device sampler's
    reverse (iact_sample_facets_backward)."""
    from iactrace_gb300.core.reflection import perturbation_delta_from_normals
    dev = pts.device
    xy = pts[..., :2].double()
    n0 = nrm.double()
    ref_z = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64, device=dev)
    ref_x = torch.tensor([1.0, 0.0, 0.0], dtype=torch.float64, device=dev)
    ref = torch.where(n0[..., 2:3].abs() > 0.9, ref_x, ref_z)
    t1 = torch.linalg.cross(n0, ref.expand_as(n0))
    t1 = t1 / torch.linalg.norm(t1, dim=-1, keepdim=True)
    t2 = torch.linalg.cross(n0, t1)
    d0 = dlt.double()
    th1, th2 = (d0 * t1).sum(-1), (d0 * t2).sum(-1)
    s64 = type(surf)(surf.curvature if not isinstance(surf.curvature, torch.Tensor) else surf.curvature.double(),
                     surf.conic if not isinstance(surf.conic, torch.Tensor) else surf.conic.double(),
                     surf.aspheric.double())
    off = group.offsets.reshape(-1, 1, 2).to(device=dev, dtype=torch.float64)
    p, n = s64.point_and_normal(xy, off)
    dl = perturbation_delta_from_normals(n, th1, th2)
    area = (n0[..., 2] / w[..., 0].double() * n_samples).detach()
    ww = n[..., 2:3] / area[..., None] * n_samples
    return p, n, dl, ww
