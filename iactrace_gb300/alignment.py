"""Mirror-alignment inverse problem on a large parabolic dish.

A 28 m parabolic dish of 876 hexagonal facets (0.90 m flat-to-flat,
f = 36 m, spherical facets of radius 2f aimed at the focus) images 256
extended sources (Gaussian angular profile, sigma = 0.05 deg) within 2 deg of
the axis onto a 2048-pixel hexagonal camera with soft (Gaussian-splat)
deposition. The target image is rendered with every facet tipped and tilted
by N(0, 1 mrad); the tips and tilts (2 x 876 parameters) are recovered from
the nominal orientation by Adam on the L2 image loss, with gradients from the
adjoint kernel (recompute-based, behind torch.autograd).

Only facet tips and tilts are free; sources, samples and the camera are the
same in the target and the fit. The image loss is the objective: with the
camera at the focus the individual tilts are only weakly identifiable from
one summed image (every facet's spot of a source falls on the same place,
and two facets whose spots trade places give almost the same image), so the
RMS tilt error is reported beside the loss but is not expected to fall with
it. With the camera below the focus (`camera_z`) the facets' spots land
apart and each moves with its own facet's tilt: there the same run recovers
the tilts (19 facets, camera 12 m below the focus: RMS error 0.85 -> 0.000
mrad in 200 steps).
"""
from __future__ import annotations

import math
import os
import time

import numpy as np
import torch

from . import _native as N
from .core.apertures import PolygonAperture
from .core.integrators import MCIntegrator
from .core.render import render
from .core.surfaces import AsphericSurface
from .sensors import DifferentiableHexagonalSensor, DifferentiableSquareSensor
from .telescope.mirrors import Mirror, group_mirrors
from .telescope.telescope import Telescope
from .utils import keys as _keys
from .workloads import hex_grid, hex_vertices


def parabolic_dish(n_facets: int = 876, focal: float = 36.0, facet_flat: float = 0.90, n_samples: int = 128,
                   seed: int = 0):
    """Facets on z = r^2 / (4f), each aimed so that its centre reflects an
    on-axis ray into the focus (normal along the bisector of +z and the
    direction to the focus)."""
    surf = AsphericSurface(curvature=1.0 / (2.0 * focal), conic=0.0, aspheric=[])
    verts = hex_vertices(facet_flat)
    mirrors = []
    for (x, y) in hex_grid(n_facets, facet_flat + 0.02):
        z = (x * x + y * y) / (4.0 * focal)
        to_f = np.array([-x, -y, focal - z])
        to_f /= np.linalg.norm(to_f)
        nvec = to_f + np.array([0.0, 0.0, 1.0])
        nvec /= np.linalg.norm(nvec)
        rot = [-math.degrees(math.asin(nvec[1])), math.degrees(math.atan2(nvec[0], nvec[2])), 0.0]
        mirrors.append(Mirror([x, y, z], rot, surf, PolygonAperture(verts), optical_stage=0))
    groups = group_mirrors(mirrors)
    integ = MCIntegrator(n_samples)
    return [integ.sample_group(g, k) for g, k in zip(groups, _keys.split(_keys.key(seed), len(groups)))]


def extended_sources(n: int = 256, max_deg: float = 2.0, sigma_deg: float = 0.05, seed: int = 1):
    """(n, 4): unit directions (towards the dish) within max_deg of the axis and sigma in radians."""
    g = torch.Generator().manual_seed(seed)
    th = math.radians(max_deg) * torch.sqrt(torch.rand(n, generator=g, dtype=torch.float64))
    ph = 2 * math.pi * torch.rand(n, generator=g, dtype=torch.float64)
    d = torch.stack([torch.sin(th) * torch.cos(ph), torch.sin(th) * torch.sin(ph), -torch.cos(th)], 1)
    return torch.cat([d, torch.full((n, 1), math.radians(sigma_deg), dtype=torch.float64)], 1).float()


def problem(n_facets: int = 876, n_samples: int = 128, n_sources: int = 256, n_pixels: int = 2048,
            sigma_true_mrad: float = 1.0, seed: int = 0, device="cuda", camera_z: float = 36.0,
            square_camera: tuple | None = None, max_deg: float = 2.0):
    """Nominal telescope, target image rendered with the perturbed tilts, and the truth.

    camera_z: height of the camera plane (36 m: the focus, where every
    facet's spot of a source falls on the same place). Below the focus the
    spots of different facets land apart (each facet's light has not yet
    converged), and each facet's tilt moves its own spot: the tilts become
    identifiable from the image. square_camera = (pixels per side, width in
    m): a soft square camera instead of the soft hexagonal one."""
    groups = parabolic_dish(n_facets=n_facets, n_samples=n_samples, seed=seed)
    if square_camera is None:
        cam = DifferentiableHexagonalSensor([0.0, 0.0, camera_z], [0.0, 0.0, 0.0],
                                            hex_grid(n_pixels, 0.042).astype(np.float32), sigma=0.5, kernel_size=1)
    else:
        n, w = square_camera
        cam = DifferentiableSquareSensor([0.0, 0.0, camera_z], [0.0, 0.0, 0.0], n, n, (-w / 2, w / 2, -w / 2, w / 2),
                                         sigma=0.5, kernel_size=2)
    tel = Telescope(groups, [], [cam], name="dish28m_alignment")
    src = extended_sources(n_sources, max_deg=max_deg, seed=seed + 1).to(device)
    val = torch.ones(n_sources, device=device)
    rng = torch.Generator().manual_seed(seed + 2)
    nominal = groups[0].rotations.clone()
    err = torch.zeros_like(nominal)
    err[:, :2] = torch.randn((nominal.shape[0], 2), generator=rng) * math.degrees(sigma_true_mrad * 1e-3)
    true_rot = nominal + err
    with torch.no_grad():
        target = render(tel.set_mirror_rotations(0, true_rot.to(device)), src, val, "extended", seed=seed)
    return {"telescope": tel, "sources": src, "values": val, "target": target, "nominal": nominal.to(device),
            "truth": true_rot.to(device), "seed": seed}


def rms_tilt_error_mrad(rot, truth) -> float:
    d = (rot[:, :2] - truth[:, :2]).detach()
    return float(torch.sqrt((d * d).mean()) * math.pi / 180.0 * 1e3)


def run(prob, steps: int = 200, lr: float = 2e-3, log_every: int = 0, checkpoint: str | None = None,
        checkpoint_every: int = 50, graph: bool = False):
    """Adam on the facet tips and tilts (degrees). Returns the history.

    checkpoint: a file; if it exists the run resumes from it (tilt offsets,
    Adam moments, step count, history) and continues up to `steps` in
    total; the state is saved there every `checkpoint_every` steps and at
    the end. graph: after three eager steps, the whole Adam step (render,
    loss, adjoint, optimiser) is captured in a CUDA graph and replayed.
    hist["launches_per_step"]: the library's kernels in one step (counted
    around an eager step, or around the capture of the replayed step)."""
    tel, src, val, target = prob["telescope"], prob["sources"], prob["values"], prob["target"]
    base = prob["nominal"]
    # the facet positions and roughness scales stay fixed: keep them on the
    # device (no per-step host copies, and nothing to copy inside a graph)
    g0 = tel.mirror_groups[0]
    g0 = g0.replace(positions=g0.positions.to(base.device), perturbation_scale=g0.perturbation_scale.to(base.device))
    tel = Telescope([g0] + list(tel.mirror_groups[1:]), tel.obstruction_groups, tel.sensors, name=tel.name)
    delta = torch.zeros((base.shape[0], 2), device=base.device, requires_grad=True)
    opt = torch.optim.Adam([delta], lr=lr, capturable=graph)
    pad = torch.zeros((base.shape[0], 1), device=base.device)
    hist = {"loss": [], "rms_mrad": [], "step_ms": []}
    start = 0
    if checkpoint is not None and os.path.exists(checkpoint):
        st = torch.load(checkpoint, map_location=base.device, weights_only=False)
        with torch.no_grad():
            delta.copy_(st["delta"])
        opt.load_state_dict(st["adam"])
        hist = st["history"]
        start = int(st["step"])

    def save(step):
        if checkpoint is not None:
            tmp = checkpoint + ".tmp"
            torch.save({"delta": delta.detach().clone(), "adam": opt.state_dict(), "history": hist, "step": step},
                       tmp)
            os.replace(tmp, checkpoint)

    scale = float(target.pow(2).sum())
    lib = N.load()

    def body():
        rot = base + torch.cat([delta, pad], 1)
        img = render(tel.set_mirror_rotations(0, rot), src, val, "extended", seed=prob["seed"])
        loss = (img - target).pow(2).sum() / scale
        loss.backward()
        opt.step()
        return loss, rot

    def record(it, t0, loss, rot):
        torch.cuda.synchronize()
        hist["step_ms"].append((time.perf_counter() - t0) * 1e3)
        hist["loss"].append(float(loss.detach()))
        hist["rms_mrad"].append(rms_tilt_error_mrad(rot, prob["truth"]))
        if log_every and (it % log_every == 0 or it == steps - 1):
            print(f"step {it:4d} loss {hist['loss'][-1]:.4e} rms tilt error {hist['rms_mrad'][-1]:.3f} mrad")
        if checkpoint is not None and (it + 1) % checkpoint_every == 0:
            save(it + 1)

    it = start
    n_eager = steps if not graph else min(steps, start + 3)
    side = torch.cuda.Stream(base.device) if graph else None
    if graph:  # eager steps on a side stream warm up the allocator, autograd and Adam state
        side.wait_stream(torch.cuda.current_stream(base.device))
    with torch.cuda.stream(side) if graph else _nullctx():
        while it < n_eager:
            t0 = time.perf_counter()
            n0 = lib.iact_kernel_launches()
            opt.zero_grad(set_to_none=True)
            loss, rot = body()
            hist["launches_per_step"] = lib.iact_kernel_launches() - n0
            record(it, t0, loss, rot)
            it += 1
    if graph and it < steps:
        torch.cuda.current_stream(base.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        opt.zero_grad(set_to_none=True)
        n0 = lib.iact_kernel_launches()
        with torch.cuda.graph(g):
            s_loss, s_rot = body()
        hist["launches_per_step"] = lib.iact_kernel_launches() - n0
        while it < steps:
            t0 = time.perf_counter()
            g.replay()
            record(it, t0, s_loss, s_rot)
            it += 1
    save(max(start, steps))
    return hist


class _nullctx:
    def __enter__(self):
        return None

    def __exit__(self, *a):
        return False
