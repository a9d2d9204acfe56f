"""Packing of a Telescope into the device tables of the C ABI.

Stage-0 groups are concatenated in list order (core/render.py:202-205);
stage >= 1 mirrors are flattened in (stage, group, mirror) order, so the
kernels' "first strict minimum" equals the reference's argmin over mirrors
and strict ``<`` over groups (core/render.py:62-71, :110). Obstruction groups
are concatenated per kind: the shadow mask only asks whether any member of
any group is hit (core/render.py:38-40).
"""
from __future__ import annotations

import ctypes
from collections import OrderedDict, defaultdict

import numpy as np
import torch

from .. import _native as N


def stages_of(tel):
    """core/render.py:12-18 _get_stages."""
    by = defaultdict(list)
    for g in tel.mirror_groups:
        by[g.optical_stage].append(g)
    return dict(sorted(by.items()))


def _f32(t, device):
    return t.detach().to(device=device, dtype=torch.float32).contiguous()


def _mirror_records(stage_groups) -> np.ndarray:
    recs = []
    for stage, groups in stage_groups:
        for g in groups:
            asph = g.aspheric.detach().cpu().float().tolist()
            if len(asph) > N.IACT_MAX_ASPH:
                raise ValueError(f"at most {N.IACT_MAX_ASPH} aspheric coefficients are supported")
            polygon = hasattr(g, "vertices")
            for i in range(len(g)):
                m = N.IactMirror()
                m.stage = int(stage)
                m.aperture = N.APERTURE_POLYGON if polygon else N.APERTURE_DISK
                m.n_asph = len(asph)
                m.pos[:] = g.positions[i].detach().cpu().tolist()
                m.rot[:] = g.rotations[i].detach().cpu().tolist()
                m.offset[:] = g.offsets[i].detach().cpu().tolist()
                m.curvature, m.conic = _value(g.curvature), _value(g.conic)
                for k, a in enumerate(asph):
                    m.asph[k] = a
                if polygon:
                    v = g.vertices[i].detach().cpu().tolist()
                    if len(v) > N.IACT_MAX_POLY:
                        raise ValueError(f"at most {N.IACT_MAX_POLY} polygon vertices are supported")
                    m.n_vert = len(v)
                    for k, (x, y) in enumerate(v):
                        m.vert[k][0], m.vert[k][1] = x, y
                else:
                    m.radius = float(g.radii[i])
                recs.append(bytes(m))
    if len(recs) > N.IACT_MAX_STAGE_MIRRORS:
        raise ValueError(f"at most {N.IACT_MAX_STAGE_MIRRORS} mirrors over all stages >= 1 are supported")
    return np.frombuffer(b"".join(recs), dtype=np.uint8) if recs else np.zeros(0, np.uint8)


def _require_finite(what: str, t: torch.Tensor) -> None:
    """Host-side input validation at pack time (once per scene): the kernels
    do not check their tables, so NaN / Inf never reach them."""
    if t.numel() and not bool(torch.isfinite(t).all()):
        raise ValueError(f"{what} contains NaN or Inf")


class PackedScene:
    """Device-resident tables + the iact_scene_t that points at them.

    The sample arrays, stage-mirror records and obstruction tables are packed
    once and cached; the per-facet transforms (rotation, position, roughness
    scale: F x 7 floats, the parameters an optimiser changes) are refreshed by
    `set_facets` on every call."""

    def __init__(self, tel, device):
        device = torch.device(device)
        st = stages_of(tel)
        prim = st.get(0, [])
        self.has_primary = len(prim) > 0
        self.F = sum(len(g) for g in prim)
        ms = {g.n_samples for g in prim}
        if len(ms) > 1:
            raise ValueError(f"all primary groups must have the same sample count, got {sorted(ms)}")
        self.M = ms.pop() if ms else 0
        d = N.IactScene()
        d.n_facets, d.n_samples = self.F, self.M
        if self.F and self.M:
            cat = lambda name: torch.cat([getattr(g, name).detach().float() for g in prim])
            for name in ("points", "normals", "perturbation_delta", "weights"):
                _require_finite(f"primary {name}", cat(name))
            self.points = _f32(cat("points"), device)
            self.normals = _f32(cat("normals"), device)
            self.delta = _f32(cat("perturbation_delta"), device)
            self.weights = _f32(cat("weights").reshape(self.F, self.M), device)
            for name in ("points", "normals", "delta", "weights"):
                setattr(d, name, getattr(self, name).data_ptr())
        later = [(s, gs) for s, gs in st.items() if s != 0]
        recs = _mirror_records(later)
        if len(recs) and not np.isfinite(recs.view(np.float32)).all():
            # the records are float32 fields and int32 counts; counts are finite as floats too
            raise ValueError("stage-mirror parameters contain NaN or Inf")
        self.n_mirrors = len(recs) // ctypes.sizeof(N.IactMirror)
        self.mirrors = torch.from_numpy(recs.copy()).to(device) if self.n_mirrors else None
        d.n_mirrors = self.n_mirrors
        d.n_stages = len(later)
        self.n_stages = len(later)
        d.mirrors = self.mirrors.data_ptr() if self.n_mirrors else None
        kinds = defaultdict(list)
        for g in (tel.obstruction_groups or []):
            t = g.table().float()
            _require_finite(f"{g.kind} obstruction table", t)
            kinds[g.kind].append(t)
        self.obst = {}
        for kind in ("cyl", "box", "sph", "obox", "tri"):
            if kinds[kind]:
                t = _f32(torch.cat(kinds[kind]), device)
                self.obst[kind] = t
                setattr(d, "n_" + kind, int(t.shape[0]))
                setattr(d, kind, t.data_ptr())
        self.desc = d
        self.device = device

    def set_facets(self, rot, pos, scale):
        """Point the descriptor at these (F,3), (F,3), (F,) float32 device tensors."""
        self.facet_rot, self.facet_pos, self.facet_scale = rot, pos, scale
        if self.F and self.M:
            self.desc.facet_rot, self.desc.facet_pos = rot.data_ptr(), pos.data_ptr()
            self.desc.facet_scale = scale.data_ptr()

    def workspace_bytes(self, sensor_desc, n_sources: int, mode: int) -> int:
        size = ctypes.c_size_t(0)
        N.check(N.load().iact_workspace_size(ctypes.byref(self.desc), ctypes.byref(sensor_desc), int(n_sources),
                                             int(mode), ctypes.byref(size)))
        return int(size.value)


def primary_params(tel, device):
    """Concatenated stage-0 facet rotations (F,3), positions (F,3), scales (F,):
    float32 on `device`, differentiable (torch.cat / .to keep the graph)."""
    prim = stages_of(tel).get(0, [])
    if not prim:
        z = torch.zeros((0, 3), device=device)
        return z, z, torch.zeros(0, device=device)
    cat = lambda name, w: torch.cat([getattr(g, name).reshape(len(g), w) if w else getattr(g, name).reshape(-1)
                                     for g in prim]).to(device=device, dtype=torch.float32)
    return cat("rotations", 3), cat("positions", 3), cat("perturbation_scale", 0)


def _value(x) -> float:
    return float(x.detach()) if isinstance(x, torch.Tensor) else float(x)


def _fingerprint(tel):
    """Identity of everything packed once (not the per-facet transforms)."""
    fp = []
    for g in tel.mirror_groups:
        names = ("points", "normals", "perturbation_delta", "weights") if g.optical_stage == 0 else \
            ("positions", "rotations", "offsets", "aspheric")
        for name in names:
            t = getattr(g, name, None)
            if t is not None:
                fp.append((id(t), t._version))
        fp.append((g.optical_stage, _value(g.curvature), _value(g.conic), len(g)))
    for g in (tel.obstruction_groups or []):
        fp.append(id(g))
    return tuple(fp)


# Packed scenes shared by telescopes built from the same sample arrays, stage
# mirrors and obstructions (an optimiser's functional updates of the facet
# transforms create a new Telescope per step). The entries keep their source
# tensors alive, so the ids in the fingerprint cannot be reused while cached.
_SHARED = OrderedDict()
_SHARED_MAX = 16


def _sources(tel):
    out = []
    for g in tel.mirror_groups:
        names = ("points", "normals", "perturbation_delta", "weights") if g.optical_stage == 0 else \
            ("positions", "rotations", "offsets", "aspheric")
        out += [getattr(g, n, None) for n in names]
    return out + list(tel.obstruction_groups or [])


def pack_scene(tel, device, facets=None) -> PackedScene:
    """Packed tables of `tel` on `device` (cached while the sample arrays,
    stage mirrors and obstructions are unchanged), with the current facet
    transforms (or the given detached `facets` = (rot, pos, scale))."""
    cache = tel.__dict__.setdefault("_packed", {})
    key = str(torch.device(device))
    fp = _fingerprint(tel)
    hit = cache.get(key)
    if hit is not None and hit[0] == fp:
        ps = hit[1]
    else:
        shared = _SHARED.get((key, fp))
        if shared is not None:
            _SHARED.move_to_end((key, fp))
            ps = shared[1]
        else:
            ps = PackedScene(tel, device)
            _SHARED[(key, fp)] = (_sources(tel), ps)
            while len(_SHARED) > _SHARED_MAX:
                _SHARED.popitem(last=False)
        cache[key] = (fp, ps)
    if facets is None:
        # device copies of the facet transforms, reused while the source
        # tensors are the same objects at the same version (kept alive here so
        # their ids stay unique)
        src = [t for g in stages_of(tel).get(0, []) for t in (g.rotations, g.positions, g.perturbation_scale)]
        fkey = tuple((id(t), getattr(t, "_version", 0)) for t in src)
        cached = ps.__dict__.get("_facet_cache")
        if cached is not None and cached[0] == fkey:
            facets = cached[2]
        else:
            facets = tuple(t.detach().contiguous() for t in primary_params(tel, ps.device))
            ps._facet_cache = (fkey, src, facets)
    ps.set_facets(*facets)
    return ps
