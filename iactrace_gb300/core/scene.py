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
    """core/render.py:12-18 _get_stages (cached per telescope and group list)."""
    key = tuple(map(id, tel.mirror_groups))
    hit = tel.__dict__.get("_stages")
    if hit is not None and hit[0] == key:
        return hit[1]
    by = defaultdict(list)
    for g in tel.mirror_groups:
        by[g.optical_stage].append(g)
    out = dict(sorted(by.items()))
    tel.__dict__["_stages"] = (key, out)
    return out


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


def _join(ts):
    """torch.cat, without the copy for a single tensor."""
    return ts[0] if len(ts) == 1 else torch.cat(ts)


def _tkey(x):
    """Cache key of a tensor by its storage (address, version, shape, stride,
    dtype): unique while the cache keeps a detached alias of it alive (the
    alias holds the storage and shares the version counter, but not the
    autograd graph); numbers by value."""
    if isinstance(x, torch.Tensor):
        return (x.data_ptr(), x._version, tuple(x.shape), tuple(x.stride()), x.dtype, str(x.device))
    return None if x is None else float(x)


def _alias(x):
    return x.detach() if isinstance(x, torch.Tensor) else x


def _require_finite(items) -> None:
    """Input validation at pack time (once per packed scene): the kernels do
    not check their tables, so NaN / Inf never reach them. items: (what,
    tensor) pairs; one device-to-host read for all of them. Skipped while
    the stream is being captured into a CUDA graph (a read is not allowed
    there): validate inputs before capturing."""
    items = [(w, t) for w, t in items if t.numel()]
    if not items or (torch.cuda.is_available() and torch.cuda.is_current_stream_capturing()):
        return
    ok = torch.stack([torch.isfinite(t).all() for _, t in items]).cpu()
    for (what, _), good in zip(items, ok.tolist()):
        if not good:
            raise ValueError(f"{what} contains NaN or Inf")


# Stage-mirror records and obstruction tables on the device, shared by every
# packed scene with the same stage >= 1 groups and obstruction groups (a
# per-step resampled primary does not rebuild or re-upload them; no host to
# device copy then happens inside a captured step). Entries keep their
# source objects alive so the ids in the key stay unique.
_STATIC = OrderedDict()
_STATIC_MAX = 16


def _static_key(tel, later, device):
    sv = _tkey
    fp = [str(torch.device(device))]
    for stage, groups in later:
        for g in groups:
            fp.append((stage, len(g), sv(g.curvature), sv(g.conic)))
            fp += [sv(getattr(g, n)) for n in ("positions", "rotations", "offsets", "aspheric", "radii", "vertices")
                   if getattr(g, n, None) is not None]
    fp += [id(g) for g in (tel.obstruction_groups or [])]
    return tuple(fp)


def _static_tables(tel, later, device):
    key = _static_key(tel, later, device)
    hit = _STATIC.get(key)
    if hit is not None:
        _STATIC.move_to_end(key)
        return hit[1], hit[2]
    recs = _mirror_records(later)
    if len(recs) and not np.isfinite(recs.view(np.float32)).all():
        # the records are float32 fields and int32 counts; counts are finite as floats too
        raise ValueError("stage-mirror parameters contain NaN or Inf")
    mirrors = torch.from_numpy(recs.copy()).to(device) if len(recs) else None
    kinds = defaultdict(list)
    for g in (tel.obstruction_groups or []):
        kinds[g.kind].append(g.table().float())
    _require_finite([(f"{kind} obstruction table", t) for kind, ts in kinds.items() for t in ts])
    obst = {kind: _f32(torch.cat(kinds[kind]), device) for kind in ("cyl", "box", "sph", "obox", "tri")
            if kinds[kind]}
    keep = [tuple(_alias(getattr(g, n, None)) for n in ("curvature", "conic", "positions", "rotations", "offsets",
                                                        "aspheric", "radii", "vertices"))
            for _, gs in later for g in gs] + list(tel.obstruction_groups or [])
    _STATIC[key] = (keep, mirrors, obst)
    while len(_STATIC) > _STATIC_MAX:
        _STATIC.popitem(last=False)
    return mirrors, obst


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
            cat = lambda name: _f32(_join([getattr(g, name).detach() for g in prim]), device)
            self.points = cat("points")
            self.normals = cat("normals")
            self.delta = cat("perturbation_delta")
            self.weights = cat("weights").reshape(self.F, self.M)
            _require_finite([(f"primary {name}", getattr(self, name))
                             for name in ("points", "normals", "delta", "weights")])
            for name in ("points", "normals", "delta", "weights"):
                setattr(d, name, getattr(self, name).data_ptr())
        later = [(s, gs) for s, gs in st.items() if s != 0]
        self.mirrors, self.obst = _static_tables(tel, later, device)
        self.n_mirrors = int(self.mirrors.numel()) // ctypes.sizeof(N.IactMirror) if self.mirrors is not None else 0
        d.n_mirrors = self.n_mirrors
        d.n_stages = len(later)
        self.n_stages = len(later)
        d.mirrors = self.mirrors.data_ptr() if self.n_mirrors else None
        for kind, t in self.obst.items():
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
        key = (ctypes.addressof(sensor_desc), bytes(sensor_desc), int(n_sources), int(mode))
        cache = self.__dict__.setdefault("_ws_bytes", {})
        if key in cache:
            return cache[key]
        size = ctypes.c_size_t(0)
        N.check(N.load().iact_workspace_size(ctypes.byref(self.desc), ctypes.byref(sensor_desc), int(n_sources),
                                             int(mode), ctypes.byref(size)))
        cache[key] = int(size.value)
        return int(size.value)


def primary_params(tel, device):
    """Concatenated stage-0 facet rotations (F,3), positions (F,3), scales (F,):
    float32 on `device`, differentiable (torch.cat / .to keep the graph)."""
    prim = stages_of(tel).get(0, [])
    if not prim:
        z = torch.zeros((0, 3), device=device)
        return z, z, torch.zeros(0, device=device)
    # a new autograd node even for one group (a view, which launches nothing):
    # autograd then accumulates a leaf's gradient behind an op of the calling
    # stream (a leaf handed to the render directly would tie its creation
    # stream into a captured backward)
    def cat(name, w):
        ts = [getattr(g, name).reshape(len(g), w) if w else getattr(g, name).reshape(-1) for g in prim]
        t = torch.cat(ts) if len(ts) > 1 else ts[0].view(ts[0].shape)
        return t.to(device=device, dtype=torch.float32)
    return cat("rotations", 3), cat("positions", 3), cat("perturbation_scale", 0)


def _value(x) -> float:
    return float(x.detach()) if isinstance(x, torch.Tensor) else float(x)


def _fingerprint(tel):
    """Identity of everything packed once (not the per-facet transforms)."""
    fp = []
    for g in tel.mirror_groups:
        names = ("points", "normals", "perturbation_delta", "weights") if g.optical_stage == 0 else \
            ("positions", "rotations", "offsets", "aspheric", "radii", "vertices")
        for name in names:
            t = getattr(g, name, None)
            if t is not None:
                fp.append(_tkey(t))
        # surface constants: values, or tensor identities (no device read)
        fp.append((g.optical_stage, _tkey(g.curvature), _tkey(g.conic), len(g)))
    for g in (tel.obstruction_groups or []):
        fp.append(id(g))
    return tuple(fp)


# Packed scenes shared by telescopes built from the same sample arrays, stage
# mirrors and obstructions (an optimiser's functional updates of the facet
# transforms create a new Telescope per step). The entries keep detached
# aliases of their source tensors: the storages stay alive, so the addresses
# in the fingerprint cannot be reused while cached, and no autograd graph is
# kept (a cached graph would pin its gradient accumulators to the streams
# they were first built on).
_SHARED = OrderedDict()
_SHARED_MAX = 16


def _sources(tel):
    out = []
    for g in tel.mirror_groups:
        names = ("points", "normals", "perturbation_delta", "weights") if g.optical_stage == 0 else \
            ("positions", "rotations", "offsets", "aspheric", "radii", "vertices")
        out += [_alias(getattr(g, n, None)) for n in names] + [_alias(g.curvature), _alias(g.conic)]
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
        fkey = tuple(_tkey(t) for t in src)
        cached = ps.__dict__.get("_facet_cache")
        if cached is not None and cached[0] == fkey:
            facets = cached[2]
        else:
            facets = tuple(t.detach().contiguous() for t in primary_params(tel, ps.device))
            ps._facet_cache = (fkey, [_alias(t) for t in src], facets)
    ps.set_facets(*facets)
    return ps
