"""Render entry points (core/render.py of the reference) over the C ABI.

``render``, ``render_response_matrix`` and ``render_debug`` keep the
reference's signatures and results; the work is one call into the CUDA
library (include/iactrace_gb300.h). There is no CPU path: without a CUDA
device or without the built library these functions raise.
"""
from __future__ import annotations

import ctypes
import math
import operator

import torch

from .. import _native as N
from .scene import _join, pack_scene, primary_params, stages_of


_HAVE_CUDA = False


def _device():
    global _HAVE_CUDA
    if not _HAVE_CUDA:
        if not torch.cuda.is_available():
            raise RuntimeError("iactrace_gb300 renders on a CUDA device; none is available")
        _HAVE_CUDA = True
    return torch.device("cuda", torch.cuda.current_device())


def source_code(source_type) -> int:
    """core/render.py:129-133: 'point' is a point source, anything else parallel.

    'extended' (not a reference type) is a parallel source with a Gaussian
    angular profile: sources are (S, 4) = (direction, sigma in radians) and
    every ray draws its own tilt from a counter-based stream (``seed``)."""
    if source_type == "point":
        return N.SRC_POINT
    if source_type == "extended":
        return N.SRC_EXTENDED
    return N.SRC_PARALLEL


def _ready(t, device, shape_ok):
    """t as it is when it is already a contiguous float32 tensor on `device`."""
    return isinstance(t, torch.Tensor) and t.dtype == torch.float32 and t.device == device and \
        t.is_contiguous() and shape_ok(t)


def _inputs(sources, values, device, source_type="point"):
    width = 4 if source_type == "extended" else 3
    device = torch.device(device)
    if _ready(sources, device, lambda t: t.dim() == 2 and t.shape[1] == width):
        src = sources
    else:
        src = torch.as_tensor(sources).to(device=device, dtype=torch.float32).reshape(-1, width).contiguous()
    if _ready(values, device, lambda t: t.dim() == 1):
        val = values
    else:
        val = torch.as_tensor(values).to(device=device, dtype=torch.float32).reshape(-1).contiguous()
    if src.shape[0] != val.shape[0]:
        raise ValueError(f"sources ({src.shape[0]}) and values ({val.shape[0]}) disagree in length")
    return src, val


def _workspace(ps, sdesc, S, mode, device):
    """Per-call scratch from torch's stream-ordered caching allocator."""
    return torch.empty(max(ps.workspace_bytes(sdesc, S, mode), 256), dtype=torch.uint8, device=device)


def _forward(ps, desc, sdesc, code, src, val, mode, shape, opts, device):
    out = torch.empty(shape, dtype=torch.float32, device=device)
    ws = _workspace(ps, sdesc, src.shape[0], mode, device)
    stream = torch.cuda.current_stream(device).cuda_stream
    N.check(N.load().iact_render(ctypes.byref(desc), ctypes.byref(sdesc), code, src.data_ptr(), val.data_ptr(),
                                 int(src.shape[0]), mode, out.data_ptr(), ws.data_ptr(), ws.numel(),
                                 ctypes.byref(opts) if opts is not None else None, stream))
    return out


def _desc_with(ps, rot, pos, scale):
    """The packed scene's descriptor with the facet transforms of these tensors."""
    d = N.IactScene()
    ctypes.memmove(ctypes.addressof(d), ctypes.addressof(ps.desc), ctypes.sizeof(d))
    d.facet_rot, d.facet_pos, d.facet_scale = rot.data_ptr(), pos.data_ptr(), scale.data_ptr()
    return d


def _sample_grads(gs, rot, scale, nrm, dlt, wts):
    """Local-frame gradients of the primary sample arrays from the adjoint's
    per-sample world sums gs [F, M, 7] = (dL/dp_world, dL/dn'_world,
    dL/d(1/w)): p_world = R p + pos; n' = R m / |m|, m = n + s delta
    (telescope/mirrors.py:64-79); value = v (-c) / w."""
    from .transforms import euler_to_matrix
    g = gs.double()
    R = euler_to_matrix(rot.double())  # (F, 3, 3)
    a, b, giw = g[..., 0:3], g[..., 3:6], g[..., 6]
    # R^T a, R^T b as broadcast products (no batched GEMM: nothing to set up
    # per stream inside a captured backward)
    Rt = R[:, None, :, :]  # (F, 1, 3(j), 3(i))
    gp = (Rt * a[..., :, None]).sum(-2)
    bl = (Rt * b[..., :, None]).sum(-2)
    m = nrm.double() + scale.double()[:, None, None] * dlt.double()
    mn = torch.linalg.norm(m, dim=-1, keepdim=True)
    u = m / mn
    gm = (bl - (bl * u).sum(-1, keepdim=True) * u) / mn
    w = wts.double()
    return gp, gm, scale.double()[:, None, None] * gm, -giw / (w * w)


class RenderFunction(torch.autograd.Function):
    """iact_render forward, iact_render_backward (recompute-based adjoint) backward.

    Differentiable inputs: concatenated stage-0 facet rotations (F,3, degrees),
    positions (F,3), perturbation scales (F,), sources (S,3), values (S,),
    per stage mirror rotations (n,3), positions (n,3) and surface parameters
    (n, 10: curvature, conic, 8 aspheric coefficients), and the primary sample
    arrays (points, normals, deltas (F,M,3), weights (F,M)) when they carry
    gradients (resampled with differentiable surface parameters).
    """

    @staticmethod
    def forward(ctx, meta, rot, pos, scale, src, val, mrot, mpos, msurf, spts, snrm, sdlt, swts):
        ps, sensor, code, mode, shape, opts = meta
        device = src.device
        sdesc, keep = sensor.pack(device)
        rot_, pos_, scale_ = (t.detach().contiguous() for t in (rot, pos, scale))
        src_, val_ = src.detach().contiguous(), val.detach().contiguous()
        out = _forward(ps, _desc_with(ps, rot_, pos_, scale_), sdesc, code, src_, val_, mode, shape, opts, device)
        ctx.meta = meta
        ctx.n_mir = mrot.shape[0]
        ctx.save_for_backward(rot_, pos_, scale_, src_, val_, snrm.detach(), sdlt.detach(), swts.detach())
        del keep
        return out

    @staticmethod
    def backward(ctx, gout):
        ps, sensor, code, mode, shape, opts = ctx.meta
        rot, pos, scale, src, val, snrm, sdlt, swts = ctx.saved_tensors
        device = src.device
        sdesc, keep = sensor.pack(device)
        need = ctx.needs_input_grad
        need_s = any(need[9:13])
        gsamp = torch.empty((ps.F, ps.M, 7), device=device) if need_s and ps.F * ps.M else None
        g = [torch.empty_like(t) if need[i + 1] else None for i, t in enumerate((rot, pos, scale, src, val))]
        nm = ctx.n_mir
        gm = [torch.empty(sh, device=device) if need[6 + i] and nm else None
              for i, sh in enumerate(((nm, 3), (nm, 3), (nm, 10)))]
        ws = torch.empty(max(ps.workspace_bytes(sdesc, src.shape[0], N.MODE_BACKWARD), 256), dtype=torch.uint8,
                         device=device)
        gout = gout.detach().to(torch.float32).contiguous()
        stream = torch.cuda.current_stream(device).cuda_stream
        ptr = lambda t: t.data_ptr() if t is not None else None
        if code == N.SRC_EXTENDED and g[3] is not None:
            raise NotImplementedError("no gradients with respect to extended sources")
        N.check(N.load().iact_render_backward(
            ctypes.byref(_desc_with(ps, rot, pos, scale)), ctypes.byref(sdesc), code, src.data_ptr(),
            val.data_ptr(), int(src.shape[0]), mode, gout.data_ptr(), ptr(g[0]), ptr(g[1]), ptr(g[2]),
            ptr(g[3]), ptr(g[4]), ptr(gm[0]), ptr(gm[1]), ptr(gm[2]), ptr(gsamp), ws.data_ptr(), ws.numel(),
            ctypes.byref(opts) if opts is not None else None, stream))
        del keep
        gm = [x if x is not None or not need[6 + i] else torch.zeros((0,) + ((3,) if i < 2 else (10,)),
                                                                      device=device)
              for i, x in enumerate(gm)]
        gs = [None] * 4
        if gsamp is not None:
            gs = [x.to(t.dtype) if need[9 + i] else None
                  for i, (x, t) in enumerate(zip(_sample_grads(gsamp, rot, scale, snrm, sdlt, swts),
                                                 (snrm, snrm, sdlt, swts)))]
        return (None, *g, *gm, *gs)


_EMPTY = {}


def _empty(shape, device):
    """A cached zero-size float32 tensor (placeholders for absent inputs)."""
    key = (tuple(shape), str(device))
    t = _EMPTY.get(key)
    if t is None:
        t = _EMPTY[key] = torch.zeros(shape, device=device)
    return t


def _as_t(x, device):
    # python numbers become device fills (no host-to-device copy)
    return x.to(device=device, dtype=torch.float32) if isinstance(x, torch.Tensor) else \
        torch.full((), float(x), device=device)


def _stage_params(tel, device):
    """Per stage mirror (packing order): rotations, positions, (c, k, a[8])."""
    rots, poss, surfs = [], [], []
    for stage, groups in stages_of(tel).items():
        if stage == 0:
            continue
        for g in groups:
            n = len(g)
            rots.append(g.rotations.reshape(n, 3).to(device=device, dtype=torch.float32))
            poss.append(g.positions.reshape(n, 3).to(device=device, dtype=torch.float32))
            a = g.aspheric.reshape(-1).to(device=device, dtype=torch.float32)
            a = torch.cat([a, torch.zeros(N.IACT_MAX_ASPH - a.shape[0], device=device)])
            surf = torch.cat([_as_t(g.curvature, device).reshape(1), _as_t(g.conic, device).reshape(1), a])
            surfs.append(surf[None, :].expand(n, 2 + N.IACT_MAX_ASPH))
    if not rots:
        z = _empty((0, 3), device)
        return z, z, _empty((0, 2 + N.IACT_MAX_ASPH), device)
    return torch.cat(rots), torch.cat(poss), torch.cat(surfs)


def primary_samples(tel, device):
    """Concatenated stage-0 sample arrays: points, normals, deltas (F,M,3)
    and weights (F,M), float32 on `device`, differentiable."""
    prim = stages_of(tel).get(0, [])
    cat = lambda name: _join([getattr(g, name) for g in prim]).to(device=device, dtype=torch.float32)
    pts, nrm, dlt, w = cat("points"), cat("normals"), cat("perturbation_delta"), cat("weights")
    return pts, nrm, dlt, w.reshape(w.shape[0], w.shape[1])


def _needs_grad(tel, src, val):
    if not torch.is_grad_enabled():
        return False
    if src.requires_grad or val.requires_grad:
        return True
    for stage, groups in stages_of(tel).items():
        for g in groups:
            ts = [g.rotations, g.positions, g.perturbation_scale, g.aspheric, g.curvature, g.conic]
            if stage == 0:
                ts += [g.points, g.normals, g.perturbation_delta, g.weights]
            if any(isinstance(t, torch.Tensor) and t.requires_grad for t in ts):
                return True
    return False


def _opts_with_seed(opts, seed):
    if not seed:
        return opts
    o = N.IactOpts()
    if opts is not None:
        ctypes.memmove(ctypes.addressof(o), ctypes.addressof(opts), ctypes.sizeof(o))
    o.seed = int(seed) & 0xFFFFFFFF
    return o


def _state_key(tel, sensor):
    """Identity of everything a forward launch packs: the telescope, its
    mirror groups and every field of them (tensors by object and version
    counter), the obstruction groups, the sensor and its fields. None when
    some group tensor requires grad (the autograd path). Objects are held by
    the telescope and the sensor, so their ids stay unique while cached."""
    key = [id(tel), id(sensor)]
    for g in tel.mirror_groups:
        key.append(id(g))
        for v in g.__dict__.values():
            if isinstance(v, torch.Tensor):
                if v.requires_grad:
                    return None
                key.append(id(v))
                key.append(v._version)
            else:
                key.append(id(v))
    key.append(-1)
    key.extend(map(id, tel.obstruction_groups or ()))
    key.append(-2)
    for v in sensor.__dict__.values():
        key.append(id(v))
        if isinstance(v, torch.Tensor):
            key.append(v._version)
    return tuple(key)


def _object_ids(tel, sensor):
    """Identities of the objects _state_key covers (C-level map/tuple work):
    the telescope, the sensor, the mirror groups and their field values, the
    obstruction groups and the sensor's field values."""
    gs = tel.mirror_groups
    return (id(tel), id(sensor), tuple(map(id, gs)), tuple(tuple(map(id, g.__dict__.values())) for g in gs),
            tuple(map(id, tel.obstruction_groups or ())), tuple(map(id, sensor.__dict__.values())))


_VERSION = operator.attrgetter("_version")
_REQUIRES_GRAD = operator.attrgetter("requires_grad")


def _tensor_fields(tel, sensor):
    """The tensors among the mirror groups' and the sensor's fields."""
    return tuple(v for g in tel.mirror_groups for v in g.__dict__.values() if isinstance(v, torch.Tensor)) + \
        tuple(v for v in sensor.__dict__.values() if isinstance(v, torch.Tensor))


def _fast_forward(tel, sensor, sensor_idx, src, val, code, mode, shape, opts, device):
    """Repeated forward calls on an unchanged telescope: the packed scene,
    the facet transforms, the sensor descriptor and the workspace size come
    from a per-telescope cache, not from re-hashing the tensor storages; the
    launch is then two allocations and one call. A cache entry is valid
    while the objects _state_key covers are the same (their identities) and
    its tensors are unchanged (version counters) and need no gradient, which
    is _state_key's condition checked without rebuilding its key. Returns
    None when the cache does not apply."""
    cache = tel.__dict__.setdefault("_fast", {})
    ck = (device.index, sensor_idx, mode, int(src.shape[0]))
    hit = cache.get(ck)
    if hit is not None and hit[0] == _object_ids(tel, sensor):
        tens = hit[1]
        if any(map(_REQUIRES_GRAD, tens)):
            return None
        if tuple(map(_VERSION, tens)) != hit[2]:
            hit = None
    else:
        hit = None
    if hit is None:
        if _state_key(tel, sensor) is None:
            return None
        ps = pack_scene(tel, device)
        sdesc, keep = sensor.pack(device)
        ws_bytes = max(ps.workspace_bytes(sdesc, int(src.shape[0]), mode), 256)
        # after packing: the packing caches stored on the sensor are part of its fields
        tens = _tensor_fields(tel, sensor)
        hit = (_object_ids(tel, sensor), tens, tuple(map(_VERSION, tens)), ps,
               (ps.facet_rot, ps.facet_pos, ps.facet_scale), sdesc, keep, ws_bytes)
        cache[ck] = hit
    ps, facets, sdesc, keep, ws_bytes = hit[3:]
    ps.set_facets(*facets)  # a packed scene may be shared by telescopes with other facet transforms
    out = torch.empty(shape, dtype=torch.float32, device=device)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    N.check(N.load().iact_render(ctypes.byref(ps.desc), ctypes.byref(sdesc), code, src.data_ptr(), val.data_ptr(),
                                 int(src.shape[0]), mode, out.data_ptr(), ws.data_ptr(), ws_bytes,
                                 ctypes.byref(opts) if opts is not None else None, stream))
    return out


def _launch(tel, sources, values, source_type, sensor_idx, mode, opts=None, seed=0):
    device = _device()
    sensor = tel.sensors[sensor_idx]
    src, val = _inputs(sources, values, device, source_type)
    opts = _opts_with_seed(opts, seed)
    S = int(src.shape[0])
    P = int(math.prod(sensor.get_accumulator_shape()))
    shape = (S, P) if mode == N.MODE_RESPONSE else tuple(sensor.get_accumulator_shape())
    if 0 not in stages_of(tel):  # core/render.py:197-199 empty telescope
        return torch.zeros(shape, device=device)
    code = source_code(source_type)
    if not (torch.is_grad_enabled() and (src.requires_grad or val.requires_grad)):
        out = _fast_forward(tel, sensor, sensor_idx, src, val, code, mode, shape, opts, device)
        if out is not None:
            return out
    if _needs_grad(tel, src, val):
        rot, pos, scale = primary_params(tel, device)
        ps = pack_scene(tel, device, tuple(t.detach().contiguous() for t in (rot, pos, scale)))
        mrot, mpos, msurf = _stage_params(tel, device)
        prim = stages_of(tel).get(0, [])
        if any(t.requires_grad for g in prim for t in (g.points, g.normals, g.perturbation_delta, g.weights)):
            spts, snrm, sdlt, swts = primary_samples(tel, device)
        else:  # sample arrays are constants: nothing to carry
            spts = snrm = sdlt = _empty((0, 0, 3), device)
            swts = _empty((0, 0), device)
        return RenderFunction.apply((ps, sensor, code, mode, shape, opts), rot, pos, scale, src, val,
                                    mrot, mpos, msurf, spts, snrm, sdlt, swts)
    ps = pack_scene(tel, device)
    sdesc, keep = sensor.pack(device)
    out = _forward(ps, ps.desc, sdesc, code, src, val, mode, shape, opts, device)
    del keep
    return out


def render(tel, sources, values, source_type="point", sensor_idx=0, opts=None, seed=0):
    """core/render.py:174-220: image with the sensor's accumulator shape."""
    return _launch(tel, sources, values, source_type, sensor_idx, N.MODE_IMAGE, opts, seed)


def render_response_matrix(tel, sources, values, source_type="point", sensor_idx=0, opts=None, seed=0):
    """core/render.py:271-324: (n_sources, n_pixels) per-source rows."""
    return _launch(tel, sources, values, source_type, sensor_idx, N.MODE_RESPONSE, opts, seed)


def render_debug(tel, sources, values, source_type="point", sensor_idx=0, extras=False, seed=0):
    """core/render.py:223-268: raw hits (F*S*M, 2) and values (F*S*M,), ray
    order (facet, source, sample). With extras=True also the hard pixel id
    and the index of the last stage mirror hit per ray."""
    device = _device()
    sensor = tel.sensors[sensor_idx]
    src, val = _inputs(sources, values, device, source_type)
    S = int(src.shape[0])
    if 0 not in stages_of(tel):
        z = (torch.zeros((0, 2), device=device), torch.zeros((0,), device=device))
        return z + (torch.zeros(0, dtype=torch.int32, device=device),) * 2 if extras else z
    lib = N.load()
    ps = pack_scene(tel, device)
    sdesc, keep = sensor.pack(device)
    n = ps.F * S * ps.M
    pts = torch.empty((n, 2), dtype=torch.float32, device=device)
    vals = torch.empty((n,), dtype=torch.float32, device=device)
    pix = torch.empty((n,), dtype=torch.int32, device=device) if extras else None
    hm = torch.empty((n,), dtype=torch.int32, device=device) if extras else None
    ws = _workspace(ps, sdesc, S, N.MODE_DEBUG, device)
    stream = torch.cuda.current_stream(device).cuda_stream
    N.check(lib.iact_render_debug(ctypes.byref(ps.desc), ctypes.byref(sdesc), source_code(source_type),
                                  src.data_ptr(), val.data_ptr(), S, pts.data_ptr(), vals.data_ptr(),
                                  pix.data_ptr() if extras else None, hm.data_ptr() if extras else None,
                                  ws.data_ptr(), ws.numel(), int(seed) & 0xFFFFFFFF, stream))
    del keep
    return (pts, vals, pix, hm) if extras else (pts, vals)
