"""Obstructions (core/obstructions.py of the reference).

Single primitives and their SoA groups. The render kernels evaluate the
intersection math on the device (shadowing is "some member's t < 1e10",
core/render.py:21-41); these classes hold the tables and pack them into the
C ABI layout.
"""
from __future__ import annotations

import torch


def _t(x):
    return torch.as_tensor(x, dtype=torch.float32)


class Obstruction:
    kind = ""


class ObstructionGroup:
    kind = ""
    stride = 0

    def __len__(self):
        raise NotImplementedError

    def table(self) -> torch.Tensor:
        """Rows in the C ABI layout of this kind (include/iactrace_gb300.h)."""
        raise NotImplementedError


class Cylinder(Obstruction):
    """core/obstructions.py:38-51."""
    kind = "cyl"

    def __init__(self, p1, p2, radius):
        self.p1, self.p2, self.radius = _t(p1), _t(p2), float(radius)


class CylinderGroup(ObstructionGroup):
    """core/obstructions.py:54-79: p1 (N,3), p2 (N,3), r (N,)."""
    kind = "cyl"
    stride = 7

    def __init__(self, cylinders=None, p1=None, p2=None, r=None):
        if cylinders is not None:
            self.p1 = torch.stack([c.p1 for c in cylinders])
            self.p2 = torch.stack([c.p2 for c in cylinders])
            self.r = _t([c.radius for c in cylinders])
        else:
            self.p1, self.p2, self.r = _t(p1).reshape(-1, 3), _t(p2).reshape(-1, 3), _t(r).reshape(-1)

    def __len__(self):
        return self.p1.shape[0]

    def table(self):
        return torch.cat([self.p1, self.p2, self.r[:, None]], 1)


class Box(Obstruction):
    """core/obstructions.py:84-95 (axis aligned)."""
    kind = "box"

    def __init__(self, p1, p2):
        self.p1, self.p2 = _t(p1), _t(p2)


class BoxGroup(ObstructionGroup):
    """core/obstructions.py:98-120."""
    kind = "box"
    stride = 6

    def __init__(self, boxes=None, p1=None, p2=None):
        if boxes is not None:
            self.p1 = torch.stack([b.p1 for b in boxes])
            self.p2 = torch.stack([b.p2 for b in boxes])
        else:
            self.p1, self.p2 = _t(p1).reshape(-1, 3), _t(p2).reshape(-1, 3)

    def __len__(self):
        return self.p1.shape[0]

    def table(self):
        return torch.cat([self.p1, self.p2], 1)


class Sphere(Obstruction):
    """core/obstructions.py:125-136."""
    kind = "sph"

    def __init__(self, center, radius):
        self.center, self.radius = _t(center), float(radius)


class SphereGroup(ObstructionGroup):
    """core/obstructions.py:139-161."""
    kind = "sph"
    stride = 4

    def __init__(self, spheres=None, centers=None, radii=None):
        if spheres is not None:
            self.centers = torch.stack([s.center for s in spheres])
            self.radii = _t([s.radius for s in spheres])
        else:
            self.centers, self.radii = _t(centers).reshape(-1, 3), _t(radii).reshape(-1)

    def __len__(self):
        return self.centers.shape[0]

    def table(self):
        return torch.cat([self.centers, self.radii[:, None]], 1)


class OrientedBox(Obstruction):
    """core/obstructions.py:166-181: rotation is local -> world."""
    kind = "obox"

    def __init__(self, center, half_extents, rotation):
        self.center, self.half_extents = _t(center), _t(half_extents)
        self.rotation = _t(rotation).reshape(3, 3)


class OrientedBoxGroup(ObstructionGroup):
    """core/obstructions.py:184-209."""
    kind = "obox"
    stride = 15

    def __init__(self, boxes=None, centers=None, half_extents=None, rotations=None):
        if boxes is not None:
            self.centers = torch.stack([b.center for b in boxes])
            self.half_extents = torch.stack([b.half_extents for b in boxes])
            self.rotations = torch.stack([b.rotation for b in boxes])
        else:
            self.centers = _t(centers).reshape(-1, 3)
            self.half_extents = _t(half_extents).reshape(-1, 3)
            self.rotations = _t(rotations).reshape(-1, 3, 3)

    def __len__(self):
        return self.centers.shape[0]

    def table(self):
        return torch.cat([self.centers, self.half_extents, self.rotations.reshape(-1, 9)], 1)


class Triangle(Obstruction):
    """core/obstructions.py:214-227."""
    kind = "tri"

    def __init__(self, v0, v1, v2):
        self.v0, self.v1, self.v2 = _t(v0), _t(v1), _t(v2)


class TriangleGroup(ObstructionGroup):
    """core/obstructions.py:230-255."""
    kind = "tri"
    stride = 9

    def __init__(self, triangles=None, v0=None, v1=None, v2=None):
        if triangles is not None:
            self.v0 = torch.stack([t.v0 for t in triangles])
            self.v1 = torch.stack([t.v1 for t in triangles])
            self.v2 = torch.stack([t.v2 for t in triangles])
        else:
            self.v0, self.v1, self.v2 = (_t(v).reshape(-1, 3) for v in (v0, v1, v2))

    def __len__(self):
        return self.v0.shape[0]

    def table(self):
        return torch.cat([self.v0, self.v1, self.v2], 1)


def group_obstructions(obstructions):
    """core/obstructions.py:258-277: one group per kind, in a fixed kind order."""
    out = []
    for cls, gcls, kw in ((Cylinder, CylinderGroup, "cylinders"), (Box, BoxGroup, "boxes"),
                          (Sphere, SphereGroup, "spheres"), (OrientedBox, OrientedBoxGroup, "boxes"),
                          (Triangle, TriangleGroup, "triangles")):
        items = [o for o in obstructions if isinstance(o, cls)]
        if items:
            out.append(gcls(**{kw: items}))
    return out
