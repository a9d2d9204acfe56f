from .mirrors import AsphericDiskMirrorGroup, AsphericPolygonMirrorGroup, Mirror, MirrorGroup, group_mirrors
from .telescope import Telescope

__all__ = ["Telescope", "Mirror", "MirrorGroup", "AsphericDiskMirrorGroup", "AsphericPolygonMirrorGroup",
           "group_mirrors"]
