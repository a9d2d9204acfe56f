from .keys import Key, key, split
from .sampling import sample_disk, sample_polygon

__all__ = ["sample_disk", "sample_polygon", "key", "split", "Key"]
