"""Per-device cache of a sensor's packed descriptor."""
from __future__ import annotations

import torch


def _key(x):
    if isinstance(x, torch.Tensor):
        return (x.data_ptr(), x._version, tuple(x.shape))
    return x


def pack_cached(sensor, device, pack):
    """pack(device) memoised on the sensor, keyed by the device, the pose
    tensors (storage and version; the entry keeps them alive, so the
    addresses stay unique) and the scalar settings."""
    scal = tuple(sorted((k, v) for k, v in vars(sensor).items()
                        if isinstance(v, (bool, int, float, str)) and not k.startswith("_")))
    key = (str(device), _key(sensor.position), _key(sensor.rotation), scal)
    hit = sensor.__dict__.get("_packed_desc")
    if hit is not None and hit[0] == key:
        return hit[2]
    out = pack(device)
    sensor.__dict__["_packed_desc"] = (key, (sensor.position, sensor.rotation), out)
    return out
