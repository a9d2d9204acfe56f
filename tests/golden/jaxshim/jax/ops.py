import numpy as _np

from .numpy import _unwrap, _wrap


def segment_sum(data, segment_ids, num_segments=None, **kw):
    d = _np.asarray(_unwrap(data))
    ids = _np.asarray(_unwrap(segment_ids)).astype(_np.int64)
    out = _np.zeros((num_segments,) + d.shape[1:], d.dtype)
    ok = (ids >= 0) & (ids < num_segments)   # XLA drops out-of-range ids
    _np.add.at(out, ids[ok], d[ok])
    return _wrap(out)
