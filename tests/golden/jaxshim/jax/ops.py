import numpy as _np


def segment_sum(data, segment_ids, num_segments=None, **kw):
    """Scatter-add; ids outside [0, num_segments) are dropped (JAX's default)."""
    data = _np.asarray(data)
    ids = _np.asarray(segment_ids).astype(_np.int64)
    out = _np.zeros((num_segments,) + data.shape[1:], dtype=data.dtype)
    ok = (ids >= 0) & (ids < num_segments)
    _np.add.at(out, ids[ok], data[ok])
    return out
