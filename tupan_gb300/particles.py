"""A minimal particle set for the extension objects, for callers without tupan.

``tupan_gb300.extensions`` reads the attributes tupan's ``ParticleSystem``
has (``n``, ``mass``, ``eps2``, ``rx`` ... ``jz``;
tupan/particles/body.py:26-39) and registers its outputs with
``register_auxiliary_attribute`` (tupan/particles/allparticles.py:64-76).
``Bodies`` is that surface over plain contiguous numpy arrays (ordinary
pageable host memory, as tupan holds them), so the drop-in objects can be
driven without importing tupan itself.
"""

import numpy as np

ATTRS = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz",
         "ax", "ay", "az", "jx", "jy", "jz")
SHORT = {"mass": "m", "eps2": "e2"}


class Bodies(object):
    """Particle attributes as contiguous 1-d arrays of ``dtype``.

    ``arrays`` maps the short names (m, e2, rx ... jz) or tupan's names
    (mass, eps2, ...) to arrays of equal length; missing attributes are
    zero.  Arrays are copied unless ``copy=False`` and they already have the
    right dtype and layout."""

    def __init__(self, arrays, dtype=np.float64, copy=True):
        n = None
        for a in ATTRS:
            v = arrays.get(SHORT.get(a, a), arrays.get(a))
            if v is not None:
                n = len(v)
                break
        if n is None:
            raise ValueError("no particle attribute given")
        self.n = n
        self._dtype = np.dtype(dtype)
        for a in ATTRS:
            v = arrays.get(SHORT.get(a, a), arrays.get(a))
            if v is None:
                v = np.zeros(n, dtype=self._dtype)
            elif copy:
                v = np.array(v, dtype=self._dtype, order="C", copy=True)
            else:
                v = np.ascontiguousarray(v, dtype=self._dtype)
            if len(v) != n:
                raise ValueError("attribute %s has %d entries, not %d"
                                 % (a, len(v), n))
            setattr(self, a, v)

    def register_auxiliary_attribute(self, name, kind):
        setattr(self, name, np.zeros(self.n, dtype=self._dtype))

    def subset(self, index):
        """A new set with the particles ``index`` (copies, like tupan's
        sub-selections)."""
        return Bodies({a: getattr(self, a)[index] for a in ATTRS},
                      dtype=self._dtype)
