"""Round a decimal literal to binary32 exactly as rustc does (round-to-nearest-even on the
exact decimal value; a leading '-' negates, so "-0.0" is negative zero)."""
import struct
from fractions import Fraction

import numpy as np


def _bits(x):
    return struct.unpack("<I", struct.pack("<f", float(x)))[0]


def f32lit(s):
    s = str(s).strip()
    neg = s.startswith("-")
    fr = abs(Fraction(s))
    x = np.float32(float(fr))
    cands = [np.nextafter(x, np.float32(0)), x, np.nextafter(x, np.float32(np.inf))]
    best = min(cands, key=lambda c: (abs(Fraction(float(c)) - fr), _bits(c) & 1))
    best = np.float32(best)
    return np.float32(-best) if neg else best


def arr(x):
    """Nested lists of literals -> float32 ndarray."""
    if isinstance(x, (list, tuple)):
        return np.array([arr(v) for v in x], dtype=np.float32)
    return f32lit(x)
