"""Hilbert keys for cell ordering (host side, numpy).

Restates ``hilbert_key_2d`` of the reference (``phd/hilbert/hilbert.pyx:9-23``) as a
vectorised loop over key bits, with the quantisation of
``LoadBalance.compute_hilbert_keys`` (``phd/load_balance/load_balance.pyx:195-217``):
``xh = int32((x - corner) * 2**order / box_length)`` (truncation toward zero),
``order = 18`` (``load_balance.pyx:14``).

The device path uses the same key (``phd_hilbert_keys_2d`` in the C-ABI); both are
checked bit-for-bit against the reference's ``py_hilbert_key_2d``.
"""
import numpy as np

ORDER = 18

# index of each (xbit, ybit) quadrant along the curve (hilbert.pyx:6)
_KEY_INDEX_2D = np.array([0, 1, 3, 2], dtype=np.int64)


def hilbert_key_2d(xh, yh, order=ORDER):
    """Keys for integer coordinates ``xh, yh`` (int32 arrays), hilbert.pyx:9-23.

    Each bit level selects a quadrant; quadrant (0,0) swaps x and y, quadrant (1,0)
    swaps and complements them (``~`` on int32, two's complement), exactly as the
    reference does.
    """
    x = np.asarray(xh, dtype=np.int32).copy()
    y = np.asarray(yh, dtype=np.int32).copy()
    key = np.zeros(x.shape, dtype=np.int64)
    for i in range(order - 1, -1, -1):
        bit = np.int32(1 << i)
        xbit = ((x & bit) != 0).astype(np.int64)
        ybit = ((y & bit) != 0).astype(np.int64)
        q00 = (xbit == 0) & (ybit == 0)
        q10 = (xbit == 1) & (ybit == 0)
        nx = np.where(q00, y, np.where(q10, ~y, x))
        ny = np.where(q00, x, np.where(q10, ~x, y))
        x, y = nx.astype(np.int32), ny.astype(np.int32)
        key = (key << 2) + _KEY_INDEX_2D[(xbit << 1) + ybit]
    return key


def quantize(x, corner, box_length, order=ORDER):
    """Integer coordinates of load_balance.pyx:195-217 (``fac = 2**order/box_length``)."""
    fac = float(2 ** order) / float(box_length)
    q = (np.asarray(x, dtype=np.float64) - float(corner)) * fac
    return np.trunc(q).astype(np.int32)


def hilbert_keys(x, y, xmin, box_length, order=ORDER):
    """Keys of positions ``x, y`` in a box with lower corner ``xmin`` (2-vector)."""
    return hilbert_key_2d(quantize(x, xmin[0], box_length, order),
                          quantize(y, xmin[1], box_length, order), order)


def hilbert_order(x, y, xmin, box_length, order=ORDER):
    """Stable permutation sorting the points along the curve."""
    return np.argsort(hilbert_keys(x, y, xmin, box_length, order), kind="stable")
