"""Operator files in the byte layout of Dcpse::save / Dcpse::load
(src/DCPSE/Dcpse.hpp:302-379): openfpm's Packer writes each openfpm::vector
of a primitive type as its element count (size_t) followed by the elements,
in native byte order, for localEps, localEpsInvPow, calcKernels (float64) and
kerOffsets (size_t), one file per rank named file + "_" + rank."""
from __future__ import annotations

import numpy as np

_U64 = np.dtype("<u8") if np.little_endian else np.dtype(">u8")


def _pack(fh, arr, dtype):
    a = np.ascontiguousarray(arr, dtype=dtype)
    np.array([a.size], dtype=np.uint64).tofile(fh)
    a.tofile(fh)


def write(path, eps, eip, K, offsets):
    """eps, eip [n], K [nnz] float64; offsets [n] start of each particle's
    kernels in K (kerOffsets)."""
    with open(path, "wb") as fh:
        _pack(fh, eps, np.float64)
        _pack(fh, eip, np.float64)
        _pack(fh, K, np.float64)
        _pack(fh, offsets, np.uint64)


def read(path):
    """-> (eps, eip, K, offsets); raises ValueError on a malformed file."""
    buf = open(path, "rb").read()
    out = []
    pos = 0
    for dtype in (np.float64, np.float64, np.float64, np.uint64):
        if pos + 8 > len(buf):
            raise ValueError("%s: truncated" % path)
        n = int(np.frombuffer(buf, dtype=np.uint64, count=1, offset=pos)[0])
        pos += 8
        if n > (len(buf) - pos) // 8:
            raise ValueError("%s: vector of %d elements does not fit the file" % (path, n))
        out.append(np.frombuffer(buf, dtype=dtype, count=n, offset=pos).copy())
        pos += 8 * n
    return tuple(out)
