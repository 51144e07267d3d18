"""uv-table ingest: the plain-text visibility tables galario's documentation uses.

Format (reference docs/quickstart.rst:32-63 and docs/uvtable.txt): one
visibility per line, whitespace-separated columns u, v [metres or
wavelengths], Re, Im [Jy], w [1/Jy^2]; lines starting with '#' are comments.
``load_uvtable`` returns C-contiguous float64 arrays with u and v divided by
the observing wavelength ``wle`` (metres; 1 when the table is already in
wavelengths), ready for ``galario_gb300.double`` or ``batch.Dataset``.
"""
from __future__ import annotations

import numpy as np


def load_uvtable(path, wle: float = 1.0, columns=(0, 1, 2, 3, 4)):
    """Read u, v, Re, Im, w from a uv-table; u, v are returned in wavelengths (u / wle)."""
    if not (wle > 0):
        raise ValueError("wle must be positive, got {}".format(wle))
    data = np.loadtxt(path, comments="#", usecols=columns, ndmin=2)
    if data.shape[1] != 5:
        raise ValueError("expected 5 columns (u, v, Re, Im, w), got {}".format(data.shape[1]))
    u, v, re, im, w = (np.ascontiguousarray(data[:, i], dtype=np.float64) for i in range(5))
    if np.any(w < 0):
        raise ValueError("negative weights in {}".format(path))
    return u / wle, v / wle, re, im, w


def write_uvtable(path, u, v, re, im, w, wle: float = 1.0, header: str = ""):
    """Write a uv-table (u, v multiplied by wle, so that load_uvtable(path, wle) restores them)."""
    cols = np.column_stack([np.asarray(u) * wle, np.asarray(v) * wle, re, im, w])
    np.savetxt(path, cols, fmt="%.17g", delimiter="\t", header=header)
