"""Host utilities of the adaptive routing cases.

Routing case 3 gives every link its own celerity (L11_calc_celerity,
src/mRM/mo_mrm_net_startup.f90:2212-2423): along the link's river path at
L0, from its source cell to its outlet cell inclusive, each cell's celerity
is slope_factor * sqrt(slope / 100) (slope in percent), and the link's is
their harmonic mean, n / sum(1 / c) summed in path order.  The reference
first bounds the L0 slopes below by 0.1 and filters outliers on the stream
network with the median-absolute-deviation test of its FORCES library
(not part of the reference tree); the slopes passed here are the filtered
ones.  mhm_set_link_celerity takes the result.
"""
from __future__ import annotations

import numpy as np


def link_celerity(slope_factor: float, path_ptr, path_slope) -> np.ndarray:
    """Celerity [m s-1] of each link from its L0 path slopes [%]: path_ptr
    [n_links + 1] offsets into path_slope (one run of cells per link)."""
    ptr = np.asarray(path_ptr, np.int64)
    sl = np.asarray(path_slope, np.float64)
    n = np.diff(ptr)
    if np.any(n < 1):
        raise ValueError("every link's path holds at least its source cell")
    inv = np.zeros(n.size)
    for j in range(int(n.max())):            # one path position at a time: sums in path order
        on = n > j
        inv[on] = inv[on] + 1.0 / (slope_factor * np.sqrt(sl[ptr[:-1][on] + j] / 100.0))
    return n.astype(np.float64) / inv
