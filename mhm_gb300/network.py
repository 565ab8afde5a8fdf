"""mRM's routing-network start-up from level-0 flow data (the library's
mhm_l11_network, host code): L11 flow directions, links, routing order, link
lengths, slopes, floodplains and their sealed fractions
(src/mRM/mo_mrm_net_startup.f90:227-1594)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


# rotate_fdir_variable (src/mRM/mo_mrm_read_data.f90:527-597): flow
# directions of an ESRI-style grid file become mRM's codes on the transposed
# (x, y) grid
_ROTATE = {1: 4, 2: 2, 4: 1, 8: 128, 16: 64, 32: 32, 64: 16, 128: 8}


def rotate_fdir(fdir):
    """mRM's internal flow-direction codes from those read from a grid file."""
    f = np.asarray(fdir, np.int32)
    out = f.copy()
    for a, b in _ROTATE.items():
        out[f == a] = b
    return out


def l11_network(nrows0: int, ncols0: int, mask0, fdir0, facc0, elev0, cellsize0: float, factor: int,
                lcover0=None, lc_class_imp: int = 2) -> dict:
    """mask0 [ncols0 * nrows0] (mHM's column-major (x, y) order), fdir0 (mRM's
    internal codes: rotate_fdir of a grid file's) / facc0 / elev0 packed over
    the mask, lcover0 [scenes][cells] or None.
    Returns the L11 arrays (1-based link and node indexes as mRM's)."""
    L = _lib.load()
    m = np.ascontiguousarray(mask0, np.uint8)
    n = C.c_int32()
    rc = L.mhm_l11_network_size(nrows0, ncols0, m.ctypes.data_as(C.POINTER(C.c_uint8)), factor, C.byref(n))
    if rc != 0:
        raise ValueError("mhm_l11_network_size failed")
    nn = n.value
    fd = np.ascontiguousarray(fdir0, np.int32)
    fa = np.ascontiguousarray(facc0, np.int32)
    el = np.ascontiguousarray(elev0, np.float64)
    lc = None if lcover0 is None else np.ascontiguousarray(np.atleast_2d(lcover0), np.int32)
    ns = 0 if lc is None else lc.shape[0]
    ip = C.POINTER(C.c_int32)
    dp = C.POINTER(C.c_double)
    inp = _lib.L0Flow(nrows0, ncols0, factor, fd.size, m.ctypes.data_as(C.POINTER(C.c_uint8)), fd.ctypes.data_as(ip),
                      fa.ctypes.data_as(ip), el.ctypes.data_as(dp), float(cellsize0), ns, lc_class_imp,
                      lc.ctypes.data_as(ip) if lc is not None else None)
    out = {k: np.zeros(nn, np.int32) for k in ("fdir11", "cell_row11", "cell_col11", "from_n", "to_n", "net_perm",
                                               "r_order", "row_out", "col_out")}
    out.update({k: np.zeros(nn) for k in ("length", "slope", "a_floodplain")})
    out["frac_fp_imp"] = np.zeros((max(ns, 1), nn))
    o = _lib.L11Network()
    for k, v in out.items():
        setattr(o, k, v.ctypes.data_as(ip if v.dtype == np.int32 else dp))
    rc = L.mhm_l11_network(C.byref(inp), C.byref(o))
    if rc != 0:
        raise ValueError("mhm_l11_network failed (see stderr)")
    nl = o.n_links
    res = dict(out)
    res.update(n_nodes=o.n_nodes, n_outlets=o.n_outlets, n_links=nl, nrows11=o.nrows11, ncols11=o.ncols11,
               n_l0_outlets=o.n_l0_outlets)
    for k in ("length", "slope", "a_floodplain"):
        res[k] = res[k][:nl]
    res["frac_fp_imp"] = res["frac_fp_imp"][:ns, :nl]
    return res


def l1_l11_mapping(nrows0: int, ncols0: int, mask0, factor1: int, factor11: int):
    """(L1_L11_Id, L11_L1_Id) of mhm_l1_l11_mapping."""
    L = _lib.load()
    m = np.ascontiguousarray(mask0, np.uint8)
    mp = m.ctypes.data_as(C.POINTER(C.c_uint8))
    n1, n11 = C.c_int32(), C.c_int32()
    if L.mhm_l11_network_size(nrows0, ncols0, mp, factor1, C.byref(n1)) or \
            L.mhm_l11_network_size(nrows0, ncols0, mp, factor11, C.byref(n11)):
        raise ValueError("grid sizes")
    a = np.zeros(n1.value, np.int32)
    b = np.zeros(n11.value, np.int32)
    ip = C.POINTER(C.c_int32)
    if L.mhm_l1_l11_mapping(nrows0, ncols0, mp, factor1, factor11, a.ctypes.data_as(ip), b.ctypes.data_as(ip)):
        raise ValueError("mhm_l1_l11_mapping failed (see stderr)")
    return a, b
