"""mRM's routing-network start-up from level-0 flow data (mhm_l11_network,
host code) against the network the reference itself built for its
regression case check/case_00: from the 500 m flow directions, flow
accumulation and elevation of test_domain (46,545 L0 cells) to the 24 km
L11 network -- flow directions, links, routing order, link lengths, slopes
and the floodplain sealed fractions of both land-cover scenes, as stored in
case_00's b1_mRM_restart_001.nc -- bit for bit.  Plus the L1 -> L11 mapping
on case_00 and on the synthetic basins."""
from pathlib import Path

import numpy as np
import pytest

from mhm_gb300 import network, synth

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def case00():
    n = np.load(GOLD / "case00_net.npz")
    m = np.load(GOLD / "case00_mpr.npz")
    r = np.load(GOLD / "case00_run.npz")
    mask0 = np.unpackbits(m["mask0"])[: int(m["n_mask0"])]
    return n, m, r, mask0


def test_case00_network_equals_the_reference(case00):
    n, m, r, mask0 = case00
    res = network.l11_network(int(n["nrows0"]), int(n["ncols0"]), mask0, network.rotate_fdir(n["fdir0"]),
                              n["facc0"], n["elev0"], float(n["cellsize0"]), int(n["factor11"]),
                              m["lcover0"].astype(np.int32))
    assert res["n_nodes"] == 34 and res["n_outlets"] == 1 and res["n_links"] == 33
    for k, g in (("fdir11", "l11_fdir"), ("from_n", "from_n"), ("to_n", "to_n"), ("net_perm", "net_perm"),
                 ("r_order", "r_order")):
        assert np.array_equal(res[k], r[g]), k
    for k, g in (("length", "length"), ("slope", "slope"), ("frac_fp_imp", "ffp_imp")):
        a, b = np.asarray(res[k], np.float64), np.asarray(r[g], np.float64)
        assert a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64)), k
    # the floodplains are areas of whole L0 cells
    assert np.all(res["a_floodplain"] > 0) and np.all(np.mod(res["a_floodplain"], 250000.0) == 0)


def test_case00_l1_mapping(case00):
    n, m, r, mask0 = case00
    f = int(n["factor11"])
    l1_l11, l11_l1 = network.l1_l11_mapping(int(n["nrows0"]), int(n["ncols0"]), mask0, f, f)
    assert np.array_equal(l1_l11, r["l1_l11_id"])
    assert np.all(l11_l1 == -9999)


@pytest.mark.parametrize("nr,nc,f11", [(24, 32, 4), (37, 21, 4), (16, 20, 2)])
def test_synthetic_l1_mapping(nr, nc, f11):
    dom = synth.make_domain(nr, nc, 2, f11, seed=2)
    mask0 = np.ones(nr * nc, np.uint8)        # L0 = L1, full rectangle
    l1_l11, l11_l1 = network.l1_l11_mapping(nr, nc, mask0, 1, f11)
    assert np.array_equal(l1_l11, dom.l1_l11_id)
    assert np.all(l11_l1 == -9999)
    # an L11 grid finer than L1: every L11 cell names its L1 cell
    l1_l11b, l11_l1b = network.l1_l11_mapping(nr, nc, mask0, 2, 1)
    assert np.all(l1_l11b == -9999) and l11_l1b.min() >= 1 and l11_l1b.max() == len(l1_l11b)


def test_fdir_rotation_is_an_involution():
    codes = np.array([1, 2, 4, 8, 16, 32, 64, 128, -9999], np.int32)
    rot = network.rotate_fdir(codes)
    assert list(rot) == [4, 2, 1, 128, 64, 32, 16, 8, -9999]
    assert np.array_equal(network.rotate_fdir(rot), codes)
