"""The C ABI library loads on a machine without a GPU and exports every
function declared in include/*.h; host-only entry points work."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(mhm_[a-z0-9_]+)\s*\(", text, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "mhm_ctx_create" in names and "mhm_run" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from mhm_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.EXPORTS)


def test_version_and_invalid_args(lib):
    a, b = C.c_int32(), C.c_int32()
    assert lib.mhm_version(C.byref(a), C.byref(b)) == 0
    assert lib.mhm_ctx_create(None, 0, None) == -1
    assert lib.mhm_run(None, 1, 1, None) == -1


def test_host_routing_order_and_calendar(lib):
    from mhm_gb300 import synth
    dom = synth.make_domain(12, 16, 2, 4, seed=4)
    assert sorted(dom.net_perm[: dom.n_links]) == list(range(1, dom.n_links + 1))
    m = np.zeros(48, np.int32)
    ip = C.POINTER(C.c_int32)
    assert lib.mhm_step_calendar(synth.JUL_2000, 1, 1, 48, m.ctypes.data_as(ip), None, None) == 0
    assert (m == 1).all()
