"""The C-ABI library loads and exports every symbol include/vgnav.h declares
(no kernel is launched: runs without a GPU)."""
import ctypes as C

from helpers import header_symbols
from vecgeom_gb300 import _native as N


def test_header_symbols_exported(vgnav):
    L = N.lib()
    syms = header_symbols()
    assert len(syms) >= 14
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(N.EXPORTED) == set(syms)


def test_state_layout_matches_navstateindex():
    assert C.sizeof(N.VgnState) == 12
    from vecgeom_gb300.workloads import STATE_DTYPE

    assert STATE_DTYPE.itemsize == 12


def test_version_and_errors(vgnav):
    L = N.lib()
    assert b"sm_103a" in L.vgn_version()
    assert L.vgn_compute_step_batch(None, 1, *([None] * 11), 0, None) == N.VGN_ERR_ARG
    assert b"null geometry" in L.vgn_last_error()
