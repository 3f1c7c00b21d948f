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
    # batches: no such device, null handles
    h = C.c_void_p()
    assert L.vgn_batch_create(9999, C.byref(h)) == N.VGN_ERR_ARG and not h
    assert L.vgn_batch_step(None, None) == N.VGN_ERR_ARG
    assert L.vgn_batch_set_jobs(None, 1, None, 0, 0, 0) == N.VGN_ERR_ARG
    assert L.vgn_batch_free(None) == N.VGN_OK


CPP_PROGRAM = r"""
#include <cstdio>
#include "vgnav.hpp"
int main() {
  // world box (lv 0) holding one box daughter (lv 1); placement 0 = daughter, 1 = world
  const int32_t lv_shape[2] = {VGN_BOX, VGN_BOX}, lv_off[2] = {0, 3};
  const double params[6] = {100, 100, 100, 10, 20, 30};
  const int32_t pv_lv[2] = {1, 0}, pv_mother[2] = {0, -1};
  const double tr[24] = {5, 6, 7, 1, 0, 0, 0, 1, 0, 0, 0, 1,  0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  vgn_geometry_desc d{2, lv_shape, lv_off, params, 6, 2, pv_lv, pv_mother, tr, 1};
  vgnav::Geometry g(d, VGN_HOST_ONLY);
  const uint32_t *tab = nullptr; size_t n = 0;
  vgnav::check(vgn_geometry_navindex(g.get(), &tab, &n));
  std::printf("%zu %u %u %zu %s\n", n, tab[2], tab[3], g.device_bytes(), vgn_version());
  try {
    vgnav::BVHNavigator nav(g);
    double x = 0; vgn_state s{}; vgnav::SOA3D p{&x, &x, &x, 1}; vgnav::NavStatePool pool{&s, 1};
    nav.LocatePoints(p, pool);
  } catch (const vgnav::Error &e) { std::printf("error %d\n", e.code()); }
  return 0;
}
"""


def test_cpp_header_builds_and_links(vgnav, tmp_path):
    """include/vgnav.hpp (the C++ host interface) compiles, links against libvgnav and runs on
    a host-only geometry; the navigation table of world + one daughter has the reference layout."""
    import subprocess

    from helpers import ROOT

    src = tmp_path / "t.cpp"
    src.write_text(CPP_PROGRAM)
    exe = tmp_path / "t"
    libdir = ROOT / "vecgeom_gb300" / "lib"
    subprocess.run(["g++", "-std=c++17", "-I", str(ROOT / "include"), str(src), "-L", str(libdir), "-lvgnav",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    n, pv_world, word3, dev_bytes, ver = out[0].split(" ", 4)
    assert "sm_103a" in ver
    assert int(pv_world) == 1  # record of the world placement (id 1)
    # world: 3 + 1 daughter + pad 0 = 4 words, pad to 8-byte boundary: (1 + 4) odd -> 1 pad word, 24 matrix words;
    # daughter: 3 words + 1 pad + ... -> table of 1 + 29 + 28 = 58 words + 1 allocation word
    assert int(n) == 59
    assert int(word3) == (1 << 16) | (0x04 << 8) | 0  # world: level 0, matrix cached (identity), 1 daughter
    assert int(dev_bytes) == 0
    assert out[1] == f"error {1}"  # kernels refused on a host-only geometry (VGN_ERR_ARG)


def test_c_header_is_plain_c(tmp_path):
    import subprocess

    from helpers import ROOT

    src = tmp_path / "t.c"
    src.write_text('#include "vgnav.h"\nint main(void) { vgn_state s; (void)s; return 0; }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                   check=True)


def test_step_config_host_logic(vgnav):
    """Launch configuration setters/getters and their argument checks (host-only geometry, no kernel)."""
    from helpers import HostTables
    from vecgeom_gb300 import workloads as W

    h = HostTables(W.box_grid_geometry(seed=7, n=5).desc)
    L = N.lib()
    v, k = C.c_int32(-1), C.c_int32(-1)
    for mixed in (0, N.VGN_PRECISION_MIXED):
        assert L.vgn_get_step_config(h.h, mixed, C.byref(v), C.byref(k)) == N.VGN_OK
        assert (v.value, k.value) == (0, 0)
    assert L.vgn_set_step_config(h.h, N.VGN_PRECISION_MIXED, 2, 4) == N.VGN_OK
    L.vgn_get_step_config(h.h, N.VGN_PRECISION_MIXED, C.byref(v), C.byref(k))
    assert (v.value, k.value) == (2, 4)
    L.vgn_get_step_config(h.h, 0, C.byref(v), C.byref(k))
    assert (v.value, k.value) == (0, 0)  # forms are configured independently
    assert L.vgn_set_step_config(h.h, 0, 99, 0) == N.VGN_ERR_ARG
    # the block-grouped variants exist for the mixed form only
    nv = C.c_int32()
    assert L.vgn_get_step_variant_count(0, C.byref(nv)) == N.VGN_OK and nv.value == 6
    assert L.vgn_get_step_variant_count(N.VGN_PRECISION_MIXED, C.byref(nv)) == N.VGN_OK and nv.value == 9
    assert L.vgn_set_step_config(h.h, N.VGN_PRECISION_MIXED, 8, 5) == N.VGN_OK
    assert L.vgn_set_step_config(h.h, N.VGN_PRECISION_MIXED, 9, 5) == N.VGN_ERR_ARG
    assert L.vgn_set_step_config(h.h, 0, 6, 5) == N.VGN_ERR_ARG
    assert L.vgn_set_step_config(h.h, N.VGN_PRECISION_MIXED, 2, 4) == N.VGN_OK
    assert L.vgn_get_step_variant_count(0, None) == N.VGN_ERR_ARG
    assert L.vgn_set_step_config(h.h, 0, 0, -1) == N.VGN_ERR_ARG
    assert L.vgn_set_step_config(h.h, 0, 0, 7) == N.VGN_ERR_ARG
    assert L.vgn_set_step_config(None, 0, 0, 0) == N.VGN_ERR_ARG
    # the safety pass's own (position-only) binning
    ks = C.c_int32(-1)
    assert L.vgn_get_safety_binning(h.h, N.VGN_PRECISION_MIXED, C.byref(ks)) == N.VGN_OK and ks.value == 0
    assert L.vgn_set_safety_binning(h.h, N.VGN_PRECISION_MIXED, 6) == N.VGN_OK
    L.vgn_get_safety_binning(h.h, N.VGN_PRECISION_MIXED, C.byref(ks))
    assert ks.value == 6
    L.vgn_get_safety_binning(h.h, 0, C.byref(ks))
    assert ks.value == 0
    for bad in (-1, 7):
        assert L.vgn_set_safety_binning(h.h, 0, bad) == N.VGN_ERR_ARG
    assert L.vgn_set_safety_binning(None, 0, 1) == N.VGN_ERR_ARG
    assert L.vgn_get_safety_binning(h.h, 0, None) == N.VGN_ERR_ARG
    # the autotuner needs a device geometry
    assert L.vgn_autotune_step(h.h, 1, *([None] * 11), 0, None, None, None, None) == N.VGN_ERR_ARG
