"""The C-ABI library builds, loads and exports every entry point the public
header declares; host-side argument validation answers without a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "diffrp_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(drp_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from diffrp_gb300 import build, _ffi
    build.build()
    return _ffi.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ["drp_rasterize_fwd", "drp_rasterize_bwd", "drp_interpolate_fwd", "drp_interpolate_bwd",
                 "drp_antialias_fwd", "drp_antialias_bwd", "drp_antialias_topology"]:
        assert name in syms


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), "libdiffrp_gb300.so does not export %s" % name


def test_abi_version_and_status_strings(lib):
    assert lib.drp_abi_version() == 1
    assert lib.drp_status_string(0) == b"ok"
    assert lib.drp_status_string(1) == b"invalid argument"


def test_kernel_launch_counter_ignores_rejected_calls(lib):
    """Calls the host-side validation rejects launch nothing."""
    from diffrp_gb300 import _ffi
    before = _ffi.kernel_launches()
    with pytest.raises(RuntimeError):
        _ffi.call("drp_l1_loss_fwd", None, 0, None, None, 0, ctypes.c_float(1.0), None, None, None)
    assert _ffi.kernel_launches() == before


def test_workspace_queries_and_validation(lib):
    from diffrp_gb300 import _ffi
    n = _ffi.size_out("drp_raster_workspace_size", 2, 1000, 512, 512, 4, 10000)
    assert n >= 2 * 1000 * 48 + 40000
    assert _ffi.size_out("drp_antialias_workspace_size", 3, 100) >= 3 * 100 * 32
    assert _ffi.size_out("drp_topology_workspace_size", 100) > 0
    out = ctypes.c_size_t(0)
    assert lib.drp_raster_workspace_size(1, 10, 512, 512, 7, 0, ctypes.byref(out)) == 1
    assert b"tile_log2" in lib.drp_last_error()
    assert lib.drp_raster_workspace_size(1, 10, 0, 512, 4, 0, ctypes.byref(out)) == 1
    # invalid calls are rejected before any device work
    st = lib.drp_rasterize_fwd(None, 0, None, 0, 0, None, 0, 0, None, 0, 16, 16, 4, 0, 0, 0, None, None, None, None,
                               None)
    assert st == 1
    st = lib.drp_rasterize_fwd(None, 0, None, 0, 0, None, 0, 1, None, 0, 16, 16, 4, 3, 0, 0, None, None, None, None,
                               None)
    assert st == 1 and b"threads_per_tri" in lib.drp_last_error()
    with pytest.raises(RuntimeError, match="invalid argument"):
        _ffi.call("drp_interpolate_fwd", None, 0, 0, 0, None, None, None, 0, 1, 4, 4, None, 0, None, None, None)


def test_fast_path_matches_ctypes_on_validation(lib):
    """The CPython fast path (when built) wraps entry points the header
    declares and reports the same status and message as ctypes."""
    from diffrp_gb300 import _ffi
    table = _ffi._fast_table()
    if not table:
        pytest.skip("CPython fast path not built (no Python headers)")
    assert set(table) <= set(declared_symbols())
    bad = (None, 0, None, None, 0, 1.0, None, None, None)  # drp_l1_loss_fwd with nothing to do
    assert table["drp_l1_loss_fwd"](*bad) == lib.drp_l1_loss_fwd(*bad) == 1
    with pytest.raises(TypeError):
        table["drp_l1_loss_fwd"](*bad[:-1])


def test_transform_and_transport_validation(lib):
    """The clip-space transform and the host-transport entry points reject
    bad arguments on the host, launching nothing; the Python wrappers refuse
    CPU / unpinned tensors before calling the library."""
    import torch
    from diffrp_gb300 import _ffi, hostio, transform
    before = _ffi.kernel_launches()
    assert lib.drp_transform_points_fwd(None, 5, None, 1, None, None) == 1      # null matrices
    assert lib.drp_transform_points_fwd(None, 5, None, 0, None, None) == 1      # no views
    assert lib.drp_transform_points_bwd(None, -1, None, 1, None, None) == 1     # negative count
    assert lib.drp_transform_points_fwd(None, 0, None, 70000, None, None) == 1  # views above the grid limit
    assert lib.drp_copy_async(None, None, ctypes.c_size_t(16), None) == 1
    assert lib.drp_copy_async(None, None, ctypes.c_size_t(0), None) == 0        # nothing to copy
    dev = ctypes.c_void_p(1)
    assert lib.drp_host_device_pointer(None, ctypes.byref(dev)) == 1
    assert _ffi.kernel_launches() == before
    with pytest.raises(RuntimeError):
        transform.clip_space(torch.zeros(4, 3), torch.eye(4))
    with pytest.raises(RuntimeError):
        transform.clip_space_packed([])
    with pytest.raises(RuntimeError):
        hostio.device_view(torch.zeros(4))


def test_texture_levels_and_validation(lib):
    """The texture entry points' host-side rules: pyramid level counts and
    sizes (floor halving to 1 x 1, max_mip_level), and bad arguments
    rejected before any device work."""
    from diffrp_gb300 import _ffi
    n = ctypes.c_int(0)
    for (h, w, mx), want in [((1024, 1024, -1), 11), ((1024, 1024, 3), 4), ((5, 7, -1), 3), ((1, 1, -1), 1),
                             ((1, 9, -1), 4), ((32768, 1, -1), 16)]:
        assert lib.drp_texture_levels(h, w, mx, ctypes.byref(n)) == 0
        assert n.value == want, (h, w, mx)
    assert lib.drp_texture_levels(0, 4, -1, ctypes.byref(n)) == 1
    f = ctypes.c_longlong(0)
    assert lib.drp_texture_pyramid_floats(2, 16, 8, 3, 5, ctypes.byref(f)) == 0
    assert f.value == 2 * 3 * (8 * 4 + 4 * 2 + 2 * 1 + 1 * 1)  # levels 1 .. 4
    before = _ffi.kernel_launches()
    p = ctypes.c_void_p(256)  # never dereferenced: every call below fails validation
    # texture larger than 2^15 a side
    assert lib.drp_texture_mip_build(p, 1, 40000, 4, 4, 2, p, None) == 1
    # levels above the texture's pyramid
    assert lib.drp_texture_mip_build(p, 1, 8, 8, 4, 5, p, None) == 1
    # num_tex neither 1 nor num_views
    assert lib.drp_texture_fwd(p, p, 3, 8, 8, 4, 1, p, None, None, 2, 4, 4, 1, 0, p, None) == 1
    # filter and boundary codes out of range
    assert lib.drp_texture_fwd(p, p, 1, 8, 8, 4, 1, p, None, None, 1, 4, 4, 4, 0, p, None) == 1
    assert lib.drp_texture_fwd(p, p, 1, 8, 8, 4, 1, p, None, None, 1, 4, 4, 1, 4, p, None) == 1
    # uv not 8-byte aligned
    assert lib.drp_texture_fwd(p, p, 1, 8, 8, 4, 1, ctypes.c_void_p(260), None, None, 1, 4, 4, 1, 0, p, None) == 1
    # mip level bias not 4-byte aligned
    assert lib.drp_texture_fwd(p, p, 1, 8, 8, 4, 1, p, None, ctypes.c_void_p(258), 1, 4, 4, 3, 0, p, None) == 1
    # uv_da gradient without uv_da
    assert lib.drp_texture_bwd(p, p, 1, 8, 8, 4, 1, p, None, None, 1, 4, 4, 1, 0, p, p, p, p, p, None, None) == 1
    # mip level bias gradient without a bias
    assert lib.drp_texture_bwd(p, p, 1, 8, 8, 4, 1, p, None, None, 1, 4, 4, 3, 0, p, p, p, p, None, p, None) == 1
    assert _ffi.kernel_launches() == before
