"""Host-side planning of the batching form (drp_batch_plan,
drp_batch_block_maps, the workspace / state size queries): item offsets,
totals and block maps for uneven items, and argument validation -- no GPU."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def batch():
    from diffrp_gb300 import build
    build.build()
    from diffrp_gb300 import batch as B
    B._register()
    return B


def _items(B, specs):
    arr = (B._Item * len(specs))()
    for i, (po, ao, tf, tc, V, H, W, C) in enumerate(specs):
        arr[i].pos_offset, arr[i].attr_offset, arr[i].tri_first, arr[i].tri_count = po, ao, tf, tc
        arr[i].num_vertices, arr[i].height, arr[i].width, arr[i].channels = V, H, W, C
    return arr


SPECS = [  # pos row, attr float, first triangle, triangles, vertices, H, W, C
    (0, 0, 0, 7, 10, 100, 37, 5),
    (10, 50, 7, 600, 20, 64, 64, 8),
    (30, 210, 607, 0, 5, 1, 1, 4),
    (10, 50, 7, 600, 20, 17, 300, 8),  # the second mesh again, another view
]


@pytest.mark.parametrize("tl", [3, 4, 5])
def test_plan_offsets_and_totals(batch, tl):
    from diffrp_gb300 import _ffi
    arr = _items(batch, SPECS)
    totals = (ctypes.c_longlong * 6)()
    _ffi.call("drp_batch_plan", ctypes.addressof(arr), len(SPECS), tl, ctypes.addressof(totals))
    T = 1 << tl
    prims = tiles = pixels = floats = pb = xb = 0
    for it, (_, _, _, tc, _, H, W, C) in zip(arr, SPECS):
        assert (it.tiles_x, it.tiles_y) == (-(-W // T), -(-H // T))
        assert (it.prim_offset, it.tile_offset, it.pixel_offset, it.image_offset) == (prims, tiles, pixels, floats)
        prims += tc
        tiles += it.tiles_x * it.tiles_y
        pixels += H * W
        floats += H * W * C
        pb += -(-tc // 256)
        xb += -(-(H * W) // 256)
    assert list(totals) == [prims, tiles, pixels, floats, pb, xb]

    pmap = (ctypes.c_int * max(2, 2 * pb))()
    xmap = (ctypes.c_int * max(2, 2 * xb))()
    _ffi.call("drp_batch_block_maps", ctypes.addressof(arr), len(SPECS), ctypes.addressof(pmap),
              ctypes.addressof(xmap))
    want_p = [(i, k) for i, s in enumerate(SPECS) for k in range(-(-s[3] // 256))]
    want_x = [(i, k) for i, s in enumerate(SPECS) for k in range(-(-(s[5] * s[6]) // 256))]
    assert [(pmap[2 * j], pmap[2 * j + 1]) for j in range(pb)] == want_p
    assert [(xmap[2 * j], xmap[2 * j + 1]) for j in range(xb)] == want_x


def test_plan_rejects_bad_items(batch):
    lib = batch._ffi.load()
    totals = (ctypes.c_longlong * 6)()
    for bad in [(0, 0, 0, 1, 3, 0, 8, 1),          # zero height
                (0, 0, 0, 1, 3, 8, 20000, 1),      # above the largest resolution
                (0, 0, 0, 1, 3, 8, 8, 0),          # no channels
                (0, 0, -1, 1, 3, 8, 8, 1),         # negative first triangle
                (-4, 0, 0, 1, 3, 8, 8, 1)]:        # negative position offset
        arr = _items(batch, [bad])
        assert lib.drp_batch_plan(ctypes.addressof(arr), 1, 4, ctypes.addressof(totals)) == 1
    arr = _items(batch, SPECS[:1])
    assert lib.drp_batch_plan(ctypes.addressof(arr), 1, 6, ctypes.addressof(totals)) == 1  # tile size
    assert lib.drp_batch_plan(ctypes.addressof(arr), 0, 4, ctypes.addressof(totals)) == 1  # no items
    assert lib.drp_batch_block_maps(ctypes.addressof(arr), 1, None, None) == 1


def test_workspace_and_state_sizes_grow_with_the_work(batch):
    from diffrp_gb300 import _ffi
    a = _ffi.size_out("drp_batch_workspace_size", 1000, 64, 0)
    b = _ffi.size_out("drp_batch_workspace_size", 2000, 64, 0)
    c = _ffi.size_out("drp_batch_workspace_size", 1000, 64, 1 << 20)
    assert a % 256 == 0 and b > a and c >= a + 4 * (1 << 20)
    s1 = _ffi.size_out("drp_batch_aa_state_size", 1 << 16)
    s2 = _ffi.size_out("drp_batch_aa_state_size", 1 << 17)
    assert s1 >= 5 * (1 << 16) and s2 > s1  # a flag byte and a list entry per pixel
