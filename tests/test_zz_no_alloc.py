"""drp_antialias_fwd_noalloc against drp_antialias_fwd, through the C ABI.

The no-allocation entry point exists for callers that cannot allocate device
memory (for example a host that owns the GPU's memory budget and hands the
library only its inputs and outputs).  It keeps its per-triangle scratch in
a fixed array inside the library instead of a caller workspace, so its
output must equal the workspace version's -- bit for bit, the tolerance of
every antialias forward test -- on consecutive calls that reuse the shared
array with different geometry.  Collected last on purpose (test_zz_*).
"""
import ctypes

import numpy as np
import pytest
import torch

from tests import scenes

pytestmark = pytest.mark.gpu


def _inputs(scene, res=(80, 96), channels=5, topology=True):
    """scene: (clip pos (V, 4) or (B, V, 4), tri).  topology=False passes a
    null topology (every edge a silhouette)."""
    from diffrp_gb300 import nvdr
    pos_np, tri_np = scene
    pos = torch.from_numpy(np.ascontiguousarray(pos_np)).cuda()
    tri = torch.from_numpy(tri_np).cuda()
    H, W = res
    B = pos.shape[0] if pos.dim() == 3 else 1
    rast, _ = nvdr.rasterize(nvdr.RasterizeCudaContext(), pos, tri, (H, W), grad_db=False)
    rng = np.random.default_rng(len(tri_np) + B)
    color = torch.from_numpy(rng.uniform(0, 1, (B, H, W, channels)).astype(np.float32)).cuda()
    nbr = nvdr.antialias_construct_topology_hash(tri) if topology else None
    return pos, tri, rast, color, nbr, H, W


def _run(lib, noalloc, pos, tri, rast, color, nbr, H, W):
    from diffrp_gb300 import _ffi
    out = torch.empty_like(color)
    stream = torch.cuda.current_stream().cuda_stream
    B = color.shape[0]
    V = pos.shape[-2]
    stride = V * 4 if pos.dim() == 3 else 0  # floats between views' positions
    nbr_ptr = None if nbr is None else nbr.data_ptr()
    common = (color.data_ptr(), color.shape[-1], rast.data_ptr(), pos.data_ptr(), stride, V, tri.data_ptr(),
              tri.shape[0], nbr_ptr, B, H, W, out.data_ptr(), stream)
    if noalloc:
        status = lib.drp_antialias_fwd_noalloc(*common)
        assert status == 0, lib.drp_last_error()
    else:
        ws = torch.empty(_ffi.size_out("drp_antialias_workspace_size", B, tri.shape[0]), dtype=torch.uint8,
                         device="cuda")
        status = lib.drp_antialias_fwd(ws.data_ptr(), ws.numel(), *common[:-1], None, stream)
        assert status == 0, lib.drp_last_error()
    torch.cuda.synchronize()
    return out


def test_noalloc_antialias_matches_workspace_version(cuda_lib):
    lib = cuda_lib
    first = _inputs(scenes.sphere_view(3, res=(80, 96), sigma=0.03, seed=4))
    second = _inputs(scenes.random_soup(150, seed=9))  # different triangles reuse the shared scratch
    for inputs in (first, second):
        got = _run(lib, True, *inputs)
        ref = _run(lib, False, *inputs)
        assert torch.equal(got, ref)
        assert bool((got != inputs[3]).any())  # silhouettes were blended


def test_noalloc_antialias_views_and_null_topology(cuda_lib):
    """Several views with per-view positions (pos_view_stride > 0), then the
    same views with no topology (every edge a silhouette)."""
    lib = cuda_lib
    views = scenes.multi_view(subdiv=2, n_views=4, res=(48, 56), seed=5)
    for topology in (True, False):
        inputs = _inputs(views, res=(48, 56), channels=3, topology=topology)
        got = _run(lib, True, *inputs)
        ref = _run(lib, False, *inputs)
        assert torch.equal(got, ref)
        for b in range(inputs[3].shape[0]):
            assert bool((got[b] != inputs[3][b]).any())  # every view was blended


def test_noalloc_rejects_sizes_above_its_scratch(cuda_lib):
    lib = cuda_lib
    f = ctypes.c_void_p(16)  # never dereferenced: the size check fails first
    status = lib.drp_antialias_fwd_noalloc(f, 3, f, f, 0, 10, f, 262145, None, 1, 8, 8, f, None)
    assert status == 1
    assert b"DRP_NOALLOC_AA_MAX_TRIANGLE_VIEWS" in lib.drp_last_error()
    # more views than a launch grid holds, even with no triangles
    status = lib.drp_antialias_fwd_noalloc(f, 3, f, f, 0, 10, f, 0, None, 65536, 8, 8, f, None)
    assert status == 1
    assert b"65535" in lib.drp_last_error()
    # more pixels than 32-bit pixel indices reach
    status = lib.drp_antialias_fwd_noalloc(f, 3, f, f, 0, 10, f, 1, None, 600, 2048, 2048, f, None)
    assert status == 1
    assert b"2^31" in lib.drp_last_error()
