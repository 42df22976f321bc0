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


def _inputs(scene):
    from diffrp_gb300 import nvdr
    pos_np, tri_np = scene
    pos = torch.from_numpy(pos_np).cuda()
    tri = torch.from_numpy(tri_np).cuda()
    H, W = 80, 96
    rast, _ = nvdr.rasterize(nvdr.RasterizeCudaContext(), pos, tri, (H, W), grad_db=False)
    rng = np.random.default_rng(len(tri_np))
    color = torch.from_numpy(rng.uniform(0, 1, (1, H, W, 5)).astype(np.float32)).cuda()
    nbr = nvdr.antialias_construct_topology_hash(tri)
    return pos, tri, rast, color, nbr, H, W


def _run(lib, noalloc, pos, tri, rast, color, nbr, H, W):
    from diffrp_gb300 import _ffi
    out = torch.empty_like(color)
    stream = torch.cuda.current_stream().cuda_stream
    common = (color.data_ptr(), color.shape[-1], rast.data_ptr(), pos.data_ptr(), 0, pos.shape[0], tri.data_ptr(),
              tri.shape[0], nbr.data_ptr(), 1, H, W, out.data_ptr(), stream)
    if noalloc:
        status = lib.drp_antialias_fwd_noalloc(*common)
        assert status == 0, lib.drp_last_error()
    else:
        ws = torch.empty(_ffi.size_out("drp_antialias_workspace_size", 1, tri.shape[0]), dtype=torch.uint8,
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


def test_noalloc_rejects_sizes_above_its_scratch(cuda_lib):
    lib = cuda_lib
    f = ctypes.c_void_p(16)  # never dereferenced: the size check fails first
    status = lib.drp_antialias_fwd_noalloc(f, 3, f, f, 0, 10, f, 262145, None, 1, 8, 8, f, None)
    assert status == 1
    assert b"DRP_NOALLOC_AA_MAX_TRIANGLE_VIEWS" in lib.drp_last_error()
