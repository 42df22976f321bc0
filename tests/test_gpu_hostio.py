"""Host transport by kernels (drp_host_device_pointer, drp_copy_async):
bit-exact copies between pinned host buffers (through their mapped device
addresses) and device memory, aligned and unaligned, eager and captured in a
CUDA graph."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _payload(n, seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    bits[:4] = [0x80000000, 0x7fc00001, 0xff800000, 0x00000001]  # -0, NaN payload, -inf, denormal
    return torch.from_numpy(bits.view(np.float32).copy())


@pytest.mark.parametrize("n", [1, 3, 4, 1000, 112651, 1 << 20])
def test_roundtrip_bit_exact(cuda_lib, n):
    from diffrp_gb300 import hostio
    h_in = _payload(max(n, 4), n)[:n].clone().pin_memory()
    h_out = torch.zeros_like(h_in).pin_memory()
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    hostio.copy_(d, hostio.device_view(h_in))
    hostio.copy_(hostio.device_view(h_out), d)
    torch.cuda.synchronize()
    assert torch.equal(h_out.view(torch.int32), h_in.view(torch.int32))
    assert torch.equal(d.cpu().view(torch.int32), h_in.view(torch.int32))


def test_unaligned_and_bytes(cuda_lib):
    from diffrp_gb300 import hostio
    h = torch.arange(4099, dtype=torch.uint8).pin_memory()
    v = hostio.device_view(h)
    d = torch.zeros(4099, dtype=torch.uint8, device="cuda")
    hostio.copy_(d[3:], v[1:4097])  # neither end 16-byte aligned: byte loop
    torch.cuda.synchronize()
    assert torch.equal(d[3:].cpu(), h[1:4097]) and int(d[:3].abs().sum()) == 0


def test_graph_captured_transfer(cuda_lib):
    from diffrp_gb300 import hostio
    h_in = torch.zeros(5000, dtype=torch.float32).pin_memory()
    h_out = torch.zeros(5000, dtype=torch.float32).pin_memory()
    vin, vout = hostio.device_view(h_in), hostio.device_view(h_out)
    d = torch.empty(5000, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        hostio.copy_(d, vin)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        hostio.copy_(d, vin)
        torch.mul(d, 2.0, out=vout)
    for k in range(3):
        h_in.copy_(torch.arange(5000, dtype=torch.float32) + k)
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(h_out, 2.0 * (torch.arange(5000, dtype=torch.float32) + k))


def test_rejects_misuse(cuda_lib):
    from diffrp_gb300 import hostio
    with pytest.raises(RuntimeError):
        hostio.device_view(torch.zeros(8))  # pageable
    with pytest.raises(RuntimeError):
        hostio.device_view(torch.zeros(8, device="cuda"))
    with pytest.raises(RuntimeError):
        hostio.copy_(torch.zeros(8, device="cuda"), torch.zeros(9, device="cuda"))
