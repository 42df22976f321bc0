"""Fused L1 loss against PyTorch's (pred - target).abs().mean()."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 1000, 2048 * 7 + 3, 1 << 20])
def test_l1_loss_matches_torch(cuda_lib, n):
    from diffrp_gb300.losses import l1_loss
    g = torch.Generator(device="cuda").manual_seed(n)
    pred = torch.rand(n, device="cuda", generator=g).requires_grad_(True)
    target = torch.rand(n, device="cuda", generator=g)
    target[: n // 10] = pred.detach()[: n // 10]  # exact ties have zero gradient
    ref_pred = pred.detach().clone().requires_grad_(True)
    ref = (ref_pred - target).abs().mean()
    ref.backward()
    loss = l1_loss(pred, target)
    loss.backward()
    assert torch.allclose(loss, ref, rtol=1e-6, atol=0)
    assert torch.allclose(pred.grad, ref_pred.grad, rtol=1e-6, atol=0)


@pytest.mark.parametrize("offset", [0, 1, 3])
def test_l1_loss_unaligned_and_large(cuda_lib, offset):
    """Views that start off a 16-byte boundary take the scalar path; a large
    input runs the grid-stride loop many times per thread."""
    from diffrp_gb300.losses import l1_loss
    n = (1 << 22) + 5
    g = torch.Generator(device="cuda").manual_seed(7)
    base_p = torch.rand(n + offset, device="cuda", generator=g)
    base_t = torch.rand(n + offset, device="cuda", generator=g)
    pred = base_p[offset:].requires_grad_(True)
    target = base_t[offset:]
    ref = (pred.detach() - target).abs().mean()
    loss = l1_loss(pred, target)
    loss.backward()
    assert torch.allclose(loss, ref, rtol=2e-6, atol=0)
    d = pred.detach() - target
    expect = torch.sign(d) / n
    assert torch.equal(pred.grad, expect)
