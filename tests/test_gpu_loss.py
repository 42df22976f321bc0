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
