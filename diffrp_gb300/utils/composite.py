"""Layer blending functions used by compose_layers
(diffrp/utils/composite.py:28-37)."""
import torch

from .shader_ops import fma, saturate

__all__ = ["alpha_blend", "additive", "alpha_additive"]


def alpha_blend(bgc, bga, fgc, fga):
    """Front-over-back: colour lerp by the front alpha, alpha = fga + bga (1 - fga)."""
    return torch.lerp(bgc, fgc, fga), fma(bga, 1 - fga, fga)


def additive(bgc, bga, fgc, fga):
    return bgc + fgc, saturate(bga + fga)


def alpha_additive(bgc, bga, fgc, fga):
    return bgc + fgc * fga, saturate(bga + fga)
