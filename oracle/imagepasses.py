"""CPU restatement of the reference's image passes, for tests only.

tonemap(): ToneMappingPass::render (src/render/passes/tonemapping/
tonemapping.cu:60-88) with the operators of tonemapping.cu:11-44 and
luminance() of src/render/spectrum.h:545-547, in float32.
"""
import numpy as np

F = np.float32


def _lum(c):
    return c[..., 0] * F(0.299) + c[..., 1] * F(0.587) + c[..., 2] * F(0.114)


def tonemap(rgba: np.ndarray, op: int, exposure: float, gamma: bool) -> np.ndarray:
    c = rgba[..., :3].astype(np.float32) * F(exposure)
    with np.errstate(divide="ignore", invalid="ignore"):
        if op == 1:
            lum = _lum(c)[..., None]
            r = lum / (lum + F(1))
            c = np.where(lum == 0, F(0), (c * r) / lum)
        elif op == 2:
            c = c * F(0.6)
            c = np.clip((c * (F(2.51) * c + F(0.03))) / (c * (F(2.43) * c + F(0.59)) + F(0.14)), 0, 1)
        elif op == 3:
            A, B, C, D, E, G = F(0.22), F(0.3), F(0.1), F(0.2), F(0.01), F(0.3)
            c = ((c * (A * c + C * B) + D * E) / (c * (A * c + B) + D * G)) - (E / G)
        elif op == 4:
            c = np.maximum(c - F(0.004), F(0))
            c = (c * (F(6.2) * c + F(0.5))) / (c * (F(6.2) * c + F(1.7)) + F(0.06))
            c = np.power(c, F(2.2))
        if gamma:
            c = np.power(c, F(0.45454545))
    out = np.ones(rgba.shape, np.float32)
    out[..., :3] = c
    return out
