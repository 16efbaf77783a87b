"""An imported configuration (OBJ/MTL room, conductor override, glass,
emissive quad, infinite light, homogeneous medium box) rendered on the GPU
against the CPU restatement, then accumulated and tone-mapped as the
configuration's passes ask."""
from pathlib import Path

import numpy as np
import pytest
import torch

from kiraray_gb300 import importer as I
from kiraray_gb300.convergence import Accumulator, tonemap
from kiraray_gb300.wavefront import WavefrontPathTracer
from oracle import pyoracle as O
from tests.test_wavefront_gpu import compare

pytestmark = pytest.mark.gpu
FIX = Path(__file__).parent / "golden" / "scene_config"


def test_imported_scene_matches_oracle_and_passes(krr_lib, cuda, tmp_path):
    cfg = I.load_config(FIX / "room.json")
    sc = cfg["scene"]
    w, h = cfg["resolution"]
    pt = WavefrontPathTracer(cfg["wavefront"])
    pt.set_scene(sc)
    pt.resize(w, h)
    pt.begin_frame(1, sc.camera)
    pt.render()
    L = pt.radiance().cpu().numpy()
    oL, _ = O.PathTracer(sc).render(cfg["wavefront"], 1)
    compare(L[:, :3], oL, "imported room")
    assert pt.device_errors() == 0
    # AccumulatePass spp frames, then the ToneMappingPass of the configuration
    acc = Accumulator(w, h)
    out = torch.empty((h, w, 4), device="cuda")
    for f in range(1, cfg["accumulate_spp"] + 1):
        pt.begin_frame(f, sc.camera)
        pt.render(out)
        acc.add(out)
    img = tonemap(acc.image(), **cfg["tonemap"]).reshape(h, w, 4).cpu().numpy()
    assert np.isfinite(img).all() and img[..., :3].max() <= 1.0 and img[..., :3].mean() > 0.01
    I.write_pfm(tmp_path / "room.pfm", img)
    assert np.array_equal(I.read_pfm(tmp_path / "room.pfm"), img[..., :3])
