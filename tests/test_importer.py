"""Scene-configuration importer (subset of the reference's JSON layout),
OBJ/MTL mapping and PFM files; CPU only."""
import math
from pathlib import Path

import numpy as np
import pytest

from kiraray_gb300 import _lib as L
from kiraray_gb300 import importer as I

FIX = Path(__file__).parent / "golden" / "scene_config"


def test_config_passes_and_resolution():
    cfg = I.load_config(FIX / "room.json")
    assert cfg["resolution"] == (64, 48)
    assert cfg["wavefront"] == {"nee": True, "rr": 0.8, "max_depth": 6}
    assert cfg["tonemap"] == {"operator": "aces", "exposure": 0.75, "gamma": True}
    assert cfg["accumulate_spp"] == 16
    assert cfg["scene"].max_depth == 6


def test_obj_groups_materials_and_emission():
    sc = I.load_config(FIX / "room.json")["scene"]
    names = [m.name for m in sc.meshes]
    assert names == ["white", "red", "light", "glass", ""]   # the medium box last
    tri_counts = [m.indices.shape[0] for m in sc.meshes]
    assert tri_counts[:4] == [4, 2, 2, 3]                   # quads -> 2, pentagon -> 3
    white, red, light, glass = (sc.materials[sc.meshes[k].material] for k in range(4))
    assert white.type == L.MATERIAL_DIFFUSE and white.diffuse == (0.7, 0.7, 0.68)
    assert math.isclose(white.roughness, math.sqrt(2.0 / 12.0))
    # the materials block overrides "red": conductor, roughness 0.3
    assert red.type == L.MATERIAL_CONDUCTOR and red.roughness == 0.3 and red.diffuse == (0.9, 0.2, 0.1)
    assert glass.type == L.MATERIAL_DIELECTRIC and glass.specular_transmission == 1.0 and glass.eta == 1.45
    assert sc.meshes[2].emission == (12.0, 10.0, 6.0)
    # explicit vertex normals where the file gives them, face normals otherwise
    assert np.allclose(sc.meshes[0].normals[:6], [0, 1, 0])
    assert np.allclose(sc.meshes[2].normals, [0, -1, 0])
    n_red = np.cross(sc.meshes[1].positions[1] - sc.meshes[1].positions[0],
                     sc.meshes[1].positions[2] - sc.meshes[1].positions[0])
    assert np.allclose(sc.meshes[1].normals[0], n_red / np.linalg.norm(n_red))


def test_node_transform_light_and_medium():
    sc = I.load_config(FIX / "room.json")["scene"]
    mesh, xf = sc.instances[0]
    assert np.allclose(xf, [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0.2]])
    assert len(sc.infinite_lights) == 1
    sky = sc.infinite_lights[0]
    assert sky.tint == (0.2, 0.3, 0.5) and sky.scale == 0.5 and sky.image is None
    med = sc.media[0]
    assert np.allclose(med.sigma_t, (0.25, 0.3, 0.35))
    assert np.allclose(med.albedo, (0.2 / 0.25, 0.25 / 0.3, 0.3 / 0.35))
    box = sc.meshes[-1]
    assert box.material == -1 and box.medium_inside == 0 and box.medium_outside == -1
    assert np.allclose(box.positions.min(0), (-0.5, 0.2, -0.5))
    assert np.allclose(box.positions.max(0), (0.5, 0.9, 0.5))


def test_orbit_camera_pose():
    sc = I.load_config(FIX / "room.json")["scene"]
    cam = sc.camera
    yaw, pitch, r = 0.25, -0.1, 3.5
    # forward of Ry(yaw) Rx(pitch) applied to -z, written out
    fwd = np.array([-math.sin(yaw) * math.cos(pitch), math.sin(pitch), -math.cos(yaw) * math.cos(pitch)])
    assert np.allclose(np.asarray(cam.position), np.array([0, 1, 0]) - fwd * r, atol=1e-6)
    R = np.asarray(cam.rotation)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-6) and np.isclose(np.linalg.det(R), 1.0)
    assert np.allclose(R @ [0, 0, -1], fwd, atol=1e-6)
    assert math.isclose(cam.aspect_ratio, 1.3333333, rel_tol=1e-6)
    assert math.isclose(cam.film_size[1], 24.0) and cam.focal_length == 21.0
    assert cam.medium == -1   # the camera is outside the medium box


def test_quaternion_rotation():
    q = [math.cos(0.3), 0.0, math.sin(0.3), 0.0]   # 0.6 rad about +y
    R = I.quat_matrix(q)
    assert np.allclose(R @ [1, 0, 0], [math.cos(0.6), 0, -math.sin(0.6)])


def test_pfm_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.random((5, 7, 3)).astype(np.float32) * 10
    I.write_pfm(tmp_path / "a.pfm", img)
    back = I.read_pfm(tmp_path / "a.pfm")
    assert back.shape == (5, 7, 3) and np.array_equal(back, img)
    raw = (tmp_path / "a.pfm").read_bytes()
    assert raw.startswith(b"PF\n7 5\n-1.0\n") and len(raw) == len(b"PF\n7 5\n-1.0\n") + 5 * 7 * 12


def test_unsupported_items_raise():
    base = {"scene": {"model": [{"type": "light", "params": {"type": "point"}}]}}
    with pytest.raises(I.ImportError_):
        I.load_config(base)
    with pytest.raises(I.ImportError_):
        I.load_config({"scene": {"camera": {"mData": {"lensRadius": 0.5}}}})
    with pytest.raises(I.ImportError_):
        I.load_config({"scene": {"media": [{"params": {"type": "heterogeneous", "file": "x.vdb"}}]}})
