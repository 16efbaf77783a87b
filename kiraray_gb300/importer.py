"""Scene-configuration importer (a subset) and PFM image files.

`load_config(path_or_dict)` reads the reference's JSON configuration
(`common/configs/*.json`; parsing as in src/scene/krrscene.cpp:195-330):

- ``resolution`` [w, h];
- ``passes``: ``WavefrontPathTracer`` params (nee, rr, max_depth,
  enable_medium, enable_clamp, clamp_max), ``ToneMappingPass`` params
  (operator, exposure, gamma), ``AccumulatePass`` params (spp);
- ``scene.camera.mData`` (focalLength, focalDistance, lensRadius,
  aspectRatio, shutterOpen, shutterTime; src/core/camera.h:20-79) and
  ``scene.cameraController.mData`` (target, radius, pitch, yaw): the orbit
  pose rotate = Ry(yaw) Rz(0) Rx(pitch), position = target - forward *
  radius (src/core/camera.cpp:48-61, krrmath/quaternion.h:31-35);
- ``scene.model``: nested nodes with ``translate``, ``rotate`` (quaternion
  [w, x, y, z]), ``scale`` (local = T R S, src/core/scenenode.cpp:42-44),
  holding ``.obj`` models or ``"type": "light"`` nodes with an infinite
  light (``color``, ``scale``, optional ``texture``);
- ``scene.environment``: an environment image file;
- ``scene.media``: homogeneous media with ``bound`` (a null-material box
  whose inside is the medium) or attached to named meshes (``meshes``,
  ``meshes_outside``), ``sigma_t``/``albedo`` or ``sigma_a``/``sigma_s``, ``g``;
- ``scene.materials``: per-name overrides (``bsdf`` diffuse / dielectric /
  conductor, ``params`` diffuse, specular, roughness,
  specular_transmission, eta, anisotropic; krrscene.cpp:195-246).

OBJ/MTL follow the reference's Assimp mapping (src/scene/assimp.cpp:60-180):
Kd diffuse, Ks specular, Ns -> roughness sqrt(2 / (Ns + 2)) (specular when
Ns >= 1000), Ni eta, d = 0 or a transmission filter -> dielectric, Ke
emission.  The reference's default material type is Disney, which this
library does not implement: such materials are imported as Lambertian
with the same diffuse colour unless a ``materials`` entry names a BSDF.

Images: `.pfm` (read and written here).  Not supported (a clear error):
point, directional and spot lights, heterogeneous (.vdb) media, model
formats other than .obj, thin-lens cameras, spectral IoR tables.
"""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

import numpy as np

from . import _lib as L
from .scenes import Camera, InfiniteLight, Material, Medium, Mesh, Scene, _unit_cube

PASS_PARAMS = ("nee", "rr", "max_depth", "enable_medium", "enable_clamp", "clamp_max")
BSDF_NAMES = {"diffuse": L.MATERIAL_DIFFUSE, "dielectric": L.MATERIAL_DIELECTRIC,
              "conductor": L.MATERIAL_CONDUCTOR}


class ImportError_(ValueError):
    """A configuration item this importer does not support."""


# ------------------------------------------------------------------ PFM files
def write_pfm(path, rgb: np.ndarray) -> None:
    """Writes float32 RGB [H, W, 3] (row 0 at the top) as a little-endian PFM."""
    img = np.asarray(rgb, np.float32)
    if img.ndim != 3 or img.shape[2] not in (3, 4):
        raise ValueError("expected [H, W, 3 or 4]")
    img = img[..., :3]
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(img[::-1]).astype("<f4").tobytes())   # PFM rows bottom-up


def read_pfm(path) -> np.ndarray:
    """float32 [H, W, 3] (row 0 at the top) from a PFM file (RGB or grey)."""
    with open(path, "rb") as f:
        kind = f.readline().strip()
        if kind not in (b"PF", b"Pf"):
            raise ValueError(f"{path}: not a PFM file")
        dims = f.readline().split()
        while len(dims) < 2:
            dims += f.readline().split()
        w, h = int(dims[0]), int(dims[1])
        scale = float(f.readline().strip())
        ch = 3 if kind == b"PF" else 1
        data = np.frombuffer(f.read(w * h * ch * 4), dtype="<f4" if scale < 0 else ">f4")
    img = data.reshape(h, w, ch)[::-1].astype(np.float32)
    if ch == 1:
        img = np.repeat(img, 3, axis=2)
    return np.ascontiguousarray(img)


def _load_image(path: Path) -> np.ndarray:
    if path.suffix.lower() != ".pfm":
        raise ImportError_(f"{path.name}: only .pfm images are read (convert EXR/HDR to PFM)")
    rgb = read_pfm(path)
    out = np.ones(rgb.shape[:2] + (4,), np.float32)
    out[..., :3] = rgb
    return out


# --------------------------------------------------------------- transforms
def quat_matrix(q) -> np.ndarray:
    """Rotation matrix of the unit quaternion [w, x, y, z]."""
    w, x, y, z = (float(v) for v in q)
    n = math.sqrt(w * w + x * x + y * y + z * z) or 1.0
    w, x, y, z = w / n, x / n, y / n, z / n
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _axis_angle(axis, angle) -> np.ndarray:
    x, y, z = axis
    c, s = math.cos(angle), math.sin(angle)
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def orbit_pose(target, radius: float, pitch: float, yaw: float):
    """Camera position and camera-to-world rotation of the orbit controller."""
    R = _axis_angle((0, 1, 0), yaw) @ _axis_angle((0, 0, 1), 0.0) @ _axis_angle((1, 0, 0), pitch)
    forward = R @ np.array([0.0, 0.0, -1.0])
    pos = np.asarray(target, np.float64) - forward * radius
    return pos, R


def _node_matrix(node: dict) -> np.ndarray:
    S = np.diag(list(np.asarray(node.get("scale", [1, 1, 1]), np.float64)) + [1.0])
    R = np.eye(4)
    if "rotate" in node:
        R[:3, :3] = quat_matrix(node["rotate"])
    T = np.eye(4)
    T[:3, 3] = np.asarray(node.get("translate", [0, 0, 0]), np.float64)
    return T @ R @ S


# ------------------------------------------------------------------ OBJ/MTL
def _spec_power_to_roughness(ns: float) -> float:
    if ns >= 1000:
        return 0.0
    return min(max(math.sqrt(2.0 / (ns + 2.0)), 0.0), 1.0)


def _read_mtl(path: Path) -> dict:
    mats, cur = {}, None
    for raw in path.read_text().splitlines():
        t = raw.split("#", 1)[0].split()
        if not t:
            continue
        key, vals = t[0], t[1:]
        if key == "newmtl":
            cur = mats.setdefault(" ".join(vals), {})
        elif cur is not None:
            cur[key] = [float(v) for v in vals if _is_number(v)]
    return mats


def _is_number(s: str) -> bool:
    try:
        float(s)
        return True
    except ValueError:
        return False


def _mtl_material(m: dict) -> tuple:
    """(Material, emission) from MTL keys, as the reference's Assimp import."""
    mat = Material()
    if "Kd" in m:
        mat.diffuse = tuple(m["Kd"][:3])
    if "Ks" in m:
        mat.specular = tuple(m["Ks"][:3])
    if "Ns" in m:
        mat.roughness = _spec_power_to_roughness(m["Ns"][0])
    if "Ni" in m:
        mat.eta = m["Ni"][0]
    if "d" in m and m["d"] and m["d"][0] == 0.0:
        mat.specular_transmission = 1.0
        mat.type = L.MATERIAL_DIELECTRIC
    if "Tf" in m and len(m["Tf"]) >= 3:
        t = [1.0 - v for v in m["Tf"][:3]]
        lum = 0.299 * t[0] + 0.587 * t[1] + 0.114 * t[2]
        mat.specular_transmission = lum
        if lum > 1 - 1e-6:
            mat.type = L.MATERIAL_DIELECTRIC
    emission = tuple(m["Ke"][:3]) if "Ke" in m else (0.0, 0.0, 0.0)
    return mat, emission


def load_obj(path) -> list:
    """Meshes of an OBJ file, one per material group: dicts with positions,
    normals (vertex normals when given, else the face normal), indices and
    the MTL material name."""
    path = Path(path)
    vs, vns = [], []
    groups: dict = {}
    mtl_lib: dict = {}
    cur = ""
    for raw in path.read_text().splitlines():
        t = raw.split("#", 1)[0].split()
        if not t:
            continue
        key = t[0]
        if key == "v":
            vs.append([float(x) for x in t[1:4]])
        elif key == "vn":
            vns.append([float(x) for x in t[1:4]])
        elif key == "mtllib":
            p = path.parent / " ".join(t[1:])
            if p.exists():
                mtl_lib.update(_read_mtl(p))
        elif key == "usemtl":
            cur = " ".join(t[1:])
        elif key == "f":
            corners = []
            for c in t[1:]:
                parts = c.split("/")
                vi = int(parts[0])
                ni = int(parts[2]) if len(parts) > 2 and parts[2] else 0
                vi = vi - 1 if vi > 0 else len(vs) + vi
                ni = (ni - 1 if ni > 0 else len(vns) + ni) if ni else -1
                corners.append((vi, ni))
            for k in range(1, len(corners) - 1):   # fan triangulation
                groups.setdefault(cur, []).append((corners[0], corners[k], corners[k + 1]))
    V = np.asarray(vs, np.float64).reshape(-1, 3)
    N = np.asarray(vns, np.float64).reshape(-1, 3)
    out = []
    for name, tris in groups.items():
        pos, nrm = [], []
        for tri in tris:
            p = [V[c[0]] for c in tri]
            fn = np.cross(p[1] - p[0], p[2] - p[0])
            ln = np.linalg.norm(fn)
            fn = fn / ln if ln > 0 else np.array([0.0, 1.0, 0.0])
            for (vi, ni), pv in zip(tri, p):
                pos.append(pv)
                nrm.append(N[ni] / (np.linalg.norm(N[ni]) or 1.0) if ni >= 0 else fn)
        pos = np.asarray(pos, np.float32)
        out.append({"name": name, "positions": pos, "normals": np.asarray(nrm, np.float32),
                    "indices": np.arange(len(pos), dtype=np.uint32).reshape(-1, 3),
                    "mtl": mtl_lib.get(name, {})})
    return out


# ------------------------------------------------------------------- config
def _resolve(base: Path, rel: str) -> Path:
    p = Path(rel)
    if p.is_absolute():
        return p
    for root in (base, *base.parents):
        if (root / p).exists():
            return root / p
    return base / p


def load_config(config, base_dir=None) -> dict:
    """Scene and pass parameters of a configuration (file path or dict).
    Returns {"scene": Scene, "resolution": (w, h), "wavefront": dict,
    "tonemap": dict or None, "accumulate_spp": int}."""
    if isinstance(config, (str, os.PathLike)):
        base = Path(config).resolve().parent if base_dir is None else Path(base_dir)
        cfg = json.loads(Path(config).read_text())
    else:
        base = Path(base_dir or ".").resolve()
        cfg = config
    w, h = (int(x) for x in cfg.get("resolution", [1280, 720]))
    wavefront, tonemap, acc_spp = {}, None, 0
    for p in cfg.get("passes", []):
        if not p.get("enable", True):
            continue
        prm = p.get("params", {})
        if p.get("name") == "WavefrontPathTracer":
            wavefront = {k: prm[k] for k in PASS_PARAMS if k in prm}
        elif p.get("name") == "ToneMappingPass":
            tonemap = {"operator": str(prm.get("operator", "linear")).lower(),
                       "exposure": float(prm.get("exposure", 1.0)),
                       "gamma": bool(prm.get("gamma", True))}
        elif p.get("name") == "AccumulatePass":
            acc_spp = int(prm.get("spp", 0))
    scene = _import_scene(cfg.get("scene", cfg), base, w, h)
    if "max_depth" in wavefront:
        scene.max_depth = int(wavefront["max_depth"])
    return {"scene": scene, "resolution": (w, h), "wavefront": wavefront, "tonemap": tonemap,
            "accumulate_spp": acc_spp}


def _import_scene(j: dict, base: Path, w: int, h: int) -> Scene:
    meshes, instances, mats, lights, media = [], [], [], [], []
    boxes: list = []   # (medium index, lo, hi) of media with a bounding box
    mat_index: dict = {}
    mesh_names: list = []

    def material_for(name: str, mtl: dict) -> int:
        if name not in mat_index:
            mat, _ = _mtl_material(mtl)
            mats.append(mat)
            mat_index[name] = len(mats) - 1
        return mat_index[name]

    def visit(node, parent: np.ndarray):
        if isinstance(node, list):
            for n in node:
                visit(n, parent)
            return
        if isinstance(node, str):
            node = {"model": node}
        M = parent @ _node_matrix(node)
        kind = node.get("type", "model")
        if kind == "light":
            prm = node.get("params", {})
            lt = prm.get("type", "infinite")
            if lt != "infinite":
                raise ImportError_(f"light type {lt!r} is not supported (infinite lights and "
                                   "emissive meshes are)")
            img = _load_image(_resolve(base, prm["texture"])) if prm.get("texture") else None
            lights.append(InfiniteLight(tint=tuple(prm.get("color", [1, 1, 1])),
                                        scale=float(prm.get("scale", 1.0)), image=img))
        if "model" in node:
            m = node["model"]
            if isinstance(m, (list, dict)):
                visit(m, M)
            else:
                path = _resolve(base, m)
                if path.suffix.lower() != ".obj":
                    raise ImportError_(f"{path.name}: only .obj models are supported")
                for g in load_obj(path):
                    mi = material_for(g["name"], g["mtl"])
                    _, emission = _mtl_material(g["mtl"])
                    meshes.append(Mesh(g["positions"], g["normals"], g["indices"], None,
                                       material=mi, emission=emission, name=g["name"]))
                    mesh_names.append(g["name"])
                    instances.append((len(meshes) - 1, M[:3, :4].astype(np.float32)))

    visit(j.get("model", []), np.eye(4))
    if "environment" in j:
        lights.append(InfiniteLight(image=_load_image(_resolve(base, j["environment"]))))
    for entry in j.get("media", []):
        prm = entry.get("params", entry)
        if prm.get("type", "homogeneous") != "homogeneous":
            raise ImportError_("heterogeneous media (.vdb) are not supported")
        st = np.asarray(prm.get("sigma_t", [1, 1, 1]), np.float64)
        al = np.asarray(prm.get("albedo", [0.5, 0.5, 0.5]), np.float64)
        if "sigma_a" in prm or "sigma_s" in prm:
            sa = np.asarray(prm.get("sigma_a", [0.5] * 3), np.float64)
            ss = np.asarray(prm.get("sigma_s", [0.5] * 3), np.float64)
            st = sa + ss
            al = ss / st
        if any(np.asarray(prm.get("Le", [0, 0, 0])) != 0):
            raise ImportError_("emissive media are not supported")
        idx = len(media)
        if "bound" in prm:
            lo, hi = (np.asarray(v, np.float64) for v in prm["bound"])
        else:
            lo, hi = np.full(3, -1e30), np.full(3, 1e30)
        media.append(Medium(None, tuple(lo), tuple(hi), sigma_t=tuple(st), albedo=tuple(al),
                            g=float(prm.get("g", 0.0)), majorant_res=(1, 1, 1)))
        if "bound" in prm:
            boxes.append((idx, lo, hi))
            cube = _unit_cube()
            cube.positions = (cube.positions * (hi - lo) + (hi + lo) / 2).astype(np.float32)
            cube.material = -1
            cube.medium_inside, cube.medium_outside = idx, -1
            meshes.append(cube)
            mesh_names.append("Medium box")
            instances.append((len(meshes) - 1, np.eye(4)[:3, :4].astype(np.float32)))
        for key, inside in (("meshes", True), ("meshes_outside", False)):
            for name in prm.get(key, []):
                for k, nm in enumerate(mesh_names):
                    if nm == name:
                        if inside:
                            meshes[k].medium_inside = idx
                        else:
                            meshes[k].medium_outside = idx
    for entry in j.get("materials", []):
        name = entry.get("name", "Untitled")
        if name not in mat_index:
            mats.append(Material())
            mat_index[name] = len(mats) - 1
        mat = mats[mat_index[name]]
        prm = entry.get("params", {})
        mat.diffuse = tuple(prm.get("diffuse", [1, 1, 1]))
        mat.specular = tuple(prm.get("specular", [0, 0, 0]))
        mat.roughness = float(prm.get("roughness", 1.0))
        mat.specular_transmission = float(prm.get("specular_transmission", 0.0))
        mat.anisotropic = float(prm.get("anisotropic", 0.0))
        if "eta" in prm:
            if not isinstance(prm["eta"], (int, float)):
                raise ImportError_("spectral IoR tables are not supported (give eta as a number)")
            mat.eta = float(prm["eta"])
        bsdf = str(entry.get("bsdf", "diffuse")).lower()
        if bsdf not in BSDF_NAMES:
            raise ImportError_(f"bsdf {bsdf!r} is not supported (diffuse, dielectric, conductor)")
        mat.type = BSDF_NAMES[bsdf]
    if not mats:
        mats.append(Material())
    cam = _camera(j, w, h, boxes)
    return Scene(meshes, instances, mats, cam, w, h, infinite_lights=lights, media=media,
                 name=str(j.get("name", "imported")))


def _camera(j: dict, w: int, h: int, boxes: list) -> Camera:
    data = j.get("camera", {}).get("mData", {})
    if float(data.get("lensRadius", 0.0)) > 1e-6:
        raise ImportError_("thin-lens cameras are not supported (lensRadius must be 0)")
    ctl = j.get("cameraController", {}).get("mData", {})
    pos, R = orbit_pose(ctl.get("target", [0, 0, 0]), float(ctl.get("radius", 5.0)),
                        float(ctl.get("pitch", 0.0)), float(ctl.get("yaw", 0.0)))
    aspect = float(data.get("aspectRatio", w / h))
    film_h = 24.0
    medium = -1
    for k, lo, hi in boxes:   # Camera::update: the medium whose box holds the camera
        if all(lo[a] <= pos[a] <= hi[a] for a in range(3)):
            medium = k
    return Camera(position=tuple(float(x) for x in pos), rotation=R.astype(np.float32),
                  film_size=(film_h * aspect, film_h), focal_length=float(data.get("focalLength", 21.0)),
                  focal_distance=float(data.get("focalDistance", 10.0)), aspect_ratio=aspect,
                  shutter_open=float(data.get("shutterOpen", 0.0)),
                  shutter_time=float(data.get("shutterTime", 0.0)), medium=medium)
