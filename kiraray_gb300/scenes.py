"""Synthetic scenes of the benchmark configurations, as flat host arrays.

The reference imports scenes from JSON/OBJ files (src/scene/krrscene.cpp);
there is no network or asset here, so the scenes are generated from fixed
seeds.  Each scene mirrors the reference's scene description: meshes with
positions / normals / texcoords / indices and one material each
(src/core/mesh.h:25-56), instances with object-to-world transforms, materials
with the JSON parameter names of krrscene.cpp:195-227, an optional infinite
light (krrscene.cpp:28-67) and media (krrscene.cpp:69-139).

Scenes:
  cornell_box()          512x512 Cornell box, Lambert walls, quad light.
  large_scene()          2048x2048 fBm heightfield (8,380,418 triangles) plus
                         500 instances of a level-4 icosphere (5,120 triangles
                         each), four emissive quads and a procedural sky.
  volume_box()           the Cornell box with a 256^3 FP16 fBm density medium
                         inside a null-material bounding box.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


@dataclass
class Mesh:
    positions: np.ndarray            # float32 [V, 3]
    normals: np.ndarray              # float32 [V, 3]
    indices: np.ndarray              # uint32 [T, 3]
    texcoords: np.ndarray | None = None
    material: int = 0                # -1 = null material (medium interface)
    emission: tuple = (0.0, 0.0, 0.0)
    medium_inside: int = -1
    medium_outside: int = -1
    name: str = ""


@dataclass
class Material:
    type: int = L.MATERIAL_DIFFUSE
    diffuse: tuple = (1.0, 1.0, 1.0)
    specular: tuple = (0.0, 0.0, 0.0)
    roughness: float = 1.0
    specular_transmission: float = 0.0
    eta: float = 1.5
    anisotropic: float = 0.0


@dataclass
class InfiniteLight:
    tint: tuple = (1.0, 1.0, 1.0)
    scale: float = 1.0
    rotation: np.ndarray = field(default_factory=lambda: np.eye(3, dtype=np.float32))
    image: np.ndarray | None = None  # float32 [H, W, 4]


@dataclass
class Medium:
    density: np.ndarray | None       # float16 [nz, ny, nx]
    bounds_min: tuple
    bounds_max: tuple
    sigma_t: tuple = (1.0, 1.0, 1.0)
    albedo: tuple = (0.9, 0.9, 0.9)
    g: float = 0.0
    scale: float = 1.0
    majorant_res: tuple = (16, 16, 16)


@dataclass
class Camera:
    position: tuple
    rotation: np.ndarray             # camera-to-world, camera looks down -Z
    film_size: tuple = (42.666667, 24.0)
    focal_length: float = 21.0
    focal_distance: float = 10.0
    lens_radius: float = 0.0
    aspect_ratio: float = 1.777777
    shutter_open: float = 0.0
    shutter_time: float = 0.0
    medium: int = -1

    def desc(self) -> L.CameraDesc:
        d = L.CameraDesc()
        d.position[:] = [float(x) for x in self.position]
        d.rotation[:] = [float(x) for x in np.asarray(self.rotation, np.float32).reshape(9)]
        d.film_size[:] = [float(x) for x in self.film_size]
        d.focal_length = self.focal_length
        d.focal_distance = self.focal_distance
        d.lens_radius = self.lens_radius
        d.aspect_ratio = self.aspect_ratio
        d.shutter_open = self.shutter_open
        d.shutter_time = self.shutter_time
        d.medium = self.medium
        return d


def pinhole_rays(scene, width=None, height=None, jitter_seed=None) -> np.ndarray:
    """Camera rays of the scene's pinhole camera through pixel centres (or
    jittered), float32 [H*W, 8]."""
    cam = scene.camera
    w = width or scene.width
    h = height or scene.height
    ys, xs = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    px = xs.reshape(-1).astype(np.float64) + 0.5
    py = ys.reshape(-1).astype(np.float64) + 0.5
    if jitter_seed is not None:
        rng = np.random.default_rng(jitter_seed)
        px += rng.random(px.shape) - 0.5
        py += rng.random(py.shape) - 0.5
    ndcx = 2 * px / w - 1
    ndcy = 1 - 2 * py / h
    tanf = (cam.film_size[1] * 0.5) / cam.focal_length
    d = np.stack([tanf * cam.aspect_ratio * ndcx, tanf * ndcy, -np.ones_like(ndcx)], -1)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    R = np.asarray(cam.rotation, np.float64)
    d = d @ R.T
    out = np.zeros((d.shape[0], 8), np.float32)
    out[:, :3] = cam.position
    out[:, 3] = 0.0
    out[:, 4:7] = d
    out[:, 7] = np.inf
    return out


@dataclass
class Scene:
    meshes: list
    instances: list                  # (mesh index, float32 [3, 4] transform)
    materials: list
    camera: Camera
    width: int
    height: int
    infinite_lights: list = field(default_factory=list)
    media: list = field(default_factory=list)
    max_depth: int = 5
    seed: int = 0
    name: str = ""

    @property
    def n_triangles(self) -> int:
        return int(sum(self.meshes[m].indices.shape[0] for m, _ in self.instances))

    def world_triangles(self) -> np.ndarray:
        """float32 [T, 9]: world-space triangle vertices, instance-major order.

        Rows are computed as m0*x + m1*y + m2*z + m3, left to right, each
        operation rounded to float32 (the device flattening does the same)."""
        out = []
        for mi, xf in self.instances:
            mesh = self.meshes[mi]
            p = mesh.positions.astype(np.float32)
            m = np.asarray(xf, np.float32)
            w = np.empty_like(p)
            for r in range(3):
                acc = (m[r, 0] * p[:, 0]).astype(np.float32)
                acc = (acc + (m[r, 1] * p[:, 1]).astype(np.float32)).astype(np.float32)
                acc = (acc + (m[r, 2] * p[:, 2]).astype(np.float32)).astype(np.float32)
                w[:, r] = (acc + m[r, 3]).astype(np.float32)
            out.append(w[mesh.indices.astype(np.int64)].reshape(-1, 9))
        if not out:
            return np.zeros((0, 9), np.float32)
        return np.ascontiguousarray(np.concatenate(out, 0), dtype=np.float32)

    def desc(self):
        """Builds a krr_scene_desc; returns (desc, keepalive)."""
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data

        meshes = (L.MeshDesc * len(self.meshes))()
        for i, m in enumerate(self.meshes):
            d = meshes[i]
            d.h_positions = ptr(m.positions.astype(np.float32))
            d.h_normals = ptr(m.normals.astype(np.float32))
            d.h_texcoords = ptr(None if m.texcoords is None else m.texcoords.astype(np.float32))
            d.h_indices = ptr(m.indices.astype(np.uint32))
            d.n_vertices = m.positions.shape[0]
            d.n_triangles = m.indices.shape[0]
            d.material = m.material
            d.emission[:] = [float(x) for x in m.emission]
            d.medium_inside = m.medium_inside
            d.medium_outside = m.medium_outside
        insts = (L.InstanceDesc * len(self.instances))()
        for i, (mi, xf) in enumerate(self.instances):
            insts[i].mesh = mi
            insts[i].transform[:] = [float(x) for x in np.asarray(xf, np.float32).reshape(12)]
        mats = (L.MaterialDesc * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            d = mats[i]
            d.type = m.type
            d.diffuse[:] = [float(x) for x in m.diffuse]
            d.specular[:] = [float(x) for x in m.specular]
            d.roughness = m.roughness
            d.specular_transmission = m.specular_transmission
            d.eta = m.eta
            d.anisotropic = m.anisotropic
        lights = (L.InfiniteLightDesc * max(1, len(self.infinite_lights)))()
        for i, li in enumerate(self.infinite_lights):
            d = lights[i]
            d.tint[:] = [float(x) for x in li.tint]
            d.scale = li.scale
            d.rotation[:] = [float(x) for x in np.asarray(li.rotation, np.float32).reshape(9)]
            if li.image is not None:
                d.h_image = ptr(li.image.astype(np.float32))
                d.height, d.width = li.image.shape[:2]
        media = (L.MediumDesc * max(1, len(self.media)))()
        for i, md in enumerate(self.media):
            d = media[i]
            if md.density is not None:
                d.h_density = ptr(md.density.astype(np.float16).view(np.uint16))
                d.nz, d.ny, d.nx = md.density.shape
            d.bounds_min[:] = [float(x) for x in md.bounds_min]
            d.bounds_max[:] = [float(x) for x in md.bounds_max]
            d.sigma_t[:] = [float(x) for x in md.sigma_t]
            d.albedo[:] = [float(x) for x in md.albedo]
            d.g = md.g
            d.scale = md.scale
            d.majorant_res[:] = list(md.majorant_res)
        sd = L.SceneDesc()
        sd.meshes = meshes
        sd.n_meshes = len(self.meshes)
        sd.instances = insts
        sd.n_instances = len(self.instances)
        sd.materials = mats
        sd.n_materials = len(self.materials)
        sd.infinite_lights = lights
        sd.n_infinite_lights = len(self.infinite_lights)
        sd.media = media
        sd.n_media = len(self.media)
        keep += [meshes, insts, mats, lights, media]
        return sd, keep


# ----------------------------------------------------------------- helpers
def bounce_rays(tris: np.ndarray, rays: np.ndarray, hits: np.ndarray, seed: int) -> np.ndarray:
    """Cosine-weighted rays from the primary hit points around the geometric
    normal facing the incoming ray (first-bounce diffuse set)."""
    prim = hits[:, 3].view(np.uint32)
    ok = prim != 0xFFFFFFFF
    t = hits[ok, 0:1].astype(np.float64)
    o = rays[ok, 0:3].astype(np.float64) + t * rays[ok, 4:7]
    v = tris[prim[ok]].reshape(-1, 3, 3).astype(np.float64)
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    n /= np.linalg.norm(n, axis=-1, keepdims=True) + 1e-30
    flip = np.sum(n * rays[ok, 4:7], -1) > 0
    n[flip] *= -1
    rng = np.random.default_rng(seed)
    u1, u2 = rng.random(n.shape[0]), rng.random(n.shape[0])
    r, phi = np.sqrt(u1), 2 * np.pi * u2
    local = np.stack([r * np.cos(phi), r * np.sin(phi), np.sqrt(np.maximum(0, 1 - u1))], -1)
    a = np.where(np.abs(n[:, :1]) > 0.9, np.array([[0, 1, 0]]), np.array([[1, 0, 0]]))
    tt = np.cross(a, n)
    tt /= np.linalg.norm(tt, axis=-1, keepdims=True)
    bb = np.cross(n, tt)
    d = local[:, :1] * tt + local[:, 1:2] * bb + local[:, 2:3] * n
    out = np.zeros((n.shape[0], 8), np.float32)
    out[:, :3] = o + n * 1e-4
    out[:, 4:7] = d
    out[:, 7] = np.inf
    return out


def _xform(scale=(1, 1, 1), rot_y_deg=0.0, translate=(0, 0, 0)) -> np.ndarray:
    c, s = math.cos(math.radians(rot_y_deg)), math.sin(math.radians(rot_y_deg))
    r = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float64)
    m = r @ np.diag(scale)
    out = np.zeros((3, 4), np.float32)
    out[:, :3] = m
    out[:, 3] = translate
    return out


IDENTITY = _xform()


def _quad(p0, p1, p2, p3, normal) -> Mesh:
    pos = np.array([p0, p1, p2, p3], np.float32)
    nrm = np.tile(np.asarray(normal, np.float32), (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    return Mesh(pos, nrm, idx, uv)


def _unit_cube() -> Mesh:
    """Cube [-0.5, 0.5]^3 with flat outward normals, 24 vertices, 12 triangles."""
    faces = [((1, 0, 0), (0, 1, 0), (0, 0, 1)), ((-1, 0, 0), (0, 0, 1), (0, 1, 0)),
             ((0, 1, 0), (0, 0, 1), (1, 0, 0)), ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
             ((0, 0, 1), (1, 0, 0), (0, 1, 0)), ((0, 0, -1), (0, 1, 0), (1, 0, 0))]
    pos, nrm, idx = [], [], []
    for n, u, v in faces:
        n, u, v = map(np.asarray, (n, u, v))
        base = len(pos)
        c = 0.5 * n
        for a, b in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            pos.append(c + 0.5 * a * u + 0.5 * b * v)
            nrm.append(n)
        # counter-clockwise seen from outside: (u, v, n) right-handed
        if np.dot(np.cross(u, v), n) > 0:
            idx += [[base, base + 1, base + 2], [base, base + 2, base + 3]]
        else:
            idx += [[base, base + 2, base + 1], [base, base + 3, base + 2]]
    return Mesh(np.array(pos, np.float32), np.array(nrm, np.float32), np.array(idx, np.uint32))


def look_at(position, target, up=(0, 1, 0)) -> np.ndarray:
    """Camera-to-world rotation for a camera looking down its local -Z."""
    f = np.asarray(target, np.float64) - np.asarray(position, np.float64)
    f /= np.linalg.norm(f)
    back = -f
    right = np.cross(np.asarray(up, np.float64), back)
    right /= np.linalg.norm(right)
    upv = np.cross(back, right)
    return np.stack([right, upv, back], axis=1).astype(np.float32)


def _camera(position, target, vfov_deg, width, height) -> Camera:
    film_h = 24.0
    focal = (film_h * 0.5) / math.tan(math.radians(vfov_deg) * 0.5)
    aspect = width / height
    return Camera(position=tuple(position), rotation=look_at(position, target),
                  film_size=(film_h * aspect, film_h), focal_length=focal, aspect_ratio=aspect)


# ------------------------------------------------------------ Cornell box
RED = (0.63, 0.065, 0.05)
GREEN = (0.14, 0.45, 0.09)
WHITE = (0.73, 0.73, 0.73)
LIGHT_LE = (17.0, 12.0, 4.0)


def cornell_box(width: int = 512, height: int = 512, max_depth: int = 5, seed: int = 0) -> Scene:
    """Cornell box in [0,1]^3: 5 walls (10 triangles), a short box 0.3^3
    rotated 18 deg and a tall box 0.3x0.6x0.3 rotated -20 deg (24 triangles),
    a 0.25x0.25 one-sided quad light at y=0.999 with radiance (17,12,4).
    Pinhole camera at (0.5,0.5,-1.4) looking down +z, 40 deg vertical fov.
    Walls face the room interior; the camera's right is world -x, so the red
    wall (x=1) appears on the left of the image."""
    mats = [Material(diffuse=WHITE), Material(diffuse=RED), Material(diffuse=GREEN),
            Material(diffuse=(0.0, 0.0, 0.0))]
    meshes = [
        _quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 1, 0)),      # floor
        _quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, -1, 0)),     # ceiling
        _quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, -1)),     # back
        _quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0), (-1, 0, 0)),     # red, x=1
        _quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0)),      # green, x=0
        _unit_cube(),                                                     # boxes
        _quad((0.375, 0.999, 0.375), (0.625, 0.999, 0.375), (0.625, 0.999, 0.625),
              (0.375, 0.999, 0.625), (0, -1, 0)),                           # light
    ]
    mat_of = [0, 0, 0, 1, 2, 0, 3]
    for m, k in zip(meshes, mat_of):
        m.material = k
    meshes[6].emission = LIGHT_LE
    # make the light quad's winding face -y (face normal agrees with shading normal)
    meshes[6].indices = meshes[6].indices[:, [0, 2, 1]].copy()
    for m in meshes[:5]:
        fn = np.cross(m.positions[1] - m.positions[0], m.positions[2] - m.positions[0])
        if np.dot(fn, m.normals[0]) < 0:
            m.indices = m.indices[:, [0, 2, 1]].copy()
    instances = [(i, IDENTITY) for i in range(5)]
    instances.append((5, _xform((0.3, 0.3, 0.3), 18.0, (0.33, 0.15, 0.37))))
    instances.append((5, _xform((0.3, 0.6, 0.3), -20.0, (0.66, 0.3, 0.66))))
    instances.append((6, IDENTITY))
    cam = _camera((0.5, 0.5, -1.4), (0.5, 0.5, 0.0), 40.0, width, height)
    return Scene(meshes, instances, mats, cam, width, height, max_depth=max_depth, seed=seed,
                 name="cornell_box")


# ------------------------------------------------------------- noise
def fbm2(n: int, octaves: int, seed: int, base_freq: int = 4, gain: float = 0.5) -> np.ndarray:
    """2-D value-noise fBm on an n x n grid, smoothstep-interpolated lattices."""
    rng = np.random.default_rng(seed)
    acc = np.zeros((n, n), np.float64)
    amp, freq, norm = 1.0, base_freq, 0.0
    x = np.linspace(0.0, 1.0, n, endpoint=False)
    for _ in range(octaves):
        lat = rng.random((freq + 1, freq + 1))
        u = x * freq
        i0 = np.floor(u).astype(np.int64)
        f = u - i0
        f = f * f * (3 - 2 * f)
        a = lat[i0][:, i0] * (1 - f)[None, :] + lat[i0][:, i0 + 1] * f[None, :]
        b = lat[i0 + 1][:, i0] * (1 - f)[None, :] + lat[i0 + 1][:, i0 + 1] * f[None, :]
        acc += amp * (a * (1 - f)[:, None] + b * f[:, None])
        norm += amp
        amp *= gain
        freq *= 2
    return acc / norm


def fbm3(n: int, octaves: int, seed: int, base_freq: int = 4, gain: float = 0.5) -> np.ndarray:
    """3-D value-noise fBm on an n^3 grid (float32)."""
    rng = np.random.default_rng(seed)
    acc = np.zeros((n, n, n), np.float32)
    amp, freq, norm = 1.0, base_freq, 0.0
    x = np.linspace(0.0, 1.0, n, endpoint=False)
    for _ in range(octaves):
        lat = rng.random((freq + 1, freq + 1, freq + 1)).astype(np.float32)
        u = x * freq
        i0 = np.floor(u).astype(np.int64)
        f = (u - i0)
        f = (f * f * (3 - 2 * f)).astype(np.float32)
        g = 1 - f
        # interpolate along x (last axis), then y, then z
        c = lat[:, :, i0] * g[None, None, :] + lat[:, :, i0 + 1] * f[None, None, :]
        c = c[:, i0, :] * g[None, :, None] + c[:, i0 + 1, :] * f[None, :, None]
        c = c[i0, :, :] * g[:, None, None] + c[i0 + 1, :, :] * f[:, None, None]
        acc += np.float32(amp) * c
        norm += amp
        amp *= gain
        freq *= 2
    return acc / np.float32(norm)


# ------------------------------------------------------------- icosphere
def icosphere(level: int) -> Mesh:
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    p = np.array(verts, np.float32)
    return Mesh(p, p.copy(), np.array(faces, np.uint32))


# --------------------------------------------------- 10M-triangle scene
def _heightfield(n: int, extent: float, amplitude: float, seed: int) -> Mesh:
    h = fbm2(n, 9, seed) * amplitude
    xs = np.linspace(-extent, extent, n, dtype=np.float64)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    pos = np.stack([X, h, Z], -1).reshape(-1, 3).astype(np.float32)
    dx = 2 * extent / (n - 1)
    gz, gx = np.gradient(h, dx)
    nrm = np.stack([-gx, np.ones_like(h), -gz], -1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    i = np.arange(n - 1, dtype=np.uint32)
    I, J = np.meshgrid(i, i, indexing="xy")   # I = column (x), J = row (z)
    v00 = (J * n + I).reshape(-1)
    v10 = v00 + 1
    v01 = v00 + n
    v11 = v01 + 1
    # winding with face normal +y: (v00, v01, v10) and (v10, v01, v11)
    idx = np.empty((2 * v00.size, 3), np.uint32)
    idx[0::2] = np.stack([v00, v01, v10], -1)
    idx[1::2] = np.stack([v10, v01, v11], -1)
    uv = np.stack([(X + extent) / (2 * extent), (Z + extent) / (2 * extent)], -1)
    return Mesh(pos, nrm.reshape(-1, 3).astype(np.float32), idx,
                uv.reshape(-1, 2).astype(np.float32)), h


def _sky(width: int, height: int) -> np.ndarray:
    """Procedural lat-long sky (float32 RGBA): horizon-to-zenith gradient, a
    darker ground half and a sun disk.  v = acos(y)/pi as in the reference's
    worldToLatLong (src/util/math_utils.h:133)."""
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    U, V = np.meshgrid(u, v, indexing="xy")
    theta = V * np.pi
    phi = (U - 0.5) * 2 * np.pi
    y = np.cos(theta)
    x = np.sin(theta) * np.sin(phi)
    z = -np.sin(theta) * np.cos(phi)
    zen = np.array([0.25, 0.45, 0.9])
    hor = np.array([0.9, 0.9, 1.0])
    t = np.clip(y, 0, 1)[..., None]
    sky = hor * (1 - t) + zen * t
    ground = np.array([0.2, 0.18, 0.15]) * np.ones_like(sky)
    img = np.where((y >= 0)[..., None], sky, ground)
    sun = np.array([0.4, 0.8, -0.45])
    sun /= np.linalg.norm(sun)
    cosang = x * sun[0] + y * sun[1] + z * sun[2]
    img += (cosang > np.cos(np.radians(2.0)))[..., None] * np.array([400.0, 380.0, 320.0])
    out = np.ones((height, width, 4), np.float32)
    out[..., :3] = img
    return out


def large_scene(width: int = 1920, height: int = 1080, max_depth: int = 8, seed: int = 1,
                grid: int = 2048, n_spheres: int = 500, sphere_level: int = 4,
                sky_size: tuple = (2048, 1024)) -> Scene:
    """10.9M-triangle scene: a grid x grid fBm heightfield (2*(grid-1)^2
    triangles over [-50,50]^2, heights up to 8) and n_spheres instances of a
    level-4 icosphere (5,120 triangles) at uniform-random positions above the
    terrain with scales U[0.5,3].  Instance materials: 40% Lambert, 40% GGX
    conductor, 20% rough dielectric (IOR 1.5), roughness U[0.05,1].  Lights:
    four emissive 4x4 quads at y=30 and a procedural 2048x1024 sky."""
    rng = np.random.default_rng(seed)
    extent = 50.0
    terrain, h = _heightfield(grid, extent, 8.0, seed)
    terrain.material = 0
    mats = [Material(diffuse=(0.55, 0.5, 0.42))]
    meshes = [terrain]
    instances = [(0, IDENTITY)]
    sphere = icosphere(sphere_level)
    kinds = rng.random(n_spheres)
    for i in range(n_spheres):
        rough = float(rng.uniform(0.05, 1.0))
        col = tuple(float(c) for c in rng.uniform(0.2, 0.95, 3))
        if kinds[i] < 0.4:
            mats.append(Material(type=L.MATERIAL_DIFFUSE, diffuse=col, roughness=rough))
        elif kinds[i] < 0.8:
            mats.append(Material(type=L.MATERIAL_CONDUCTOR, diffuse=col, roughness=rough, eta=1.5))
        else:
            mats.append(Material(type=L.MATERIAL_DIELECTRIC, diffuse=(1.0, 1.0, 1.0),
                                 roughness=rough, eta=1.5, specular_transmission=1.0))
        # one mesh record per instance (the material is per mesh in the
        # reference); the records share the icosphere's arrays
        meshes.append(Mesh(sphere.positions, sphere.normals, sphere.indices, None,
                           material=1 + i))
    sx = rng.uniform(-45, 45, n_spheres)
    sz = rng.uniform(-45, 45, n_spheres)
    sc = rng.uniform(0.5, 3.0, n_spheres)
    n = grid
    for i in range(n_spheres):
        gi = int(np.clip((sz[i] + extent) / (2 * extent) * (n - 1), 0, n - 1))
        gj = int(np.clip((sx[i] + extent) / (2 * extent) * (n - 1), 0, n - 1))
        y = float(h[gi, gj]) + sc[i] + rng.uniform(0.0, 6.0)
        instances.append((1 + i, _xform((sc[i],) * 3, float(rng.uniform(0, 360)),
                                        (sx[i], y, sz[i]))))
    # four emissive quads facing down
    mats.append(Material(diffuse=(0.0, 0.0, 0.0)))
    light_mat = len(mats) - 1
    for k, (cx, cz) in enumerate([(-20, -20), (20, -20), (-20, 20), (20, 20)]):
        q = _quad((cx - 2, 30, cz - 2), (cx + 2, 30, cz - 2), (cx + 2, 30, cz + 2),
                  (cx - 2, 30, cz + 2), (0, -1, 0))
        q.indices = q.indices[:, [0, 2, 1]].copy()
        q.material = light_mat
        q.emission = (40.0, 38.0, 34.0)
        meshes.append(q)
        instances.append((len(meshes) - 1, IDENTITY))
    sky = InfiniteLight(scale=1.0, image=_sky(*sky_size))
    cam = _camera((0.0, 22.0, -62.0), (0.0, 2.0, 0.0), 45.0, width, height)
    return Scene(meshes, instances, mats, cam, width, height, infinite_lights=[sky],
                 max_depth=max_depth, seed=seed, name="large_scene")


# ------------------------------------------------------------ volume box
def volume_density(n: int = 256, seed: int = 2, threshold: float = 0.4) -> np.ndarray:
    """256^3 FP16 density: 6-octave fBm thresholded at 0.4, rescaled to [0,1]."""
    d = fbm3(n, 6, seed)
    d = np.clip((d - threshold) / (1.0 - threshold), 0.0, 1.0)
    return d.astype(np.float16)


def volume_box(width: int = 1024, height: int = 1024, max_depth: int = 16, seed: int = 2,
               grid: int = 256) -> Scene:
    """The Cornell box with a heterogeneous medium (sigma_t scale 20, albedo
    0.9, HG g=0.3, 16^3 majorant grid) filling [0.15,0.85]x[0.05,0.75]x
    [0.15,0.85] inside a null-material box that is the medium interface."""
    sc = cornell_box(width, height, max_depth, seed)
    lo, hi = (0.15, 0.05, 0.15), (0.85, 0.75, 0.85)
    med = Medium(volume_density(grid, seed), lo, hi, sigma_t=(1.0, 1.0, 1.0),
                 albedo=(0.9, 0.9, 0.9), g=0.3, scale=20.0, majorant_res=(16, 16, 16))
    cube = _unit_cube()
    ext = np.array(hi) - np.array(lo)
    cen = (np.array(hi) + np.array(lo)) / 2
    cube.positions = (cube.positions * ext + cen).astype(np.float32)
    cube.material = -1
    cube.medium_inside = 0
    cube.medium_outside = -1
    sc.meshes.append(cube)
    sc.instances.append((len(sc.meshes) - 1, IDENTITY))
    sc.media = [med]
    sc.name = "volume_box"
    return sc
