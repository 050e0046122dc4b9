"""Seeded synthetic scenes with the shapes of the benchmark workloads.

The reference measures on OBJ scenes that are not available here, so these generators stand in
for them. Every scene is built in screen space (pixel x, pixel y, view depth) and unprojected
through a fixed perspective camera (camera at the origin looking down -Z), so the rasterised
image of each triangle is exactly the 2D triangle that was drawn. Geometry is handed over in
the reference's input format: float3 world positions, ``quads_ib`` with 4 indices per quad
(a lone triangle is the degenerate quad ``(a, b, c, c)``, as ``genQuads`` emits it in
src/quad_generator.cpp:192) and ``InstanceData`` records of at most 1024 quads, split from draw
calls the way ``LucidRenderer::uploadInstances`` does (src/lucid_renderer.cpp:388-400).

Workloads (all seeded; the seed is recorded in ``Scene.meta``):

* ``random_tris`` (the 1280x720 / 100k-triangle CPU workload and its variants): triangle
  centroids uniform over the viewport or Gaussian around the centre, area log-normal, a random
  orientation and shape, per-vertex view depth uniform in [0.1, 100], RGBA colours.
* ``meshes`` (3840x2160, 5M triangles): 2000 noisy spheres or grids of 2500 triangles built
  from real quads, per-mesh random rotation, log-uniform scale and placement, 30% translucent.
* ``batch_views``: 64 random-triangle views of random resolution and triangle count.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

# LUCID_INST_* flags (data/shaders/shared/definitions.glsl:85-94)
INST_HAS_VERTEX_COLORS = 0x001
INST_HAS_VERTEX_NORMALS = 0x004
INST_TEX_OPAQUE = 0x010
INST_HAS_UV_RECT = 0x020
INST_HAS_ALBEDO_TEXTURE = 0x040
INST_HAS_COLOR = 0x200

COLOR_RGBA8 = 0
COLOR_RGBA16F = 1
COLOR_RGBA32F = 2

MAX_INSTANCE_QUADS = 1024


class LucidConfig(ctypes.Structure):
    """ctypes mirror of ``lucid_config`` (LucidConfig, structures.glsl:102-111; 352 bytes)."""

    _fields_ = [
        ("ws_origins", ctypes.c_float * 16),
        ("ws_dirs", ctypes.c_float * 16),
        ("ws_origin0", ctypes.c_float * 4),
        ("ws_dir0", ctypes.c_float * 4),
        ("ws_dirx", ctypes.c_float * 4),
        ("ws_diry", ctypes.c_float * 4),
        ("view_proj_matrix", ctypes.c_float * 16),
        ("ambient_color", ctypes.c_float * 4),
        ("sun_color", ctypes.c_float * 4),
        ("sun_dir", ctypes.c_float * 4),
        ("sun_power", ctypes.c_float),
        ("ambient_power", ctypes.c_float),
        ("_pad0", ctypes.c_float * 2),
        ("background_color", ctypes.c_float * 4),
        ("enable_backface_culling", ctypes.c_uint32),
        ("num_instances", ctypes.c_int32),
        ("instance_packet_size", ctypes.c_int32),
        ("_pad1", ctypes.c_uint32),
    ]


assert ctypes.sizeof(LucidConfig) == 352


@dataclass
class Camera:
    position: tuple = (0.0, 0.0, 0.0)
    right: tuple = (1.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    forward: tuple = (0.0, 0.0, -1.0)
    fov_y: float = math.radians(60.0)
    near: float = 0.05
    far: float = 500.0


def make_config(cam: Camera, width: int, height: int, background=(0.0, 0.0, 0.0, 1.0),
                backface_culling: bool = False) -> LucidConfig:
    """Fills a LucidConfig from a camera.

    Follows FrustumInfo (src/shading.cpp:46-74): corner rays 0..3 at NDC (-1,-1), (-1,1),
    (1,1), (1,-1); dir0 = dirs[0], dirx = (dirs[3]-dirs[0])/W, diry = (dirs[1]-dirs[0])/H,
    origin0 = camera position. Lighting is SceneLighting::makeDefault (src/shading.cpp:26-34).
    All values are computed in double precision and rounded to float once, in the same order
    as ``lucid_make_config`` in the C library (a CPU test checks the two agree bit for bit).
    """
    f32 = lambda v: float(np.float32(v))  # the C camera struct holds floats
    p = [f32(v) for v in cam.position]
    r = [f32(v) for v in cam.right]
    u = [f32(v) for v in cam.up]
    f = [f32(v) for v in cam.forward]
    ty = math.tan(f32(cam.fov_y) * 0.5)
    tx = ty * (float(width) / float(height))

    def corner(nx, ny):
        return [f[i] + r[i] * (nx * tx) + u[i] * (ny * ty) for i in range(3)]

    dirs = [corner(-1.0, -1.0), corner(-1.0, 1.0), corner(1.0, 1.0), corner(1.0, -1.0)]
    dirx = [(dirs[3][i] - dirs[0][i]) * (1.0 / width) for i in range(3)]
    diry = [(dirs[1][i] - dirs[0][i]) * (1.0 / height) for i in range(3)]

    # view matrix rows: right, up, -forward; translation -R.p etc.
    zb = [-f[0], -f[1], -f[2]]
    view = [[r[0], r[1], r[2], -(r[0] * p[0] + r[1] * p[1] + r[2] * p[2])],
            [u[0], u[1], u[2], -(u[0] * p[0] + u[1] * p[1] + u[2] * p[2])],
            [zb[0], zb[1], zb[2], -(zb[0] * p[0] + zb[1] * p[1] + zb[2] * p[2])],
            [0.0, 0.0, 0.0, 1.0]]
    n, fa = f32(cam.near), f32(cam.far)
    proj = [[1.0 / tx, 0.0, 0.0, 0.0],
            [0.0, 1.0 / ty, 0.0, 0.0],
            [0.0, 0.0, (fa + n) / (n - fa), (2.0 * fa * n) / (n - fa)],
            [0.0, 0.0, -1.0, 0.0]]
    vp = [[sum(proj[i][k] * view[k][j] for k in range(4)) for j in range(4)] for i in range(4)]

    cfg = LucidConfig()
    for c in range(4):
        for i in range(3):
            cfg.ws_dirs[c * 4 + i] = dirs[c][i]
            cfg.ws_origins[c * 4 + i] = p[i]
    for i in range(3):
        cfg.ws_origin0[i] = p[i]
        cfg.ws_dir0[i] = dirs[0][i]
        cfg.ws_dirx[i] = dirx[i]
        cfg.ws_diry[i] = diry[i]
    cfg.ws_origin0[3] = 1.0
    for col in range(4):
        for row in range(4):
            cfg.view_proj_matrix[col * 4 + row] = vp[row][col]
    cfg.ambient_color[:] = (0.8, 0.8, 0.6, 1.0)
    cfg.sun_color[:] = (0.8, 0.8, 0.8, 1.0)
    cfg.sun_dir[:] = (0.842121, -0.300567, -0.447763, 0.0)
    cfg.sun_power = 2.5
    cfg.ambient_power = 0.4
    for i in range(4):
        cfg.background_color[i] = float(background[i])
    cfg.enable_backface_culling = 1 if backface_culling else 0
    cfg.num_instances = 0
    cfg.instance_packet_size = 1
    return cfg


def build_instances(draw_calls, max_instances: int = 64 * 1024):
    """Splits draw calls into instances of <= 1024 quads.

    Mirrors LucidRenderer::uploadInstances (src/lucid_renderer.cpp:352-429): index_offset =
    4*(quad_offset + i), vertex_offset = 0, flags = draw-call options (plus INST_HAS_COLOR when
    the material colour is not white), truncated to ``max_instances``.
    ``draw_calls``: iterable of (quad_offset, num_quads, opts, material_rgba8).
    Returns (instances int32[N,4], colors uint32[N], total_quads).
    """
    inst, cols = [], []
    total = 0
    for quad_offset, num_quads, opts, color in draw_calls:
        if num_quads <= 0:
            continue
        opts = int(opts)
        color = int(color) & 0xFFFFFFFF
        if color != 0xFFFFFFFF:
            opts |= INST_HAS_COLOR
        total += num_quads
        for i in range(0, num_quads, MAX_INSTANCE_QUADS):
            n = min(MAX_INSTANCE_QUADS, num_quads - i)
            inst.append((4 * (quad_offset + i), 0, n, opts & 0xFFFF))
            cols.append(color)
    if len(inst) > max_instances:
        inst = inst[:max_instances]
        cols = cols[:max_instances]
    instances = np.array(inst, dtype=np.int64).reshape(-1, 4).astype(np.int32)
    colors = np.array(cols, dtype=np.uint64).astype(np.uint32)
    return instances, colors, int(instances[:, 2].sum()) if len(inst) else 0


@dataclass
class Texture:
    """RGBA8 texture with its mip chain: levels[l] is uint32 [max(1, h >> l), max(1, w >> l)]."""
    levels: list

    @property
    def width(self):
        return int(self.levels[0].shape[1])

    @property
    def height(self):
        return int(self.levels[0].shape[0])

    def packed(self) -> np.ndarray:
        return np.concatenate([lv.reshape(-1) for lv in self.levels]).astype(np.uint32)


def make_texture(width, height, seed=0, alpha_range=(1.0, 1.0), levels=None) -> Texture:
    """Seeded RGBA8 texture (smooth colour waves plus noise) with a 2x2 box-filtered mip chain."""
    rng = np.random.default_rng(seed)
    yy, xx = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    base = np.stack([0.5 + 0.5 * np.sin(xx * (0.3 + 0.2 * rng.random()) + rng.random() * 6),
                     0.5 + 0.5 * np.sin(yy * (0.25 + 0.2 * rng.random()) + rng.random() * 6),
                     0.5 + 0.5 * np.sin((xx + yy) * 0.11 + rng.random() * 6)], -1)
    base = np.clip(base + rng.normal(0, 0.05, base.shape), 0, 1)
    alpha = rng.uniform(alpha_range[0], alpha_range[1], size=(height, width, 1))
    img = np.concatenate([base, alpha], -1)
    n = levels or (int(math.log2(max(width, height))) + 1)
    out = []
    cur = img
    for _ in range(n):
        q = np.clip(np.rint(cur * 255.0), 0, 255).astype(np.uint32)
        out.append(q[..., 0] | (q[..., 1] << 8) | (q[..., 2] << 16) | (q[..., 3] << 24))
        h, w = cur.shape[:2]
        if h == 1 and w == 1:
            break
        nh, nw = max(1, h // 2), max(1, w // 2)
        cur = cur[:nh * (h // nh), :nw * (w // nw)].reshape(nh, h // nh, nw, w // nw, 4).mean((1, 3))
    return Texture(out)


def encode_normals(n: np.ndarray) -> np.ndarray:
    """10 bits per axis, v = round(n * 511 + 512) (the inverse of funcs.glsl:61-66)."""
    q = np.clip(np.rint(n * 511.0 + 512.0), 0, 1023).astype(np.uint32)
    return q[..., 0] | (q[..., 1] << 10) | (q[..., 2] << 20)


@dataclass
class Scene:
    width: int
    height: int
    positions: np.ndarray          # float32 [V, 3]
    colors: np.ndarray             # uint32 [V] (RGBA8) | float16 [V, 4] | float32 [V, 4]
    color_format: int
    quads: np.ndarray              # uint32 [Q, 4]
    instances: np.ndarray          # int32 [N, 4]: index_offset, vertex_offset, num_quads, flags
    instance_colors: np.ndarray    # uint32 [N]
    config: LucidConfig
    tri_opacity: np.ndarray | None = None  # float32 [Q*2] or None
    meta: dict = field(default_factory=dict)
    # optional shading inputs (shading.glsl:125-176)
    tex_coords: np.ndarray | None = None   # float32 [V, 2]
    uv_rects: np.ndarray | None = None     # float32 [N, 4]: uv min, uv size per instance
    normals: np.ndarray | None = None      # uint32 [V] encoded normals
    opaque_tex: "Texture | None" = None
    trans_tex: "Texture | None" = None

    @property
    def num_quads(self) -> int:
        return int(self.quads.shape[0])

    @property
    def num_tris(self) -> int:
        return int(self.meta.get("num_tris", self.quads.shape[0]))

    def input_bytes(self) -> int:
        n = self.positions.nbytes + self.colors.nbytes + self.quads.nbytes
        n += self.instances.nbytes + self.instance_colors.nbytes
        if self.tri_opacity is not None:
            n += self.tri_opacity.nbytes
        return int(n)


def _unproject(sx, sy, depth, width, height, cam: Camera):
    """Screen (pixel) position and view depth -> world position for the default camera."""
    ty = math.tan(cam.fov_y * 0.5)
    tx = ty * (float(width) / float(height))
    nx = 2.0 * sx / width - 1.0
    ny = 2.0 * sy / height - 1.0
    return np.stack([nx * tx * depth, ny * ty * depth, -depth], axis=-1)


def _random_triangles(rng, n, centers, areas):
    """Random-orientation triangles with given centroids [n,2] and areas [n] (pixels)."""
    theta0 = rng.uniform(0.0, 2.0 * math.pi, size=n)
    jitter = rng.uniform(-0.45, 0.45, size=(n, 3))
    radius = rng.uniform(0.6, 1.0, size=(n, 3))
    ang = theta0[:, None] + np.array([0.0, 2.0 * math.pi / 3, 4.0 * math.pi / 3])[None] + jitter
    pts = np.stack([np.cos(ang) * radius, np.sin(ang) * radius], axis=-1)  # [n,3,2]
    e1 = pts[:, 1] - pts[:, 0]
    e2 = pts[:, 2] - pts[:, 0]
    a0 = 0.5 * np.abs(e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
    scale = np.sqrt(areas / np.maximum(a0, 1e-6))
    pts = pts * scale[:, None, None]
    pts = pts - pts.mean(axis=1, keepdims=True) + centers[:, None, :]
    flip = rng.random(n) < 0.5  # random winding (backface culling is off by default)
    pts[flip] = pts[flip][:, ::-1]
    return pts


def _rgba8(r, g, b, a):
    q = lambda v: np.clip(np.rint(np.asarray(v) * 255.0), 0, 255).astype(np.uint32)
    return q(r) | (q(g) << 8) | (q(b) << 16) | (q(a) << 24)


def random_tris(width=1280, height=720, num_tris=100_000, seed=0, center_sigma=None,
                area_median=40.0, area_sigma=1.5, alpha_range=(0.2, 0.8), depth_range=(0.1, 100.0),
                large_fraction=0.0, large_area=(10_000.0, 50_000.0), color_format=COLOR_RGBA8,
                tri_opacity_range=None, background=(0.0, 0.0, 0.0, 1.0), cam: Camera | None = None):
    """Independent random triangles (each the degenerate quad (a, b, c, c))."""
    cam = cam or Camera()
    rng = np.random.default_rng(seed)
    if center_sigma is None:
        centers = np.stack([rng.uniform(0, width, num_tris), rng.uniform(0, height, num_tris)], -1)
    else:
        centers = rng.normal(0.0, center_sigma, size=(num_tris, 2)) + np.array([width, height]) * 0.5
    areas = np.exp(rng.normal(math.log(area_median), area_sigma, size=num_tris))
    if large_fraction > 0:
        big = rng.random(num_tris) < large_fraction
        lo, hi = large_area
        areas[big] = np.exp(rng.uniform(math.log(lo), math.log(hi), size=int(big.sum())))
    pts = _random_triangles(rng, num_tris, centers, areas)
    depth = rng.uniform(depth_range[0], depth_range[1], size=(num_tris, 3))
    pos = _unproject(pts[..., 0], pts[..., 1], depth, width, height, cam)
    positions = pos.reshape(-1, 3).astype(np.float32)
    nv = positions.shape[0]
    rgb = rng.random((nv, 3))
    alpha = rng.uniform(alpha_range[0], alpha_range[1], size=nv)
    if color_format == COLOR_RGBA8:
        colors = _rgba8(rgb[:, 0], rgb[:, 1], rgb[:, 2], alpha)
    elif color_format == COLOR_RGBA16F:
        colors = np.concatenate([rgb, alpha[:, None]], 1).astype(np.float16)
    else:
        colors = np.concatenate([rgb, alpha[:, None]], 1).astype(np.float32)
    base = np.arange(num_tris, dtype=np.uint32) * 3
    quads = np.stack([base, base + 1, base + 2, base + 2], axis=1).astype(np.uint32)
    instances, inst_colors, _ = build_instances([(0, num_tris, INST_HAS_VERTEX_COLORS, 0xFFFFFFFF)])
    tri_opacity = None
    if tri_opacity_range is not None:
        tri_opacity = np.zeros(num_tris * 2, dtype=np.float32)
        tri_opacity[0::2] = rng.uniform(tri_opacity_range[0], tri_opacity_range[1], num_tris)
    cfg = make_config(cam, width, height, background)
    meta = dict(kind="random_tris", seed=seed, num_tris=num_tris, width=width, height=height,
                area_median=area_median, area_sigma=area_sigma, large_fraction=large_fraction,
                center_sigma=center_sigma, color_format=color_format)
    return Scene(width, height, positions, colors, color_format, quads, instances, inst_colors, cfg,
                 tri_opacity, meta)


def _sphere_grid(nu, nv):
    """Unit sphere as an nu x nv grid of quads (poles included as thin quads)."""
    u = np.linspace(0.0, 2.0 * math.pi, nu + 1)
    v = np.linspace(0.02, math.pi - 0.02, nv + 1)
    uu, vv = np.meshgrid(u, v, indexing="xy")
    pts = np.stack([np.sin(vv) * np.cos(uu), np.cos(vv), np.sin(vv) * np.sin(uu)], -1)
    return pts  # [nv+1, nu+1, 3]


def _plane_grid(nu, nv):
    u = np.linspace(-1.0, 1.0, nu + 1)
    v = np.linspace(-1.0, 1.0, nv + 1)
    uu, vv = np.meshgrid(u, v, indexing="xy")
    return np.stack([uu, vv, np.zeros_like(uu)], -1)


def _grid_quads(nu, nv, base):
    """Quads of an (nv+1) x (nu+1) vertex grid, ordered in 8x4-cell patches so that every 64
    consecutive triangles form a compact meshlet."""
    quads = []
    for pv in range(0, nv, 4):
        for pu in range(0, nu, 8):
            for j in range(pv, min(pv + 4, nv)):
                for i in range(pu, min(pu + 8, nu)):
                    a = base + j * (nu + 1) + i
                    quads.append((a, a + 1, a + 1 + (nu + 1), a + (nu + 1)))
    return np.array(quads, dtype=np.uint32)


def textured_scene(width=160, height=120, num_tris=800, seed=0, uv_rects=True, vertex_normals=True,
                   opaque_fraction=0.5, tex_size=(64, 32), tri_opacity_range=None, color_format=COLOR_RGBA8):
    """Random triangles with texture coordinates (spanning up to a few texture repeats), two
    instance groups sampling the opaque and the transparent texture (optionally through per-instance
    uv rects), optional per-vertex normals: the shading inputs of shading.glsl:125-176."""
    sc = random_tris(width, height, num_tris, seed=seed, area_median=300.0, area_sigma=1.0,
                     color_format=color_format, tri_opacity_range=tri_opacity_range)
    rng = np.random.default_rng(seed + 1)
    nv = sc.positions.shape[0]
    tex = rng.uniform(-1.0, 3.0, size=(nv, 2)).astype(np.float32)
    n_op = int(round(num_tris * opaque_fraction))
    base = INST_HAS_VERTEX_COLORS | INST_HAS_ALBEDO_TEXTURE | (INST_HAS_VERTEX_NORMALS if vertex_normals else 0)
    if uv_rects:
        base |= INST_HAS_UV_RECT
    dcs = [(0, n_op, base | INST_TEX_OPAQUE, 0xFFFFFFFF), (n_op, num_tris - n_op, base, 0xFFC0E0FF)]
    instances, inst_colors, _ = build_instances([dc for dc in dcs if dc[1] > 0])
    rects = np.zeros((instances.shape[0], 4), np.float32)
    rects[:, :2] = rng.uniform(0.0, 0.5, size=(instances.shape[0], 2))
    rects[:, 2:] = rng.uniform(0.25, 0.5, size=(instances.shape[0], 2))
    normals = None
    if vertex_normals:
        nrm = rng.normal(size=(nv, 3))
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        normals = encode_normals(nrm)
    ot = make_texture(tex_size[0], tex_size[1], seed=seed + 2)
    tt = make_texture(tex_size[1], tex_size[0], seed=seed + 3, alpha_range=(0.2, 1.0))
    return Scene(width, height, sc.positions, sc.colors, sc.color_format, sc.quads, instances, inst_colors,
                 sc.config, sc.tri_opacity, dict(sc.meta, kind="textured"), tex_coords=tex,
                 uv_rects=rects if uv_rects else None, normals=normals, opaque_tex=ot, trans_tex=tt)


def tri_mesh(kind="sphere", nu=64, nv=32, seed=0, noise=0.01, shuffle=True):
    """Triangle mesh for the quad generator: a sphere or plane grid whose cells are split into two
    triangles along a random diagonal, vertices jittered by `noise`, triangles in random order
    (shuffle) or grid order. Returns (positions float32 [V, 3], tris int32 [T, 3])."""
    rng = np.random.default_rng(seed)
    pts = _sphere_grid(nu, nv) if kind == "sphere" else _plane_grid(nu, nv)
    pos = pts.reshape(-1, 3) + rng.normal(0.0, noise, size=(pts.shape[0] * pts.shape[1], 3))
    tris = []
    for j in range(nv):
        for i in range(nu):
            a = j * (nu + 1) + i
            b, c, d = a + 1, a + 1 + (nu + 1), a + (nu + 1)
            if rng.random() < 0.5:
                tris += [(a, b, c), (a, c, d)]
            else:
                tris += [(a, b, d), (b, c, d)]
    tris = np.array(tris, np.int32)
    if shuffle:
        tris = tris[rng.permutation(len(tris))]
    return pos.astype(np.float32), tris


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def meshes(width=3840, height=2160, num_meshes=2000, seed=2, cells=(50, 25),
           translucent_fraction=0.3, alpha_range=(0.2, 0.6), scale_range=(0.5, 20.0),
           depth_range=(30.0, 400.0), noise=0.03, color_format=COLOR_RGBA16F,
           background=(0.0, 0.0, 0.0, 1.0), cam: Camera | None = None):
    """Noisy spheres and grids of 2*cells[0]*cells[1] triangles each, built from real quads.

    Each mesh gets a random rotation, a log-uniform scale over ``scale_range`` and a position
    in view space (a random screen point at a random view depth); 30% of meshes are
    translucent with alpha in ``alpha_range``, the rest opaque. Quads of a mesh are ordered in
    patches of 32 quads (64 triangles), the meshlets of the workload.
    """
    cam = cam or Camera(far=2000.0)
    rng = np.random.default_rng(seed)
    nu, nv = cells
    sphere = _sphere_grid(nu, nv).reshape(-1, 3)
    plane = _plane_grid(nu, nv).reshape(-1, 3)
    vpm = sphere.shape[0]
    quads_local = _grid_quads(nu, nv, 0)
    qpm = quads_local.shape[0]
    all_pos = np.empty((num_meshes * vpm, 3), dtype=np.float64)
    all_col = np.empty((num_meshes * vpm, 4), dtype=np.float64)
    quads = np.empty((num_meshes * qpm, 4), dtype=np.uint32)
    kinds = rng.random(num_meshes) < 0.5
    scales = np.exp(rng.uniform(math.log(scale_range[0]), math.log(scale_range[1]), num_meshes))
    translucent = rng.random(num_meshes) < translucent_fraction
    for m in range(num_meshes):
        base_pts = sphere if kinds[m] else plane
        pts = base_pts * (1.0 + noise * rng.normal(size=(vpm, 1)))
        pts = pts @ _rotation(rng).T * scales[m]
        sx, sy = rng.uniform(0, width), rng.uniform(0, height)
        d = rng.uniform(depth_range[0], depth_range[1])
        center = _unproject(np.array(sx), np.array(sy), np.array(d), width, height, cam)
        all_pos[m * vpm:(m + 1) * vpm] = pts + center
        rgb = rng.random(3) * 0.6 + 0.2
        col = np.clip(rgb[None, :] + 0.15 * rng.normal(size=(vpm, 3)), 0.0, 1.0)
        alpha = rng.uniform(*alpha_range, size=vpm) if translucent[m] else np.ones(vpm)
        all_col[m * vpm:(m + 1) * vpm, :3] = col
        all_col[m * vpm:(m + 1) * vpm, 3] = alpha
        quads[m * qpm:(m + 1) * qpm] = quads_local + m * vpm
    positions = all_pos.astype(np.float32)
    if color_format == COLOR_RGBA16F:
        colors = all_col.astype(np.float16)
    elif color_format == COLOR_RGBA32F:
        colors = all_col.astype(np.float32)
    else:
        colors = _rgba8(all_col[:, 0], all_col[:, 1], all_col[:, 2], all_col[:, 3])
    dcs = [(m * qpm, qpm, INST_HAS_VERTEX_COLORS, 0xFFFFFFFF) for m in range(num_meshes)]
    instances, inst_colors, _ = build_instances(dcs)
    cfg = make_config(cam, width, height, background)
    meta = dict(kind="meshes", seed=seed, num_meshes=num_meshes, num_tris=2 * quads.shape[0],
                width=width, height=height, color_format=color_format)
    return Scene(width, height, positions, colors, color_format, quads, instances, inst_colors, cfg,
                 None, meta)


# ---------------------------------------------------------------------------------------------
# Named workloads

def workload(name: str, seed: int | None = None) -> Scene:
    """The benchmark workloads by name.

    cpu720:   1280x720, 100k triangles, centroids uniform, area log-normal (median 40 px^2,
              sigma 1.5), depth U[0.1,100], RGBA8, alpha U[0.2,0.8].
    heavy1080: 1920x1080, 1M triangles, centroids Gaussian (sigma 0.2*width) around the centre,
              area log-normal (median 60, sigma 2) with 5% of triangles drawn log-uniformly in
              [10k, 50k] px^2, depth U[0.1,100], RGBA8, alpha U[0.1,0.9].
    meshes4k: 3840x2160, 2000 meshes x 2500 triangles, FP16 RGBA.
    grad512:  512x512, 200k triangles as cpu720, FP32 RGBA, per-triangle opacity U[0.1,0.9].
    """
    if name == "cpu720":
        return random_tris(1280, 720, 100_000, seed=0 if seed is None else seed)
    if name == "heavy1080":
        return random_tris(1920, 1080, 1_000_000, seed=1 if seed is None else seed,
                           center_sigma=0.2 * 1920, area_median=60.0, area_sigma=2.0,
                           alpha_range=(0.1, 0.9), large_fraction=0.05)
    if name == "heavy1080_small":  # same distributions, 250k triangles (profiling captures)
        return random_tris(1920, 1080, 250_000, seed=1 if seed is None else seed,
                           center_sigma=0.2 * 1920, area_median=60.0, area_sigma=2.0,
                           alpha_range=(0.1, 0.9), large_fraction=0.05)
    if name == "meshes4k":
        return meshes(seed=2 if seed is None else seed)
    if name == "grad512":
        return random_tris(512, 512, 200_000, seed=4 if seed is None else seed,
                           color_format=COLOR_RGBA32F, tri_opacity_range=(0.1, 0.9))
    raise ValueError(f"unknown workload {name}")


def batch_views(num_views=64, seed=3, min_tris=10_000, max_tris=500_000):
    """Random-triangle views (cpu720 style) with resolutions drawn from {256^2, 512^2,
    1280x720, 1920x1080} and triangle counts log-uniform in [min_tris, max_tris]."""
    rng = np.random.default_rng(seed)
    sizes = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    views = []
    for v in range(num_views):
        w, h = sizes[int(rng.integers(0, 4))]
        n = int(round(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))))
        views.append(random_tris(w, h, n, seed=seed * 1000 + v))
    return views


def screen_triangles(tris, colors, width, height, background=(0.0, 0.0, 0.0, 1.0),
                     cam: Camera | None = None, backface_culling=False) -> Scene:
    """Scene from explicit screen-space triangles.

    tris: [N, 3, 3] of (pixel x, pixel y, view depth); colors: [N, 3, 4] RGBA8 per vertex.
    Each triangle becomes the degenerate quad (a, b, c, c).
    """
    cam = cam or Camera()
    tris = np.asarray(tris, np.float64).reshape(-1, 3, 3)
    n = tris.shape[0]
    pos = _unproject(tris[..., 0], tris[..., 1], tris[..., 2], width, height, cam)
    positions = pos.reshape(-1, 3).astype(np.float32)
    cols = np.asarray(colors, np.uint32).reshape(-1, 4)
    colors32 = cols[:, 0] | (cols[:, 1] << 8) | (cols[:, 2] << 16) | (cols[:, 3] << 24)
    base = np.arange(n, dtype=np.uint32) * 3
    quads = np.stack([base, base + 1, base + 2, base + 2], axis=1).astype(np.uint32)
    instances, inst_colors, _ = build_instances([(0, n, INST_HAS_VERTEX_COLORS, 0xFFFFFFFF)])
    cfg = make_config(cam, width, height, background, backface_culling)
    return Scene(width, height, positions, colors32.astype(np.uint32), COLOR_RGBA8, quads, instances,
                 inst_colors, cfg, None, dict(kind="screen_triangles", num_tris=n))


def small_scene(width=96, height=72, num_tris=300, seed=7, **kw) -> Scene:
    """Small random scene for parity tests (seconds on the oracle)."""
    kw.setdefault("area_median", 60.0)
    return random_tris(width, height, num_tris, seed=seed, **kw)
