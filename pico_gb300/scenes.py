"""Seeded synthetic scenes and ray batches for the two benchmark workloads.

* Cornell box: five wall quads of the unit cube (two triangles each, inward
  normals), two boxes rotated by -18 and +18 degrees that share one unit-cube
  mesh, a 0.25 x 0.25 ceiling light of radiance (17, 12, 4); white 0.73, red
  (0.65, 0.05, 0.05) and green (0.12, 0.45, 0.15) Lambert walls.
* Instance field: 4096 instances of a level-4 icosphere (5120 triangles,
  2562 vertices, normals = positions) with translations uniform in
  [-50, 50]^3, uniform scale log-uniform in [0.5, 4] and uniformly random
  rotations; 16,777,216 rays, half coherent primary rays of a 4096 x 4096
  pinhole, half cosine-distributed rays leaving random surface points.
* Lit field (full renders): the instance field with metalness-roughness
  materials, a ground quad and eight quad area lights, seen by a 1920 x 1080
  camera.

Transforms are built in float64 and stored as float32 in glm's column-major
order (array row c is glm column c).  Everything is a pure function of the
seed.
"""
from __future__ import annotations

import numpy as np

from .types import (BTDF, DELTA, DIELECTRIC, DIFFUSE, FRESNEL, LIGHT, RAY_DTYPE, SHAPE_CUBE, SHAPE_SPHERE, SKY_CONSTANT,
                    Camera, Instance, Material, Mesh, SceneData, Sky)


# ----------------------------------------------------------------------------- matrices
def glm_storage(m: np.ndarray) -> np.ndarray:
    """Mathematical 4x4 matrix (acting on column vectors) -> glm storage order, float32."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.float64).T.astype(np.float32))


def translate(t) -> np.ndarray:
    m = np.eye(4)
    m[:3, 3] = t
    return m


def scale(s) -> np.ndarray:
    return np.diag([*np.broadcast_to(np.asarray(s, dtype=np.float64), (3,)), 1.0])


def rotate_y(deg: float) -> np.ndarray:
    a = np.deg2rad(deg)
    c, s = np.cos(a), np.sin(a)
    m = np.eye(4)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def quat_matrix(q) -> np.ndarray:
    """Rotation matrix of a unit quaternion (x, y, z, w)."""
    x, y, z, w = q
    m = np.eye(4)
    m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return m


def random_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform rotations: points drawn uniformly in the unit 4-ball, normalised."""
    out = np.empty((0, 4))
    while len(out) < n:
        q = rng.uniform(-1.0, 1.0, size=(2 * (n - len(out)) + 16, 4))
        r2 = (q * q).sum(axis=1)
        q = q[(r2 <= 1.0) & (r2 > 1e-6)]
        out = np.concatenate([out, q / np.sqrt((q * q).sum(axis=1, keepdims=True))])
    return out[:n]


# ----------------------------------------------------------------------------- meshes
def quad_mesh(corners, normal) -> Mesh:
    """Two triangles (0,1,2) and (0,2,3) over four corners, flat normal."""
    p = np.asarray(corners, np.float64)
    n = np.tile(np.asarray(normal, np.float64), (4, 1))
    return Mesh(p, n, np.array([[0, 1, 2], [0, 2, 3]], np.uint32))


def implicit_mesh(shape: int) -> Mesh:
    """The implicit "Sphere" (radius 0.5) or "Cube" ([-0.5, 0.5]^3) asset."""
    z = np.zeros((0, 3))
    return Mesh(z, z, np.zeros((0, 3), np.uint32), shape=shape)


def cube_mesh() -> Mesh:
    """Unit cube [-0.5, 0.5]^3, 12 triangles, 24 vertices with outward face normals."""
    faces = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            n = np.zeros(3)
            n[axis] = sign
            u = np.zeros(3)
            u[(axis + 1) % 3] = 1.0
            v = np.cross(n, u)
            c = n * 0.5
            pts = [c - 0.5 * u - 0.5 * v, c + 0.5 * u - 0.5 * v, c + 0.5 * u + 0.5 * v, c - 0.5 * u + 0.5 * v]
            faces.append((pts, n))
    pos, nrm, idx = [], [], []
    for f, (pts, n) in enumerate(faces):
        pos += pts
        nrm += [n] * 4
        b = 4 * f
        idx += [[b, b + 1, b + 2], [b, b + 2, b + 3]]
    return Mesh(np.array(pos), np.array(nrm), np.array(idx, np.uint32))


def icosphere(level: int = 4) -> Mesh:
    """Subdivided icosahedron on the unit sphere (20 * 4^level triangles), normals = positions."""
    t = (1.0 + np.sqrt(5.0)) / 2.0
    verts = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
             [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
             [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
             [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
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
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        faces = nf
    p = np.array(verts)
    return Mesh(p, p, np.array(faces, np.uint32))


# ----------------------------------------------------------------------------- Cornell box
WHITE = Material(diffuse=(0.73, 0.73, 0.73))
RED = Material(diffuse=(0.65, 0.05, 0.05))
GREEN = Material(diffuse=(0.12, 0.45, 0.15))
LAMP = Material(diffuse=(0.78, 0.78, 0.78), emissive=(17.0, 12.0, 4.0))


def cornell_box() -> SceneData:
    s = SceneData(materials=[WHITE, RED, GREEN, LAMP])
    eye = glm_storage(np.eye(4))
    walls = [  # (corners, inward normal, material)
        ([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]], [0, 1, 0], 0),      # floor
        ([[0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 1, 0]], [0, -1, 0], 0),     # ceiling
        ([[0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], [0, 0, -1], 0),     # back
        ([[0, 0, 0], [0, 0, 1], [0, 1, 1], [0, 1, 0]], [1, 0, 0], 1),      # left (x = 0), red
        ([[1, 0, 0], [1, 1, 0], [1, 1, 1], [1, 0, 1]], [-1, 0, 0], 2),     # right (x = 1), green
    ]
    for corners, n, mat in walls:
        s.meshes.append(quad_mesh(corners, n))
        s.instances.append(Instance(len(s.meshes) - 1, eye, DIFFUSE, mat))
    s.meshes.append(cube_mesh())
    cube = len(s.meshes) - 1
    short_box = translate([0.33, 0.15, 0.35]) @ rotate_y(-18.0) @ scale([0.3, 0.3, 0.3])
    tall_box = translate([0.66, 0.3, 0.67]) @ rotate_y(18.0) @ scale([0.3, 0.6, 0.3])
    s.instances.append(Instance(cube, glm_storage(short_box), DIFFUSE, 0))
    s.instances.append(Instance(cube, glm_storage(tall_box), DIFFUSE, 0))
    y = 0.999
    s.meshes.append(quad_mesh([[0.375, y, 0.375], [0.375, y, 0.625], [0.625, y, 0.625], [0.625, y, 0.375]],
                              [0, -1, 0]))
    s.instances.append(Instance(len(s.meshes) - 1, eye, LIGHT, 3))
    return s


def cornell_camera(width: int = 256, height: int = 256) -> Camera:
    """Looks into the open front (z = 0) of the box; the reference camera's fixed
    image plane (half-height 0.5 at distance 1) frames the opening from z = -1.05."""
    return Camera(position=(0.5, 0.5, -1.05), direction=(0.0, 0.0, 1.0), resolution=(width, height),
                  aspect=float(width // height) if width >= height else width / height)


# ----------------------------------------------------------------------------- instance field
def instance_field(n_instances: int = 4096, level: int = 4, seed: int = 12345, extent: float = 50.0) -> SceneData:
    rng = np.random.default_rng(seed)
    s = SceneData(materials=[Material(diffuse=(0.5, 0.5, 0.5))])
    s.meshes.append(icosphere(level))
    trans = rng.uniform(-extent, extent, size=(n_instances, 3))
    scales = np.exp(rng.uniform(np.log(0.5), np.log(4.0), size=n_instances))
    quats = random_quaternions(rng, n_instances)
    for i in range(n_instances):
        m = translate(trans[i]) @ quat_matrix(quats[i]) @ scale(scales[i])
        s.instances.append(Instance(0, glm_storage(m), DIFFUSE, 0))
    return s


def metalness_roughness(albedo, metalness: float, roughness: float) -> Material:
    """Render::ConstantMetalnessRoughnessMaterial (Render/BasicMaterials.cpp:28-39) in float32:
    diffuse = albedo * (1 - 0.04) * (1 - metalness), specular = lerp(0.04, albedo, metalness)."""
    f = np.float32
    a = np.asarray(albedo, f)
    m = f(metalness)
    diffuse = (a * (f(1.0) - f(0.04))) * (f(1.0) - m)
    spec = f(0.04) * (f(1.0) - m) + a * m
    return Material(diffuse=tuple(float(x) for x in diffuse), specular=tuple(float(x) for x in spec),
                    roughness=float(f(roughness)))


def lit_field(n_instances: int = 4096, level: int = 4, seed: int = 12345, n_lights: int = 8,
              extent: float = 50.0) -> SceneData:
    """The instance field with a ground plane and quad area lights, for full renders.

    Per instance: base colour U[0.1, 0.9]^3, metalness Bernoulli(0.3), roughness
    U[0.05, 1], as a Dielectric BSRDF with the reference's metalness-roughness
    material.  Ground: a 400 x 400 Lambert quad (albedo 0.5) below the field.
    Lights: n_lights downward-facing quads of side U[4, 12] above the field,
    radiance log-uniform in [1, 50].  Sky: black (the reference's default).
    """
    s = instance_field(n_instances=n_instances, level=level, seed=seed, extent=extent)
    rng = np.random.default_rng(seed + 1)
    s.materials = []
    for i, inst in enumerate(s.instances):
        albedo = rng.uniform(0.1, 0.9, 3)
        metal = 1.0 if rng.random() < 0.3 else 0.0
        rough = rng.uniform(0.05, 1.0)
        s.materials.append(metalness_roughness(albedo, metal, rough))
        inst.material = i
        inst.bsdf = DIELECTRIC
    y0 = -1.2 * extent
    s.meshes.append(quad_mesh([[-4 * extent, y0, -4 * extent], [-4 * extent, y0, 4 * extent],
                               [4 * extent, y0, 4 * extent], [4 * extent, y0, -4 * extent]], [0, 1, 0]))
    s.materials.append(Material(diffuse=(0.5, 0.5, 0.5)))
    s.instances.append(Instance(len(s.meshes) - 1, glm_storage(np.eye(4)), DIFFUSE, len(s.materials) - 1))
    for _ in range(n_lights):
        cx, cz = rng.uniform(-extent, extent, 2)
        y = rng.uniform(1.1, 1.3) * extent
        h = 0.5 * rng.uniform(4.0, 12.0)
        le = float(np.exp(rng.uniform(np.log(1.0), np.log(50.0))))
        s.meshes.append(quad_mesh([[cx - h, y, cz - h], [cx + h, y, cz - h], [cx + h, y, cz + h],
                                   [cx - h, y, cz + h]], [0, -1, 0]))
        s.materials.append(Material(diffuse=(0.8, 0.8, 0.8), emissive=(le, le, le)))
        s.instances.append(Instance(len(s.meshes) - 1, glm_storage(np.eye(4)), LIGHT, len(s.materials) - 1))
    return s


BATCH_RESOLUTIONS = ((128, 128), (256, 256), (512, 512), (768, 432), (1024, 1024))
BATCH_SPP = (4, 16, 64)


def batch_workload(n_renders: int = 64, seed: int = 2024, level: int = 4, size_scale: float = 1.0):
    """Heterogeneous renders for batched rendering, each from its own seed: resolution uniform
    from 128^2, 256^2, 512^2, 768x432, 1024^2 (times size_scale), a lit field of 64-4096
    instances (log-uniform), spp uniform from {4, 16, 64}, depth uniform in 4-8.  Returns a list
    of dicts with scene, camera, max_samples, max_depth and seed."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_renders):
        W, H = BATCH_RESOLUTIONS[rng.integers(len(BATCH_RESOLUTIONS))]
        W, H = max(8, int(W * size_scale)), max(8, int(H * size_scale))
        n_inst = int(round(np.exp(rng.uniform(np.log(64), np.log(4096)))))
        spp = int(BATCH_SPP[rng.integers(len(BATCH_SPP))])
        depth = int(rng.integers(4, 9))
        scene_seed = int(rng.integers(1, 2**31 - 1))
        out.append({"scene": lit_field(n_instances=n_inst, level=level, seed=scene_seed),
                    "camera": lit_field_camera(W, H), "max_samples": spp, "max_depth": depth, "seed": k + 1,
                    "instances": n_inst})
    return out


def cornell_shapes() -> SceneData:
    """The Cornell box with the implicit assets and the remaining lobes: a Transparent
    and a Fresnel glass sphere (IoR 1.5), a Delta mirror cube, and a small sphere and a
    small cube as extra area lights."""
    s = cornell_box()
    sph, cub = len(s.meshes), len(s.meshes) + 1
    s.meshes += [implicit_mesh(SHAPE_SPHERE), implicit_mesh(SHAPE_CUBE)]
    glass, mirror, lamp = len(s.materials), len(s.materials) + 1, len(s.materials) + 2
    s.materials += [Material(diffuse=(0.9, 0.9, 0.9), specular=(0.04, 0.04, 0.04), roughness=0.1, ior=1.5),
                    Material(diffuse=(0.1, 0.1, 0.1), specular=(0.9, 0.8, 0.7), roughness=0.2),
                    Material(diffuse=(0.8, 0.8, 0.8), emissive=(6.0, 6.0, 6.0))]

    def place(t, sc, rot=0.0):
        return glm_storage(translate(t) @ rotate_y(rot) @ scale(sc))

    s.instances += [Instance(sph, place((0.3, 0.25, 0.4), 0.35), BTDF, glass),
                    Instance(sph, place((0.7, 0.2, 0.6), 0.3), FRESNEL, glass),
                    Instance(cub, place((0.55, 0.6, 0.3), 0.2, 30.0), DELTA, mirror),
                    Instance(sph, place((0.2, 0.8, 0.7), 0.1), LIGHT, lamp),
                    Instance(cub, place((0.8, 0.85, 0.3), 0.08), LIGHT, lamp)]
    return s


def glossy_field(n_instances: int = 48, level: int = 2, seed: int = 21) -> SceneData:
    """A small lit field for the physical estimator: metalness-roughness spheres, one of
    them a Specular_Delta mirror, a Lambert ground, three quad lights, a constant blue sky
    and a sun."""
    s = lit_field(n_instances=n_instances, level=level, seed=seed, n_lights=3, extent=8.0)
    mirror = len(s.materials)
    s.materials.append(Material(specular=(0.9, 0.9, 0.9)))
    s.instances[0].bsdf = DELTA
    s.instances[0].material = mirror
    s.sky = (0.10, 0.15, 0.25)
    d = np.array([0.3, -1.0, 0.2])
    s.sky_image = Sky(SKY_CONSTANT, None, True, tuple(d / np.linalg.norm(d)), (2.0, 1.8, 1.5))
    return s


def glossy_field_camera(width: int = 64, height: int = 48) -> Camera:
    return Camera(position=(0.0, 4.0, -24.0), direction=(0.0, -0.12, 1.0), resolution=(width, height),
                  aspect=width / height)


def lit_field_camera(width: int = 1920, height: int = 1080) -> Camera:
    return Camera(position=(0.0, 10.0, -140.0), direction=(0.0, -0.08, 1.0), resolution=(width, height),
                  aspect=width / height)


def field_camera(resolution: int = 4096) -> Camera:
    return Camera(position=(0.0, 0.0, -130.0), direction=(0.0, 0.0, 1.0), resolution=(resolution, resolution))


def primary_rays(cam: Camera, rows: tuple[int, int] | None = None, seed: int = 7, jitter: bool = True) -> np.ndarray:
    """Camera::generate_ray (Core/Camera.cpp:11-28) over whole rows of the image, in float32
    with the reference's operation order; xi is a seeded uniform jitter."""
    W, H = int(cam.resolution[0]), int(cam.resolution[1])
    r0, r1 = rows if rows else (0, H)
    n = W * (r1 - r0)
    rng = np.random.default_rng(seed)
    xi = rng.random((n, 2), dtype=np.float32) if jitter else np.zeros((n, 2), np.float32)
    f = np.float32
    py, px = np.divmod(np.arange(n, dtype=np.int64), W)
    py = py + r0
    rx, ry = xi[:, 0] / f(2.0), xi[:, 1] / f(2.0)
    dx = ((px.astype(f) + rx) / f(W) - f(0.5)) * f(cam.aspect)
    dy = (py.astype(f) + ry) / f(H) - f(0.5)
    D = np.asarray(cam.direction, f)
    U = np.asarray(cam.up, f)
    Dn = D * (f(1.0) / np.sqrt((D[0] * D[0] + D[1] * D[1]) + D[2] * D[2]))
    R = np.array([Dn[1] * U[2] - U[1] * Dn[2], Dn[2] * U[0] - U[2] * Dn[0], Dn[0] * U[1] - U[0] * Dn[1]], f)
    v = (f(1.0) * D)[None, :] + dy[:, None] * U[None, :]
    v = v + dx[:, None] * R[None, :]
    inv = f(1.0) / np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])
    v = v * inv[:, None]
    rays = np.zeros(n, RAY_DTYPE)
    rays["org"][:, :3] = np.asarray(cam.position, f)
    rays["org"][:, 3] = 1.0
    rays["dir"][:, :3] = v
    rays["dir"][:, 3] = cam.far_plane
    return rays


def surface_rays(scene: SceneData, n: int, seed: int = 11, offset: float = 0.01) -> np.ndarray:
    """Cosine-distributed rays leaving random points of random instances, origin
    pushed 0.01 along the normal as the integrator does (Render/Integrators.cpp:199)."""
    rng = np.random.default_rng(seed)
    inst = rng.integers(0, len(scene.instances), n)
    out = np.zeros(n, RAY_DTYPE)
    mats = np.stack([np.asarray(i.transform, np.float64).reshape(4, 4).T for i in scene.instances])
    mesh_of = np.array([i.mesh for i in scene.instances])
    P = np.empty((n, 3))
    N = np.empty((n, 3))
    for mi, mesh in enumerate(scene.meshes):
        sel = np.nonzero(mesh_of[inst] == mi)[0]
        if len(sel) == 0:
            continue
        tri = rng.integers(0, len(mesh.indices), len(sel))
        r1, r2 = rng.random(len(sel)), rng.random(len(sel))
        su = np.sqrt(r1)
        b0, b1 = 1.0 - su, r2 * su
        b2 = 1.0 - b0 - b1
        ids = mesh.indices[tri].astype(np.int64)
        pos = mesh.positions.astype(np.float64)
        nrm = mesh.normals.astype(np.float64)
        p = b0[:, None] * pos[ids[:, 0]] + b1[:, None] * pos[ids[:, 1]] + b2[:, None] * pos[ids[:, 2]]
        nn = b0[:, None] * nrm[ids[:, 0]] + b1[:, None] * nrm[ids[:, 1]] + b2[:, None] * nrm[ids[:, 2]]
        M = mats[inst[sel]]
        P[sel] = np.einsum("kij,kj->ki", M[:, :3, :3], p) + M[:, :3, 3]
        N[sel] = np.einsum("kij,kj->ki", M[:, :3, :3], nn)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    helper = np.where(np.abs(N[:, 2:3]) < 0.9, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]])
    T = np.cross(N, helper)
    T /= np.linalg.norm(T, axis=1, keepdims=True)
    B = np.cross(N, T)
    u1, u2 = rng.random(n), rng.random(n)
    r, phi = np.sqrt(u1), 2.0 * np.pi * u2
    d = (r * np.cos(phi))[:, None] * T + (r * np.sin(phi))[:, None] * B + np.sqrt(1.0 - u1)[:, None] * N
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out["org"][:, :3] = P + offset * N
    out["org"][:, 3] = 1.0
    out["dir"][:, :3] = d
    out["dir"][:, 3] = 10000.0
    return out


def field_rays(scene: SceneData, n_total: int = 1 << 24, resolution: int = 4096, seed: int = 7) -> np.ndarray:
    """Half primary rays (a centred band of whole image rows), half surface rays."""
    cam = field_camera(resolution)
    n_primary = n_total // 2
    rows = max(1, n_primary // resolution)
    r0 = (resolution - rows) // 2
    prim = primary_rays(cam, (r0, r0 + rows), seed=seed)[:n_primary]
    bounce = surface_rays(scene, n_total - len(prim), seed=seed + 1)
    return np.concatenate([prim, bounce])
