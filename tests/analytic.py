"""A scene with a closed-form answer for the physical estimator: direct light from one
uniformly emitting quad onto a Lambertian plane.

The irradiance at a point x with normal n from a polygon of constant radiance L is
Lambert's contour integral (Lambert 1760; see Arvo, "Irradiance tensors", SIGGRAPH
1995):  E = L/2 * sum_i theta_i * (n . c_i), with theta_i the angle the polygon's
edge i subtends at x and c_i the unit normal of the plane through x and that edge.
A Lambertian point of albedo rho then leaves radiance rho / pi * E towards the
camera.  With a black sky, nothing but the plane and the light, and the camera
looking down at the plane past the light, every camera path's value is this
direct term: the plane cannot see itself and the light ends a path.

A pixel's expectation is that radiance averaged over the pixel (the physical
estimator jitters its camera rays over the whole pixel), here by a 16 x 16 grid of
sub-pixel points; the radiance is smooth, so the grid's error is far below the
renders' noise.
"""
import numpy as np

from pico_gb300 import scenes
from pico_gb300.types import DIFFUSE, LIGHT, Camera, Instance, Material, SceneData

ALBEDO = 0.5
RADIANCE = (40.0, 25.0, 10.0)
LIGHT_QUAD = np.array([[6.0, 3.0, -2.0], [10.0, 3.0, -2.0], [10.0, 3.0, 2.0], [6.0, 3.0, 2.0]])
CAMERA_HEIGHT = 10.0


def polygon_irradiance(x, n, verts):
    """E / L at points x (m, 3) with normal n from the polygon `verts` (k, 3)."""
    x = np.atleast_2d(np.asarray(x, np.float64))
    u = np.asarray(verts, np.float64)[None, :, :] - x[:, None, :]
    u /= np.linalg.norm(u, axis=2, keepdims=True)
    total = np.zeros(len(x))
    k = u.shape[1]
    for i in range(k):
        a, b = u[:, i], u[:, (i + 1) % k]
        theta = np.arccos(np.clip(np.sum(a * b, axis=1), -1.0, 1.0))
        c = np.cross(a, b)
        c /= np.linalg.norm(c, axis=1, keepdims=True)
        total += theta * (c @ np.asarray(n, np.float64))
    return np.abs(total) / 2


def lit_plane_scene() -> SceneData:
    s = SceneData(materials=[Material(diffuse=(ALBEDO, ALBEDO, ALBEDO)),
                             Material(diffuse=(0.0, 0.0, 0.0), emissive=RADIANCE)])
    s.meshes.append(scenes.quad_mesh([[-60, 0, -60], [-60, 0, 60], [60, 0, 60], [60, 0, -60]], [0, 1, 0]))
    s.meshes.append(scenes.quad_mesh(LIGHT_QUAD, [0, -1, 0]))
    s.instances.append(Instance(0, scenes.glm_storage(np.eye(4)), DIFFUSE, 0))
    s.instances.append(Instance(1, scenes.glm_storage(np.eye(4)), LIGHT, 1))
    return s


def lit_plane_camera(size: int = 32) -> Camera:
    """Straight down from 10 above the origin, up = +z: pixel (px, py) looks at the plane point
    (-10 dx, 0, 10 dy) with dx = (px + rx) / W - 1/2, dy = (py + ry) / H - 1/2 (the library's
    camera_ray with right = cross(dir, up) = -x), so the plane fills the image and the light (at
    x >= 6, 3 above the plane) stays out of view."""
    return Camera(position=(0.0, CAMERA_HEIGHT, 0.0), direction=(0.0, -1.0, 0.0), resolution=(size, size),
                  aspect=1.0, up=(0.0, 0.0, 1.0))


def expected_pixels(size: int = 32, sub: int = 16) -> np.ndarray:
    """(size * size, 3): every pixel's expected value, pixel index py * size + px."""
    f = (np.arange(sub) + 0.5) / sub
    px, py = np.meshgrid(np.arange(size), np.arange(size))
    dx = ((px.reshape(-1, 1, 1) + f[None, :, None]) / size - 0.5) * np.ones((1, 1, sub))
    dy = ((py.reshape(-1, 1, 1) + f[None, None, :]) / size - 0.5) * np.ones((1, sub, 1))
    pts = np.stack([-CAMERA_HEIGHT * dx, np.zeros_like(dx), CAMERA_HEIGHT * dy], axis=-1).reshape(-1, 3)
    e = polygon_irradiance(pts, (0.0, 1.0, 0.0), LIGHT_QUAD).reshape(size * size, sub * sub).mean(axis=1)
    return (ALBEDO / np.pi) * e[:, None] * np.asarray(RADIANCE)[None, :]


def glass_slab_scene(kind: int, roughness: float = 0.0, ior: float = 1.5, tint=(1.0, 1.0, 1.0)) -> SceneData:
    """A slab of glass (Transparent or Fresnel kind) between y = -1 and y = 0, 2000 wide, under a
    uniform sky of radiance 1: a smooth dielectric neither creates nor absorbs light and the
    eta^2 factors of entering and leaving cancel, so with a white tint every pixel's expectation
    is 1 (a furnace test of the interface)."""
    s = SceneData(materials=[Material(diffuse=tint, roughness=roughness, ior=ior)], sky=(1.0, 1.0, 1.0))
    w = 1000.0
    s.meshes.append(scenes.quad_mesh([[-w, 0, -w], [-w, 0, w], [w, 0, w], [w, 0, -w]], [0, 1, 0]))
    s.meshes.append(scenes.quad_mesh([[-w, -1, -w], [w, -1, -w], [w, -1, w], [-w, -1, w]], [0, -1, 0]))
    s.instances.append(Instance(0, scenes.glm_storage(np.eye(4)), kind, 0))
    s.instances.append(Instance(1, scenes.glm_storage(np.eye(4)), kind, 0))
    return s


def glass_slab_camera(size: int = 16) -> Camera:
    return Camera(position=(0.0, 5.0, 0.0), direction=(0.0, -1.0, 0.0), resolution=(size, size), aspect=1.0,
                  up=(0.0, 0.0, 1.0))
