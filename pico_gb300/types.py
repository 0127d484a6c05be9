"""Scene data in host memory and its ctypes image for the C ABI (include/pico_gpu.h).

A scene is what the reference's Scene gathers before it renders
(Core/Scene.hpp:105-122): meshes (LowerLevelMeshBVH inputs copied out of an
aiMesh), instances (UpperLevelBVH::Entry: mesh, transform, BSRDF, material)
and constant materials (Core::EvaluatedMaterial).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

# BSRDF kinds, numbered like Render::BSRDF_Type (Render/BSRDF.hpp:32-39).
DIFFUSE, SPECULAR, DIELECTRIC, BTDF, LIGHT, FRESNEL, DELTA = 0, 1, 2, 3, 4, 5, 6
# Mesh shapes (pico_shape).
SHAPE_TRIANGLES, SHAPE_SPHERE, SHAPE_CUBE = 0, 1, 2
# Render estimators (pico_estimator).
ESTIMATOR_REFERENCE, ESTIMATOR_PHYSICAL, ESTIMATOR_RADIANCE_CACHE = 0, 1, 2

RAY_DTYPE = np.dtype([("org", "<f4", (4,)), ("dir", "<f4", (4,))])
HIT_DTYPE = np.dtype([("inst", "<u4"), ("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
MISS = 0xFFFFFFFF


class CMesh(C.Structure):
    _fields_ = [("nverts", C.c_uint32), ("ntris", C.c_uint32),
                ("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("uvs", C.POINTER(C.c_float)), ("indices", C.POINTER(C.c_uint32)),
                ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3), ("shape", C.c_uint32)]


class CInstance(C.Structure):
    _fields_ = [("mesh", C.c_uint32), ("bsdf", C.c_uint32), ("material", C.c_uint32),
                ("reserved", C.c_uint32), ("transform", C.c_float * 16)]


class CMaterial(C.Structure):
    _fields_ = [("diffuse", C.c_float * 3), ("specular", C.c_float * 3), ("roughness", C.c_float),
                ("emissive", C.c_float * 3), ("index_of_refraction", C.c_float)]


# Sky kinds (pico_sky_kind).
SKY_CONSTANT, SKY_CUBE_RGBA8, SKY_EQUIRECT_RGBAF = 0, 1, 2


class CSky(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("pixels", C.c_void_p), ("use_sun", C.c_int32),
                ("sun_direction", C.c_float * 3), ("sun_colour", C.c_float * 3)]


class CSceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(CMesh)), ("nmeshes", C.c_uint32),
                ("instances", C.POINTER(CInstance)), ("ninstances", C.c_uint32),
                ("materials", C.POINTER(CMaterial)), ("nmaterials", C.c_uint32),
                ("sky_rgb", C.c_float * 3), ("sky", C.POINTER(CSky))]


class CCamera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("direction", C.c_float * 3), ("up", C.c_float * 3),
                ("resolution", C.c_uint32 * 2), ("aspect", C.c_float), ("near_plane", C.c_float),
                ("far_plane", C.c_float), ("fov", C.c_float)]


class CLaunchParams(C.Structure):
    _fields_ = [("wavefront", C.c_uint32), ("extend_ctas_per_sm", C.c_uint32), ("branches", C.c_uint32),
                ("piece_paths", C.c_uint32), ("extend_threads", C.c_uint32), ("reserved", C.c_uint32)]


class CBatchReport(C.Structure):
    _fields_ = [("build_ms", C.c_double), ("run_ms", C.c_double), ("graph_nodes", C.c_uint64),
                ("samples", C.c_uint64), ("rays", C.c_uint64)]


class CNrcConfig(C.Structure):
    """pico_nrc_config: the radiance cache's encoding, optimiser and per-frame training budget."""
    _fields_ = [("log2_table_size", C.c_uint32), ("base_resolution", C.c_float), ("max_resolution", C.c_float),
                ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3), ("learning_rate", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float), ("train_paths", C.c_uint32),
                ("train_batch", C.c_uint32), ("max_train_steps", C.c_uint32), ("warmup_frames", C.c_uint32),
                ("seed", C.c_uint64), ("bounces", C.c_uint32), ("infer_groups", C.c_uint32)]


# pico_nrc_query: 16 x 4 bytes.
NRC_QUERY_DTYPE = np.dtype([("position", "<f4", (3,)), ("direction", "<f4", (3,)), ("normal", "<f4", (3,)),
                            ("roughness", "<f4"), ("albedo", "<f4", (3,)), ("payload", "<u4"), ("pad", "<u4", (2,))])


class CRenderConfig(C.Structure):
    _fields_ = [("max_ray_depth", C.c_uint32), ("max_samples", C.c_uint32), ("max_variance", C.c_float),
                ("height", C.c_uint32), ("width", C.c_uint32), ("tonemap", C.c_int32),
                ("denoise", C.c_int32), ("estimator", C.c_uint32), ("seed", C.c_uint64)]


class CRenderItem(C.Structure):
    """pico_render_item: one render of a batch (scene handle, camera, config, progressive buffers)."""
    _fields_ = [("scene", C.c_void_p), ("camera", CCamera), ("config", CRenderConfig),
                ("pixels_rgb", C.POINTER(C.c_float)), ("sample_count", C.POINTER(C.c_uint32)),
                ("variance_rgb", C.POINTER(C.c_float))]


@dataclass
class Mesh:
    positions: np.ndarray            # (nverts, 3) float32
    normals: np.ndarray              # (nverts, 3) float32
    indices: np.ndarray              # (ntris, 3) uint32
    uvs: np.ndarray | None = None    # (nverts, 2) float32
    shape: int = SHAPE_TRIANGLES     # SHAPE_SPHERE / SHAPE_CUBE: implicit asset, arrays empty

    def __post_init__(self):
        self.positions = np.ascontiguousarray(self.positions, dtype=np.float32).reshape(-1, 3)
        self.normals = np.ascontiguousarray(self.normals, dtype=np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(self.indices, dtype=np.uint32).reshape(-1, 3)
        if self.uvs is not None:
            self.uvs = np.ascontiguousarray(self.uvs, dtype=np.float32).reshape(-1, 2)

    @property
    def aabb(self) -> tuple[np.ndarray, np.ndarray]:
        """aiMesh::mAABB as aiProcess_GenBoundingBoxes computes it: min/max of the positions."""
        if len(self.positions) == 0:
            z = np.zeros(3, np.float32)
            return z, z
        return self.positions.min(axis=0), self.positions.max(axis=0)


@dataclass
class Material:
    diffuse: tuple = (0.0, 0.0, 0.0)
    specular: tuple = (0.0, 0.0, 0.0)
    roughness: float = 1.0
    emissive: tuple = (0.0, 0.0, 0.0)
    ior: float = 0.0                 # index of refraction of a transparent material


@dataclass
class Instance:
    mesh: int
    transform: np.ndarray            # (4, 4) float32, column-major storage order like glm
    bsdf: int = DIFFUSE
    material: int = 0


@dataclass
class Sky:
    """The scene's sky image and sun (Scene::process_globals, Core/Scene.cpp:639-700).

    kind SKY_CUBE_RGBA8: pixels (6, H, W, 4) uint8, faces in the order of the
    scene file's "Skybox" array (+x, -x, +y, -y, +z, -z); SKY_EQUIRECT_RGBAF:
    pixels (H, W, 4) float32 (an HDRI); SKY_CONSTANT: no image (SceneData.sky).
    """
    kind: int = SKY_CONSTANT
    pixels: np.ndarray | None = None
    use_sun: bool = False
    sun_direction: tuple = (0.0, -1.0, 0.0)
    sun_colour: tuple = (1.0, 1.0, 1.0)

    def __post_init__(self):
        if self.kind == SKY_CUBE_RGBA8:
            self.pixels = np.ascontiguousarray(self.pixels, dtype=np.uint8)
            assert self.pixels.ndim == 4 and self.pixels.shape[0] == 6 and self.pixels.shape[3] == 4
        elif self.kind == SKY_EQUIRECT_RGBAF:
            self.pixels = np.ascontiguousarray(self.pixels, dtype=np.float32)
            assert self.pixels.ndim == 3 and self.pixels.shape[2] == 4

    def to_c(self) -> CSky:
        c = CSky()
        c.kind = self.kind
        if self.pixels is not None:
            c.height, c.width = self.pixels.shape[-3], self.pixels.shape[-2]
            c.pixels = self.pixels.ctypes.data
        c.use_sun = int(bool(self.use_sun))
        c.sun_direction[:] = [float(x) for x in self.sun_direction]
        c.sun_colour[:] = [float(x) for x in self.sun_colour]
        return c


@dataclass
class SceneData:
    meshes: list = field(default_factory=list)
    instances: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    sky: tuple = (0.0, 0.0, 0.0)
    sky_image: Sky | None = None


@dataclass
class Camera:
    """Scene::Camera (Core/Camera.hpp:16-29); up defaults to +y as in the reference."""
    position: tuple
    direction: tuple
    resolution: tuple
    aspect: float = 1.0
    up: tuple = (0.0, 1.0, 0.0)
    near_plane: float = 0.1
    far_plane: float = 10000.0
    fov: float = 90.0

    def to_c(self) -> CCamera:
        c = CCamera()
        c.position[:] = [float(x) for x in self.position]
        c.direction[:] = [float(x) for x in self.direction]
        c.up[:] = [float(x) for x in self.up]
        c.resolution[:] = [int(x) for x in self.resolution]
        c.aspect, c.near_plane, c.far_plane, c.fov = self.aspect, self.near_plane, self.far_plane, self.fov
        return c


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else C.POINTER(C.c_float)()


class MarshalledScene:
    """ctypes image of a SceneData; keeps the numpy arrays it points into alive."""

    def __init__(self, scene: SceneData):
        self.keep = []
        n = len(scene.meshes)
        self.meshes = (CMesh * max(n, 1))()
        for i, m in enumerate(scene.meshes):
            cm = self.meshes[i]
            cm.nverts, cm.ntris = len(m.positions), len(m.indices)
            cm.positions, cm.normals = _fptr(m.positions), _fptr(m.normals)
            cm.uvs = _fptr(m.uvs)
            cm.indices = m.indices.ctypes.data_as(C.POINTER(C.c_uint32))
            lo, hi = m.aabb
            cm.aabb_min[:] = [float(x) for x in lo]
            cm.aabb_max[:] = [float(x) for x in hi]
            cm.shape = m.shape
            self.keep.append(m)
        k = len(scene.instances)
        self.instances = (CInstance * max(k, 1))()
        for i, inst in enumerate(scene.instances):
            ci = self.instances[i]
            ci.mesh, ci.bsdf, ci.material = inst.mesh, inst.bsdf, inst.material
            t = np.asarray(inst.transform, dtype=np.float32).reshape(4, 4)
            ci.transform[:] = [float(x) for x in t.reshape(-1)]
        q = len(scene.materials)
        self.materials = (CMaterial * max(q, 1))()
        for i, mat in enumerate(scene.materials):
            cm = self.materials[i]
            cm.diffuse[:] = list(mat.diffuse)
            cm.specular[:] = list(mat.specular)
            cm.roughness = mat.roughness
            cm.emissive[:] = list(mat.emissive)
            cm.index_of_refraction = mat.ior
        self.desc = CSceneDesc()
        self.desc.meshes, self.desc.nmeshes = self.meshes, n
        self.desc.instances, self.desc.ninstances = self.instances, k
        self.desc.materials, self.desc.nmaterials = self.materials, q
        self.desc.sky_rgb[:] = [float(x) for x in scene.sky]
        self.sky = None
        if scene.sky_image is not None:
            self.sky = scene.sky_image.to_c()
            self.keep.append(scene.sky_image)
            self.desc.sky = C.pointer(self.sky)
