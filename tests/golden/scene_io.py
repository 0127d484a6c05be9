"""Save and load SceneData and cameras inside .npz fixtures (exact float32 bits)."""
from __future__ import annotations

import numpy as np

from pico_gb300.types import Camera, Instance, Material, Mesh, SceneData, Sky


def scene_arrays(scene: SceneData, prefix: str = "scene") -> dict:
    out = {f"{prefix}_nmeshes": np.array(len(scene.meshes))}
    for i, m in enumerate(scene.meshes):
        out[f"{prefix}_m{i}_pos"] = m.positions
        out[f"{prefix}_m{i}_nrm"] = m.normals
        out[f"{prefix}_m{i}_idx"] = m.indices
        if m.shape:
            out[f"{prefix}_m{i}_shape"] = np.array(m.shape)
    out[f"{prefix}_inst_meta"] = np.array([[i.mesh, i.bsdf, i.material] for i in scene.instances], np.uint32)
    out[f"{prefix}_inst_xf"] = np.stack([np.asarray(i.transform, np.float32).reshape(4, 4)
                                         for i in scene.instances])
    out[f"{prefix}_mats"] = np.array([[*m.diffuse, *m.specular, m.roughness, *m.emissive, m.ior]
                                      for m in scene.materials], np.float32)
    out[f"{prefix}_sky"] = np.array(scene.sky, np.float32)
    if scene.sky_image is not None:
        out.update(sky_arrays(scene.sky_image, f"{prefix}_skyimg"))
    return out


def sky_arrays(sky: Sky, prefix: str) -> dict:
    out = {f"{prefix}_kind": np.array(sky.kind), f"{prefix}_sun": np.array(int(sky.use_sun)),
           f"{prefix}_sun_dir": np.array(sky.sun_direction, np.float32),
           f"{prefix}_sun_col": np.array(sky.sun_colour, np.float32)}
    if sky.pixels is not None:
        out[f"{prefix}_pixels"] = sky.pixels
    return out


def load_sky(z, prefix: str) -> Sky:
    px = z[f"{prefix}_pixels"] if f"{prefix}_pixels" in z else None
    return Sky(int(z[f"{prefix}_kind"]), px, bool(int(z[f"{prefix}_sun"])), tuple(z[f"{prefix}_sun_dir"]),
               tuple(z[f"{prefix}_sun_col"]))


def load_scene(z, prefix: str = "scene") -> SceneData:
    n = int(z[f"{prefix}_nmeshes"])
    meshes = [Mesh(z[f"{prefix}_m{i}_pos"], z[f"{prefix}_m{i}_nrm"], z[f"{prefix}_m{i}_idx"],
                   shape=int(z[f"{prefix}_m{i}_shape"]) if f"{prefix}_m{i}_shape" in z else 0) for i in range(n)]
    insts = [Instance(int(a), x, int(b), int(c)) for (a, b, c), x in zip(z[f"{prefix}_inst_meta"], z[f"{prefix}_inst_xf"])]
    mats = [Material(tuple(r[0:3]), tuple(r[3:6]), float(r[6]), tuple(r[7:10]), float(r[10]) if len(r) > 10 else 0.0)
            for r in z[f"{prefix}_mats"]]
    sky = load_sky(z, f"{prefix}_skyimg") if f"{prefix}_skyimg_kind" in z else None
    return SceneData(meshes, insts, mats, tuple(z[f"{prefix}_sky"]), sky)


def camera_array(cam: Camera) -> np.ndarray:
    return np.array([*cam.position, *cam.direction, *cam.up, *cam.resolution, cam.aspect, cam.near_plane,
                     cam.far_plane, cam.fov], np.float64)


def load_camera(a) -> Camera:
    a = np.asarray(a, np.float64)
    return Camera(position=tuple(a[0:3]), direction=tuple(a[3:6]), up=tuple(a[6:9]),
                  resolution=(int(a[9]), int(a[10])), aspect=float(a[11]), near_plane=float(a[12]),
                  far_plane=float(a[13]), fov=float(a[14]))
