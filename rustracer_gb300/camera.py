"""Camera matrices and the per-frame UBO, as the reference computes them.

* view = look_at_rh(position, position + direction, +y)
  (crates/libs/app/src/camera.rs:98-104, nalgebra Matrix4::look_at_rh)
* projection = OPENGL_TO_VULKAN_RT * perspective(aspect, fovy, near, far)
  (camera.rs:106-118, nalgebra Matrix4::new_perspective)
* UBO fill: crates/examples/gltf_viewer/src/main.rs:197-237 (inverses, random
  seed 3, fov_angle 1.0, GUI defaults from gui_state.rs:303-331).

Matrices are computed in float64 and stored float32 column-major.
"""
import math

import numpy as np

from .types import UBO

OPENGL_TO_VULKAN_RT = np.array([[1, 0, 0, 0], [0, -1, 0, 0], [0, 0, 0.5, 0.5], [0, 0, 0, 1]], np.float64)


def look_at_rh(eye, target, up):
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[0, 3] = -s @ eye
    m[1, 3] = -u @ eye
    m[2, 3] = f @ eye
    return m


def perspective(aspect, fovy_rad, znear, zfar):
    t = 1.0 / math.tan(fovy_rad / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = t / aspect
    m[1, 1] = t
    m[2, 2] = (zfar + znear) / (znear - zfar)
    m[2, 3] = 2.0 * zfar * znear / (znear - zfar)
    m[3, 2] = -1.0
    return m


def colmajor(m):
    return np.asarray(m, np.float64).T.reshape(16).astype(np.float32)


def make_ubo(width, height, eye, direction, fov_deg=60.0, znear=0.1, zfar=10.0, *, samples=1, total=None,
             bounces=5, aperture=0.0, focus_distance=10.0, antialiasing=True, has_sky=False, exposure=5.0,
             tone_mapping_mode=0, mapping=0, fully_opaque=False, debug=0, orthographic_fov_dis=0.0,
             heatmap_scale=1.0, frame_count=0):
    """One UniformBufferObject.  Defaults are the reference GUI's
    (gui_state.rs:303-331): 5 bounces, exposure 5, AA on, sky off, aperture 0,
    focus distance 10.  total defaults to samples (first frame)."""
    eye = np.asarray(eye, np.float64)
    view = look_at_rh(eye, eye + np.asarray(direction, np.float64), (0, 1, 0))
    proj = OPENGL_TO_VULKAN_RT @ perspective(width / height, math.radians(fov_deg), znear, zfar)
    u = np.zeros((), UBO)
    u["model_view"] = colmajor(view)
    u["projection"] = colmajor(proj)
    u["model_view_inverse"] = colmajor(np.linalg.inv(view))
    u["projection_inverse"] = colmajor(np.linalg.inv(proj))
    u["aperture"] = aperture
    u["focus_distance"] = focus_distance
    u["fov_angle"] = 1.0
    u["orthographic_fov_dis"] = orthographic_fov_dis
    u["heatmap_scale"] = heatmap_scale
    u["total_number_of_samples"] = samples if total is None else total
    u["number_of_samples"] = samples
    u["number_of_bounces"] = bounces
    u["random_seed"] = 3
    u["has_sky"] = int(has_sky)
    u["antialiasing"] = int(antialiasing)
    u["mapping"] = mapping
    u["frame_count"] = frame_count
    u["debug"] = debug
    u["fully_opaque"] = int(fully_opaque)
    u["exposure"] = exposure
    u["tone_mapping_mode"] = tone_mapping_mode
    return u
