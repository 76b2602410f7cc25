"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the rustracer_gb300 package.  Parity
status of the oracle: unpinned (see oracle.h).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
DIAG_LIB_PATH = os.path.join(HERE, "_build", "liboracle_diag.so")

_libs = {}


def build(force=False):
    """Builds liboracle.so and liboracle_diag.so with the committed Makefile."""
    if force or not (os.path.exists(LIB_PATH) and os.path.exists(DIAG_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib(diag=False):
    """The oracle library: the plain build (timed CPU baseline), or with
    diag=True the build with parity diagnostics (branch margins, ulp nudges),
    which renders the same bits when no diagnostics are asked for."""
    if diag not in _libs:
        build()
        L = C.CDLL(DIAG_LIB_PATH if diag else LIB_PATH)
        P = C.c_void_p
        u32, i32 = C.c_uint32, C.c_int
        L.orc_scene_create.restype = P
        L.orc_scene_create.argtypes = [P, u32, P, u32, P, u32, P, u32, P, u32]
        L.orc_scene_destroy.argtypes = [P]
        L.orc_blas_build.argtypes = [P, P, u32]
        L.orc_tlas_build.argtypes = [P, P, u32]
        L.orc_build_flags.argtypes = [P, u32]
        L.orc_lights_set.argtypes = [P, P, u32, P, u32]
        L.orc_skybox_set.argtypes = [P, u32, P]
        L.orc_skybox_set_ex.argtypes = [P, u32, P, u32]
        L.orc_skin.argtypes = [P, P, u32]
        L.orc_get_vertices.argtypes = [P, P, u32]
        L.orc_trace.argtypes = [P, P, u32, u32, P, i32, i32, P]
        L.orc_render.argtypes = [P, P, u32, u32, u32, u32, P, P, P, P, i32, i32, P]
        L.orc_render_diag.argtypes = [P, P, u32, u32, u32, u32, P, P, P, P, P, u32, i32, i32, P]
        L.orc_pcg4d.argtypes = [P, P]
        L.orc_tea.restype = u32
        L.orc_tea.argtypes = [u32, u32]
        L.orc_rand.restype = C.c_float
        L.orc_rand.argtypes = [P]
        L.orc_random_float.restype = C.c_float
        L.orc_random_float.argtypes = [P]
        L.orc_eval_combined_brdf.argtypes = [P, P, P, P, C.c_float, C.c_float, C.c_float, P]
        L.orc_tonemap.argtypes = [u32, P, P]
        L.orc_offset_ray.argtypes = [P, P, P]
        L.orc_sample_texture.argtypes = [P, i32, C.c_float, C.c_float, P]
        L.orc_sample_skybox.argtypes = [P, P, P]
        L.orc_blend_hash.restype = u32
        L.orc_blend_hash.argtypes = [u32, u32, u32]
        _libs[diag] = L
    return _libs[diag]


STATS = np.dtype([("rays_camera", "<u8"), ("rays_extension", "<u8"), ("rays_shadow", "<u8"),
                  ("hits_shaded", "<u8"), ("node_visits", "<u8"), ("tri_tests", "<u8"), ("seconds", "<f8"),
                  ("threads", "<u4"), ("_pad", "<u4")])


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class TexDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32), ("wrap_s", C.c_uint32),
                ("wrap_t", C.c_uint32), ("_pad", C.c_uint32), ("data", C.c_void_p)]


def tex_descs(textures):
    arr = (TexDesc * max(1, len(textures)))()
    keep = []
    for i, (w, h, fmt, ws, wt, data) in enumerate(textures):
        data = np.ascontiguousarray(data)
        keep.append(data)
        arr[i] = TexDesc(w, h, fmt, ws, wt, 0, data.ctypes.data)
    return arr, keep


class OracleScene:
    """The oracle's copy of a SceneData, with its BLAS/TLAS built.  diag=True
    loads it into the diagnostics build (render(want_margins=..., nudge_ulps=...))."""

    def __init__(self, sd, build_flags=0, diag=False):
        L = self.L = lib(diag)
        self.sd = sd
        descs, keep = tex_descs(sd.textures)
        self.h = L.orc_scene_create(_p(sd.vertices), len(sd.vertices), _p(sd.indices), len(sd.indices),
                                    _p(sd.prims), len(sd.prims), _p(sd.materials), len(sd.materials),
                                    C.cast(descs, C.c_void_p), len(sd.textures))
        assert L.orc_blas_build(self.h, _p(sd.geo_ranges), len(sd.geo_ranges)) == 0
        assert L.orc_build_flags(self.h, build_flags) == 0
        assert L.orc_tlas_build(self.h, _p(sd.instances), len(sd.instances)) == 0
        assert L.orc_lights_set(self.h, _p(sd.dlights), len(sd.dlights), _p(sd.plights), len(sd.plights)) == 0
        if sd.skybox is not None:
            size, faces = sd.skybox
            if np.asarray(faces).dtype == np.float32:  # linear RGBA32F faces
                faces = np.ascontiguousarray(faces, np.float32)
                assert L.orc_skybox_set_ex(self.h, size, _p(faces), 3) == 0
            else:
                faces = np.ascontiguousarray(faces, np.uint8)
                assert L.orc_skybox_set(self.h, size, _p(faces)) == 0

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_scene_destroy(self.h)
            self.h = None

    def tlas(self, instances):
        """New instances (orc_tlas_build): the oracle builds its TLAS, and its
        world BVH where instances are flattened, from scratch."""
        instances = np.ascontiguousarray(instances)
        assert self.L.orc_tlas_build(self.h, _p(instances), len(instances)) == 0
        self._instances = instances

    def skin(self, skins):
        skins = np.ascontiguousarray(skins)
        assert self.L.orc_skin(self.h, _p(skins), len(skins)) == 0

    def vertices(self):
        out = np.zeros_like(self.sd.vertices)
        assert self.L.orc_get_vertices(self.h, _p(out), len(out)) == 0
        return out

    def trace(self, rays, flags=0, fp64=False, threads=0):
        from rustracer_gb300 import types as T
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(len(rays), T.HIT)
        st = np.zeros((), STATS)
        assert self.L.orc_trace(self.h, _p(rays), len(rays), flags, _p(hits), int(fp64), threads, _p(st)) == 0
        return hits, st

    def render(self, ubo, width, height, rows=None, accum=None, want_samples=False, want_hits=False,
               fp64=False, threads=0, out=True, want_margins=False, nudge_ulps=0, nudge_draw=0):
        """Renders rows [row0, row1) (all by default).  want_margins adds
        'margins' [pixel][sample][2] (smallest branch-decision margin,
        smallest secondary-hit barycentric); nudge_ulps > 0 moves every
        transcendental, shading division and square root, dot product and
        normalised vector by that many ulps with signs of draw `nudge_draw`
        (orc_render_diag)."""
        from rustracer_gb300 import types as T
        assert 0 <= nudge_ulps < 1 << 16 and 0 <= nudge_draw < 1 << 16
        ns = int(ubo["number_of_samples"])
        row0, row1 = rows if rows is not None else (0, height)
        img = np.zeros((height, width, 4), np.uint8) if out else None
        samples = np.zeros((height * width, ns, 3), np.float32) if want_samples else None
        hits = np.zeros((height * width, ns), T.HIT) if want_hits else None
        margins = np.full((height * width, ns, 2), np.inf, np.float32) if want_margins else None
        st = np.zeros((), STATS)
        ubo = np.ascontiguousarray(ubo)
        rc = self.L.orc_render_diag(self.h, _p(ubo), width, height, row0, row1, _p(accum), _p(img), _p(samples),
                                   _p(hits), _p(margins), int(nudge_ulps) | (int(nudge_draw) << 16), int(fp64),
                                   threads, _p(st))
        assert rc == 0, rc
        return dict(image=img, samples=samples, hits=hits, stats=st, margins=margins)


# --- shader-library entry points ----------------------------------------
def pcg4d(v):
    a = np.asarray(v, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_pcg4d(_p(a), _p(out))
    return out


def tea(a, b):
    return lib().orc_tea(a, b)


def rand_sequence(state, n):
    st = np.asarray(state, np.uint32).copy()
    return np.array([lib().orc_rand(_p(st)) for _ in range(n)], np.float32), st


def random_float_sequence(seed, n):
    s = np.array([seed], np.uint32)
    return np.array([lib().orc_random_float(_p(s)) for _ in range(n)], np.float32)


def eval_combined_brdf(N, L, V, base_color, metallic, roughness, ior=1.5):
    a = [np.asarray(x, np.float32) for x in (N, L, V, base_color)]
    out = np.zeros(3, np.float32)
    lib().orc_eval_combined_brdf(*[_p(x) for x in a], metallic, roughness, ior, _p(out))
    return out


def tonemap(mode, rgb):
    a = np.asarray(rgb, np.float32)
    out = np.zeros(3, np.float32)
    lib().orc_tonemap(mode, _p(a), _p(out))
    return out


def offset_ray(p, n):
    a, b = np.asarray(p, np.float32), np.asarray(n, np.float32)
    out = np.zeros(3, np.float32)
    lib().orc_offset_ray(_p(a), _p(b), _p(out))
    return out


def blend_hash(instance, prim, tag):
    return lib().orc_blend_hash(instance, prim, tag)
