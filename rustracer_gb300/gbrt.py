"""ctypes binding of libgbrt.so (include/gbrt.h) and a thin host layer that
mirrors the reference's render-frame API.

The reference's per-frame path (crates/examples/gltf_viewer/src/main.rs) is:
``create_as`` (BLAS per geometry + TLAS, acceleration_structures.rs:79-129),
``create_top_as`` (TLAS only, :136-249), a UBO upload and ``trace_rays``
(main.rs:215-270) into an accumulation image.  :class:`Renderer` exposes the
same steps (``create_as``, ``create_top_as``, ``update_lights``,
``render``) on top of the C ABI.  Failures raise :class:`GbrtError` carrying
the library's status code and message (the reference panics/propagates
``anyhow`` errors instead).

There is no CPU fallback: if libgbrt.so or a CUDA device is missing, calls
raise.
"""
import ctypes as C
import os

import numpy as np

from . import types as T

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libgbrt.so")

OK, E_INVALID, E_CUDA, E_OOM, E_DEVICE_LIMIT, E_NOT_BUILT, E_NO_DEVICE, E_BUSY = 0, -1, -2, -3, -4, -5, -6, -7
E_CANCELLED = -8
INJECT_ADMIT_OOM = 1
BUILD_NO_FLATTEN = 0x1
BUILD_WIDTH4 = 0x2
MODE_AUTO, MODE_MEGAKERNEL, MODE_WAVEFRONT = 0, 1, 2
RENDER_STAGE_TIMING, RENDER_ASYNC = 0x1, 0x2

# name -> (restype, argtypes); every symbol include/gbrt.h declares
P, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
SIGNATURES = {
    "gbrt_version": (C.c_char_p, []),
    "gbrt_last_error": (C.c_char_p, [P]),
    "gbrt_ctx_create": (i32, [i32, C.POINTER(P)]),
    "gbrt_ctx_destroy": (i32, [P]),
    "gbrt_ctx_mem_info": (i32, [P, C.POINTER(u64), C.POINTER(u64)]),
    "gbrt_sync": (i32, [P]),
    "gbrt_scene_create": (i32, [P, P, u32, P, u32, P, u32, P, u32, P, u32, C.POINTER(P)]),
    "gbrt_scene_destroy": (i32, [P]),
    "gbrt_blas_build": (i32, [P, P, u32, u32]),
    "gbrt_tlas_build": (i32, [P, P, u32]),
    "gbrt_tlas_update": (i32, [P, P, u32]),
    "gbrt_skin_and_refit": (i32, [P, P, u32]),
    "gbrt_lights_set": (i32, [P, P, u32, P, u32]),
    "gbrt_skybox_set": (i32, [P, u32, P]),
    "gbrt_skybox_set_ex": (i32, [P, u32, P, u32]),
    "gbrt_accum_create": (i32, [P, u32, u32, C.POINTER(P)]),
    "gbrt_accum_reset": (i32, [P]),
    "gbrt_accum_download": (i32, [P, P]),
    "gbrt_accum_upload": (i32, [P, P]),
    "gbrt_accum_destroy": (i32, [P]),
    "gbrt_render": (i32, [P, P, P, P, P]),
    "gbrt_render_ex": (i32, [P, P, P, P, P, P]),
    "gbrt_trace_rays": (i32, [P, P, u32, u32, P, P]),
    "gbrt_trace_rays_device": (i32, [P, P, u32, u32, P]),
    "gbrt_device_alloc": (i32, [P, u64, C.POINTER(P)]),
    "gbrt_device_free": (i32, [P, P]),
    "gbrt_memcpy_h2d": (i32, [P, P, P, u64]),
    "gbrt_memcpy_d2h": (i32, [P, P, P, u64]),
    "gbrt_timer_begin": (i32, [P]),
    "gbrt_timer_end": (i32, [P, C.POINTER(C.c_double)]),
    "gbrt_scene_rebuild_noalloc": (i32, [P, P]),
    "gbrt_job_submit": (i32, [P, P, C.POINTER(u64)]),
    "gbrt_job_poll": (i32, [P, u64, P]),
    "gbrt_job_wait": (i32, [P, u64, u32, P]),
    "gbrt_job_cancel": (i32, [P, u64]),
    "gbrt_jobs_inject": (i32, [P, u32, u32]),
    "gbrt_jobs_configure": (i32, [P, u64, u32]),
    "gbrt_nrc_create": (i32, [P, P, C.POINTER(P)]),
    "gbrt_nrc_destroy": (i32, [P]),
    "gbrt_nrc_params": (i32, [P, P, P, i32]),
    "gbrt_nrc_query": (i32, [P, P, u32, P]),
    "gbrt_nrc_query_device": (i32, [P, P, u32, P, P]),
    "gbrt_nrc_train": (i32, [P, P, P, u32, i32, P, P, P]),
    "gbrt_render_nrc": (i32, [P, P, P, P, P, P, P, P]),
    "gbrt_scene_autotune": (i32, [P, P, u32, u32, P]),
    "gbrt_scene_set_tuning": (i32, [P, u32, u32]),
    "gbrt_scene_info_get": (i32, [P, P]),
}
JOB_QUEUED, JOB_RUNNING, JOB_DONE = 0, 1, 2
POLICY_SRPT, POLICY_FIFO = 0, 1
JOB_LARGE_WAVES = 0x100  # OR into the policy before the first submit: waves up to 2^26 paths
NOALLOC_MAX_TRIANGLES = 65536


class GbrtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbrt error {code}: {msg}")
        self.code = code


_lib = None


def load(path=LIB_PATH):
    """Loads libgbrt.so (building it first if absent) and binds SIGNATURES."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            from . import build
            build.build()
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class TexDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32), ("wrap_s", C.c_uint32),
                ("wrap_t", C.c_uint32), ("_pad", C.c_uint32), ("data", C.c_void_p)]


class RenderOpts(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("flags", C.c_uint32), ("sample_radiance", C.c_void_p),
                ("primary_hits", C.c_void_p)]


class JobDesc(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("ubo", C.c_void_p), ("accum", C.c_void_p), ("out_rgba8", C.c_void_p),
                ("skins", C.c_void_p), ("nskin", C.c_uint32), ("flags", C.c_uint32), ("cache", C.c_void_p),
                ("cache_opts", C.c_void_p)]


class Context:
    """gbrt_ctx: one CUDA device + stream."""

    def __init__(self, device=0):
        self.L = load()
        h = P()
        rc = self.L.gbrt_ctx_create(device, C.byref(h))
        if rc != OK:
            raise GbrtError(rc, self.L.gbrt_last_error(None).decode())
        self.h = h

    def check(self, rc):
        if rc != OK:
            raise GbrtError(rc, self.L.gbrt_last_error(self.h).decode())

    def mem_info(self):
        f, t = u64(), u64()
        self.check(self.L.gbrt_ctx_mem_info(self.h, C.byref(f), C.byref(t)))
        return f.value, t.value

    def sync(self):
        self.check(self.L.gbrt_sync(self.h))

    # -- jobs (asynchronous frames, continuous batching) ----------------------
    def jobs_configure(self, hbm_budget=0, policy=POLICY_SRPT):
        self.check(self.L.gbrt_jobs_configure(self.h, hbm_budget, policy))

    def jobs_inject(self, kind, count):
        """gbrt_jobs_inject: host-side fault injection (INJECT_ADMIT_OOM)."""
        self.check(self.L.gbrt_jobs_inject(self.h, kind, count))

    def submit(self, scene, ubo, accum, image=True, skins=None, cache=None, min_roughness=0.0,
               train_samples=1 << 16, train_steps=1, cache_mode=0):
        """Queues one frame of `scene` into `accum` (through the radiance
        cache `cache`, an Nrc, when given); returns a Job."""
        return Job(self, scene, ubo, accum, image, skins, cache,
                   None if cache is None else NrcRenderOpts(min_roughness, train_samples, train_steps, 0, cache_mode))

    def close(self):
        if getattr(self, "h", None):
            self.L.gbrt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Job:
    """A submitted frame: ``wait()`` returns its info (state, status, queue
    and end-to-end latency in ms, stats) and fills ``image``."""

    def __init__(self, ctx, scene, ubo, accum, image=True, skins=None, cache=None, cache_opts=None):
        self.ctx = ctx
        self._ubo = np.asarray(ubo, T.UBO).reshape(())
        self.image = np.zeros((accum.h_, accum.w, 4), np.uint8) if image else None
        self._skins = None if skins is None else np.ascontiguousarray(skins, T.SKIN)
        self._copts = cache_opts
        d = JobDesc(scene.h, self._ubo.ctypes.data, accum.h,
                    self.image.ctypes.data if image else None,
                    self._skins.ctypes.data if self._skins is not None else None,
                    0 if self._skins is None else len(self._skins), 0,
                    cache.h if cache is not None else None,
                    C.addressof(cache_opts) if cache_opts is not None else None)
        jid = u64()
        ctx.check(ctx.L.gbrt_job_submit(ctx.h, C.byref(d), C.byref(jid)))
        self.id = jid.value
        self.info = None

    def _finish(self, rc, info):
        if rc == E_BUSY:
            return None
        self.info = {"state": int(info["state"]), "status": int(info["status"]),
                     "queue_ms": float(info["queue_ms"]), "latency_ms": float(info["latency_ms"]),
                     "stats": info["stats"].copy()}
        self.ctx.check(rc)
        return self.info

    def cancel(self):
        """gbrt_job_cancel."""
        self.ctx.check(self.ctx.L.gbrt_job_cancel(self.ctx.h, self.id))

    def poll(self):
        if self.info is not None:
            return self.info
        info = np.zeros((), T.JOB_INFO)
        return self._finish(self.ctx.L.gbrt_job_poll(self.ctx.h, self.id, _p(info)), info)

    def wait(self, timeout_ms=0xFFFFFFFF):
        if self.info is not None:
            return self.info
        info = np.zeros((), T.JOB_INFO)
        return self._finish(self.ctx.L.gbrt_job_wait(self.ctx.h, self.id, timeout_ms, _p(info)), info)


class NrcConfig(C.Structure):
    _fields_ = [("log2_table", C.c_uint32), ("base_resolution", C.c_uint32), ("growth", C.c_float),
                ("learning_rate", C.c_float), ("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3),
                ("seed", C.c_uint64), ("flags", C.c_uint32), ("_pad", C.c_uint32)]


NRC_QUERY_MMA_SYNC = 0x1
NRC_TRAIN_FP32 = 0x2
NRC_MODE_SUFFIX = 0
NRC_MODE_PRIMARY_INDIRECT = 1


class NrcRenderOpts(C.Structure):
    _fields_ = [("min_roughness", C.c_float), ("train_samples", C.c_uint32), ("train_steps", C.c_uint32),
                ("disabled", C.c_uint32), ("mode", C.c_uint32)]


class Nrc:
    """gbrt_nrc: the neural radiance cache (hash grid + 5x64 MLP)."""
    MLP_PARAMS = 18624

    def __init__(self, ctx, box_lo, box_hi, log2_table=19, base_resolution=16, growth=1.447, learning_rate=1e-2,
                 seed=1, flags=0):
        self.ctx = ctx
        self.cfg = NrcConfig(log2_table, base_resolution, growth, learning_rate, (C.c_float * 3)(*box_lo),
                             (C.c_float * 3)(*box_hi), seed, flags, 0)
        h = P()
        ctx.check(ctx.L.gbrt_nrc_create(ctx.h, C.byref(self.cfg), C.byref(h)))
        self.h = h
        self.grid_size = 16 * (1 << log2_table) * 2

    def params(self):
        mlp = np.zeros(self.MLP_PARAMS, np.float32)
        grid = np.zeros(self.grid_size, np.float32)
        self.ctx.check(self.ctx.L.gbrt_nrc_params(self.h, _p(mlp), _p(grid), 0))
        return mlp, grid

    def set_params(self, mlp=None, grid=None):
        m = None if mlp is None else np.ascontiguousarray(mlp, np.float32)
        g = None if grid is None else np.ascontiguousarray(grid, np.float32)
        self.ctx.check(self.ctx.L.gbrt_nrc_params(self.h, _p(m) if m is not None else None,
                                                  _p(g) if g is not None else None, 1))

    def query(self, pos):
        q = np.zeros((len(pos), 4), np.float32)
        q[:, :3] = pos
        out = np.zeros_like(q)
        self.ctx.check(self.ctx.L.gbrt_nrc_query(self.h, _p(q), len(q), _p(out)))
        return out[:, :3]

    def query_device(self, pos4_ptr, n, out4_ptr):
        """Queries on device buffers of n float4 (e.g. tensor.data_ptr()); returns the device ms."""
        ms = C.c_float(0)
        self.ctx.check(self.ctx.L.gbrt_nrc_query_device(self.h, C.c_void_p(pos4_ptr), n, C.c_void_p(out4_ptr),
                                                        C.byref(ms)))
        return ms.value

    def train(self, pos, target, step=True, grads=False):
        q = np.zeros((len(pos), 4), np.float32)
        q[:, :3] = pos
        t = np.zeros((len(pos), 4), np.float32)
        t[:, :3] = np.asarray(target)[:, :3]
        loss = np.zeros(1, np.float32)
        gm = np.zeros(self.MLP_PARAMS, np.float32) if grads else None
        gg = np.zeros(self.grid_size, np.float32) if grads else None
        self.ctx.check(self.ctx.L.gbrt_nrc_train(self.h, _p(q), _p(t), len(q), int(step), _p(loss),
                                                 _p(gm) if grads else None, _p(gg) if grads else None))
        return (float(loss[0]), gm, gg) if grads else float(loss[0])

    def render(self, scene, ubo, accum, image=True, min_roughness=0.0, train_samples=1 << 16, train_steps=1,
               disabled=False, mode=NRC_MODE_SUFFIX):
        """One frame with the cache (gbrt_render_nrc); returns dict(image, stats, loss)."""
        ubo = np.asarray(ubo, T.UBO).reshape(())
        img = np.zeros((accum.h_, accum.w, 4), np.uint8) if image else None
        st = np.zeros((), T.STATS)
        loss = np.zeros(1, np.float32)
        opts = NrcRenderOpts(min_roughness, train_samples, train_steps, int(disabled), mode)
        self.ctx.check(self.ctx.L.gbrt_render_nrc(scene.h, self.h, _p(ubo), accum.h, _p(img) if image else None,
                                                  _p(st), C.byref(opts), _p(loss)))
        return dict(image=img, stats=st, loss=float(loss[0]))

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.L.gbrt_nrc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Accum:
    """gbrt_accum: device RGBA32F running sum (the reference's acc_image)."""

    def __init__(self, ctx, width, height):
        self.ctx, self.w, self.h_ = ctx, width, height
        h = P()
        ctx.check(ctx.L.gbrt_accum_create(ctx.h, width, height, C.byref(h)))
        self.h = h

    def reset(self):
        self.ctx.check(self.ctx.L.gbrt_accum_reset(self.h))

    def download(self):
        out = np.zeros((self.h_, self.w, 4), np.float32)
        self.ctx.check(self.ctx.L.gbrt_accum_download(self.h, _p(out)))
        return out

    def upload(self, rgba32f):
        """gbrt_accum_upload: restore a running sum saved with download() (checkpoint / resume)."""
        a = np.ascontiguousarray(rgba32f, np.float32).reshape(self.h_, self.w, 4)
        self.ctx.check(self.ctx.L.gbrt_accum_upload(self.h, _p(a)))

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.L.gbrt_accum_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Scene:
    """gbrt_scene created from a scenes.SceneData (the reference's Buffers +
    textures), with create_as / create_top_as like
    crates/libs/asset_loader/src/acceleration_structures.rs."""

    def __init__(self, ctx, sd, build=True, build_flags=0):
        self.ctx, self.sd = ctx, sd
        self.build_flags = build_flags
        L = ctx.L
        descs = (TexDesc * max(1, len(sd.textures)))()
        self._keep = []
        for i, (w, h, fmt, ws, wt, data) in enumerate(sd.textures):
            data = np.ascontiguousarray(data)
            self._keep.append(data)
            descs[i] = TexDesc(w, h, fmt, ws, wt, 0, data.ctypes.data)
        h = P()
        ctx.check(L.gbrt_scene_create(ctx.h, _p(sd.vertices), len(sd.vertices), _p(sd.indices), len(sd.indices),
                                      _p(sd.prims), len(sd.prims), _p(sd.materials), len(sd.materials),
                                      C.cast(descs, P), len(sd.textures), C.byref(h)))
        self.h = h
        if build:
            self.create_as()
            self.update_lights(sd.dlights, sd.plights)
            if sd.skybox is not None:
                self.set_skybox(*sd.skybox)

    def create_as(self, ranges=None, instances=None):
        """BLAS per geometry, then the TLAS (create_as, acceleration_structures.rs:79-129)."""
        ranges = self.sd.geo_ranges if ranges is None else ranges
        self.ctx.check(self.ctx.L.gbrt_blas_build(self.h, _p(ranges), len(ranges), self.build_flags))
        self.create_top_as(instances)

    def create_top_as(self, instances=None):
        """TLAS only (create_top_as, acceleration_structures.rs:136-249)."""
        inst = self.sd.instances if instances is None else np.ascontiguousarray(instances, T.INSTANCE)
        self.ctx.check(self.ctx.L.gbrt_tlas_build(self.h, _p(inst), len(inst)))

    def update_tlas(self, instances):
        inst = np.ascontiguousarray(instances, T.INSTANCE)
        self.ctx.check(self.ctx.L.gbrt_tlas_update(self.h, _p(inst), len(inst)))

    def skin_and_refit(self, skins):
        skins = np.ascontiguousarray(skins, T.SKIN)
        self.ctx.check(self.ctx.L.gbrt_skin_and_refit(self.h, _p(skins), len(skins)))

    def rebuild_noalloc(self, d_vertices=None):
        """Allocation-free rebuild of the world BVH (gbrt_scene_rebuild_noalloc);
        d_vertices is a device pointer (int) to a full replacement vertex array,
        or None to rebuild from the current vertices."""
        self.ctx.check(self.ctx.L.gbrt_scene_rebuild_noalloc(self.h, None if d_vertices is None else P(d_vertices)))

    def update_lights(self, dlights, plights):
        d = np.ascontiguousarray(dlights, T.LIGHT)
        p = np.ascontiguousarray(plights, T.LIGHT)
        self.ctx.check(self.ctx.L.gbrt_lights_set(self.h, _p(d), len(d), _p(p), len(p)))

    def set_skybox(self, size, faces):
        """6 faces of size^2 texels: uint8 RGBA (sRGB) or float32 RGBA (linear, HDR)."""
        if faces is not None and np.asarray(faces).dtype == np.float32:
            faces = np.ascontiguousarray(faces, np.float32)
            self.ctx.check(self.ctx.L.gbrt_skybox_set_ex(self.h, size, _p(faces), T.TEX_RGBA32F))
            return
        faces = None if faces is None else np.ascontiguousarray(faces, np.uint8)
        self.ctx.check(self.ctx.L.gbrt_skybox_set(self.h, size, _p(faces)))

    def autotune(self, ubo, width, height):
        """gbrt_scene_autotune: picks the fastest BVH layout (binary, 4- or
        8-wide) and whether to group extension rays by octant; returns
        dict(ms_binary, ms_wide, ms_wide4, ms_sorted, chosen_width, sort_rays)."""
        rep = np.zeros(5, np.float64)
        ubo = np.asarray(ubo, T.UBO).reshape(())
        self.ctx.check(self.ctx.L.gbrt_scene_autotune(self.h, _p(ubo), width, height, _p(rep)))
        u = rep[4:].view(np.uint32)
        return dict(ms_binary=float(rep[0]), ms_wide=float(rep[1]), ms_wide4=float(rep[2]),
                    ms_sorted=float(rep[3]), chosen_width=int(u[0]), sort_rays=int(u[1]))

    def info(self):
        """gbrt_scene_info_get: world BVH sizes, refit count, drift rebuilds, incremental instance
        updates and SAH cost proxies."""
        raw = np.zeros(5, np.float64)
        self.ctx.check(self.ctx.L.gbrt_scene_info_get(self.h, _p(raw)))
        u = raw[:3].view(np.uint32)
        return dict(world_triangles=int(u[0]), wide_nodes=int(u[1]), wide_width=int(u[2]), refits=int(u[3]),
                    drift_rebuilds=int(u[4]), instance_updates=int(u[5]), sah_built=float(raw[3]),
                    sah_now=float(raw[4]))

    def set_tuning(self, width=8, sort_rays=False):
        """gbrt_scene_set_tuning: BVH width 2/4/8 and the ray-sort key, set directly."""
        self.ctx.check(self.ctx.L.gbrt_scene_set_tuning(self.h, width, int(bool(sort_rays))))

    def render(self, ubo, accum, image=True, mode=MODE_AUTO, want_samples=False, want_hits=False,
               asynchronous=False, out=None):
        """One frame (record_raytracing_commands + the shaders).  Returns a dict
        with 'image' (HxWx4 uint8 or None), 'stats', and the optional
        per-sample radiance [pixel][sample][3] and primary hits.  With
        asynchronous=True the frame is only queued (GBRT_RENDER_ASYNC): the
        image (written into `out` when given) is valid after ctx.sync()."""
        ubo = np.asarray(ubo, T.UBO).reshape(())
        W, H = accum.w, accum.h_
        ns = int(ubo["number_of_samples"])
        img = (out if out is not None else np.zeros((H, W, 4), np.uint8)) if image else None
        st = np.zeros((), T.STATS)
        samples = np.zeros((H * W, ns, 3), np.float32) if want_samples else None
        hits = np.zeros((H * W, ns), T.HIT) if want_hits else None
        opts = RenderOpts(mode, RENDER_ASYNC if asynchronous else 0, samples.ctypes.data if want_samples else None,
                          hits.ctypes.data if want_hits else None)
        self.ctx.check(self.ctx.L.gbrt_render_ex(self.h, _p(ubo), accum.h, _p(img), _p(st), C.byref(opts)))
        return dict(image=img, stats=st, samples=samples, hits=hits)

    def trace(self, rays, flags=0):
        rays = np.ascontiguousarray(rays, T.RAY)
        hits = np.zeros(len(rays), T.HIT)
        st = np.zeros((), T.STATS)
        self.ctx.check(self.ctx.L.gbrt_trace_rays(self.h, _p(rays), len(rays), flags, _p(hits), _p(st)))
        return hits, st

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.L.gbrt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Renderer:
    """The reference's GltfViewer render-frame loop on the C ABI: owns a
    scene and an accumulation buffer and accumulates samples frame after
    frame (main.rs:189-270; reset on change, main.rs:336-353)."""

    def __init__(self, ctx, sd, width, height):
        self.ctx, self.sd = ctx, sd
        self.scene = Scene(ctx, sd)
        self.accum = Accum(ctx, width, height)
        self.width, self.height = width, height
        self.total_number_of_samples = 0

    def reset_samples(self):
        self.total_number_of_samples = 0
        self.accum.reset()

    def frame(self, samples=3, **ubo_kw):
        self.total_number_of_samples += samples
        ubo = self.sd.ubo(self.width, self.height, samples=samples, total=self.total_number_of_samples, **ubo_kw)
        return self.scene.render(ubo, self.accum)
