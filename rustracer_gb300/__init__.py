"""rustracer_gb300 — GB300-native ray-tracing core with rustracer's behaviour.

The compute path is libgbrt.so (CUDA, sm_103a) behind the C ABI in
include/gbrt.h; this package holds its Python host side: ctypes bindings
(gbrt.py), the reference's device data layouts (types.py), camera/UBO math
(camera.py), seeded scene generators (scenes.py) and the build step
(build.py).
"""
from . import types, camera, scenes  # noqa: F401
