"""ctypes binding of libqbcuda (include/qbcuda.h).

The library is the product; this module only declares its C signatures and
turns a negative status into QbcError. There is no fallback: if the shared
library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

c_float_p = C.POINTER(C.c_float)
c_int32_p = C.POINTER(C.c_int32)
c_int64_p = C.POINTER(C.c_int64)

QBC_GL_INT = 0x1404
QBC_GL_FLOAT = 0x1406

STATIC_COLOR, STATIC_NORMAL, STATIC_OCTREE, DYNAMIC_COLOR, DYNAMIC_NORMAL, DYNAMIC_OCTREE = range(6)
MAX_LEVEL = 17
NOALLOC_MAX_VIEWS = 256

PX_PRIMARY_LEAF = 1 << 0
PX_DISCARD = 1 << 1
PX_SHADED = 1 << 2
PX_SHADOW_LEAF = 1 << 3
PX_LIT = 1 << 4
PX_FLARE_TEST = 1 << 5
PX_FLARE_WHITE = 1 << 6
PX_OOB = 1 << 7

SCENE_FLOOR = 0
SCENE_ROOM = 1
SCENE_HOUSE = 2

ERRORS = {-1: "QBC_E_ARG", -2: "QBC_E_CUDA", -3: "QBC_E_NOMEM", -4: "QBC_E_STATE", -5: "QBC_E_TIMEOUT", -6: "QBC_E_IO"}


class QbcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class View(C.Structure):
    """qbc_view: the uniforms of one frame."""

    _fields_ = [
        ("camfp", C.c_float * 3),
        ("light", C.c_float * 3),
        ("basecube", C.c_float * 4),
        ("dim", C.c_float * 2),
        ("cfp", C.c_float * 3),
        ("qz", C.c_float * 4),
        ("qx", C.c_float * 4),
        ("ncamlight", C.c_float * 3),
        ("flare_cos", C.c_float),
        ("coord_scale", C.c_float * 2),
        ("width_px", C.c_int32),
        ("height_px", C.c_int32),
        ("maxlevel", C.c_int32),
        ("shoot", C.c_int32),
    ]

    def to_bytes(self) -> bytes:
        return bytes(memoryview(self).cast("B"))

    @classmethod
    def from_bytes(cls, b: bytes) -> "View":
        v = cls()
        C.memmove(C.addressof(v), b, C.sizeof(cls))
        return v


class Outputs(C.Structure):
    """qbc_outputs: per-view output pointers (host or device)."""

    _fields_ = [
        ("rgba8", C.c_void_p),
        ("rgba32f", C.c_void_p),
        ("flags", C.c_void_p),
        ("leaf", C.c_void_p),
        ("isp", C.c_void_p),
        ("visits", C.c_void_p),
    ]


class RayHits(C.Structure):
    """qbc_ray_hits: per-ray output pointers (host or device)."""

    _fields_ = [
        ("status", C.c_void_p),
        ("leaf", C.c_void_p),
        ("model", C.c_void_p),
        ("isp", C.c_void_p),
        ("col", C.c_void_p),
        ("nrm", C.c_void_p),
        ("visits", C.c_void_p),
    ]


class RenderOpts(C.Structure):
    """qbc_render_opts."""

    _fields_ = [
        ("two_pass", C.c_int32),
        ("proposals", C.c_int32),
        ("log", C.c_int32),
        ("proposal_level", C.c_int32),
        ("seed", C.c_uint64),
    ]


class DynamicUpdate(C.Structure):
    """qbc_dynamic_update: device pointers of one per-frame dynamic update."""

    _fields_ = [
        ("rest_pnts", C.c_void_p),
        ("rest_nrms", C.c_void_p),
        ("bone", C.c_void_p),
        ("bones", C.c_void_p),
        ("pnts", C.c_void_p),
        ("nrms", C.c_void_p),
        ("n", C.c_int64),
        ("n_bones", C.c_int32),
        ("levels", C.c_int32),
        ("basesize", C.c_float),
        ("pad", C.c_int32),
    ]


class RenderStats(C.Structure):
    """qbc_render_stats."""

    _fields_ = [
        ("queued", C.c_uint64),
        ("shadow_rays", C.c_uint64),
        ("shadow_visits", C.c_uint64),
        ("proposals_tried", C.c_uint64),
        ("proposals_proven", C.c_uint64),
        ("proposal_visits", C.c_uint64),
        ("box_words", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


PROPOSE_NONE, PROPOSE_MLP, PROPOSE_LOGGED, PROPOSE_RANDOM = 0, 1, 2, 3
PROPOSAL_PARAMS = 41360


class TuneResult(C.Structure):
    """qbc_tune_result."""

    _fields_ = [("tile_width", C.c_int32), ("blocks_per_sm", C.c_int32), ("service_min", C.c_int32),
                ("candidates", C.c_int32), ("ms_initial", C.c_float), ("ms_best", C.c_float),
                ("proposal_gate", C.c_int32), ("proposal_count", C.c_int32), ("proposal_level", C.c_int32),
                ("split_trees", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: (float(getattr(self, f)) if f.startswith("ms") else int(getattr(self, f))) for f, _ in self._fields_}


class TrainOpts(C.Structure):
    """qbc_train_opts."""

    _fields_ = [("steps", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("pad", C.c_int32),
                ("seed", C.c_uint64)]


class TrainStats(C.Structure):
    """qbc_train_stats."""

    _fields_ = [("samples", C.c_uint64), ("occluded", C.c_uint64), ("loss_first", C.c_float),
                ("loss_last", C.c_float)]

    def as_dict(self) -> dict:
        return {f: (float(getattr(self, f)) if "loss" in f else int(getattr(self, f))) for f, _ in self._fields_}


class SceneDesc(C.Structure):
    """qbc_scene_desc."""

    _fields_ = [
        ("kind", C.c_int32),
        ("levels", C.c_int32),
        ("n_points", C.c_int64),
        ("seed", C.c_uint64),
        ("basesize", C.c_float),
        ("n_boxes", C.c_int32),
        ("box_min", C.c_float),
        ("box_max", C.c_float),
        ("n_spheres", C.c_int32),
        ("sphere_min", C.c_float),
        ("sphere_max", C.c_float),
        ("color_noise", C.c_float),
    ]


# name -> (restype, argtypes)
SIGNATURES = {
    "qbc_version": (C.c_char_p, []),
    "qbc_last_error": (C.c_char_p, []),
    "qbc_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "qbc_destroy": (C.c_int, [C.c_void_p]),
    "qbc_upload": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_int]),
    "qbc_upload_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_size_t, C.c_size_t, C.c_size_t,
                                    C.c_size_t, C.c_int]),
    "qbc_skin_rigid": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, c_float_p, C.c_int,
                                 C.c_void_p, C.c_void_p]),
    "qbc_view_setup": (C.c_int, [C.c_float, C.c_float, c_float_p, c_float_p, C.c_float, C.c_int, C.c_int,
                                 C.c_float, C.c_int, C.c_float, C.POINTER(View)]),
    "qbc_render": (C.c_int, [C.c_void_p, C.c_float, C.c_float, c_float_p, c_float_p, C.c_float, C.c_int, C.c_int,
                             C.c_float, C.c_int, C.c_void_p]),
    "qbc_render_views": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(Outputs), C.c_int, C.c_int]),
    "qbc_trace_rays": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, c_float_p, C.c_int,
                                 C.POINTER(RayHits), C.c_int]),
    "qbc_camera_rays": (C.c_int, [C.c_void_p, C.POINTER(View), C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                  C.c_int]),
    "qbc_render_views_ex": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(Outputs), C.c_int, C.c_int,
                                      C.POINTER(RenderOpts), C.POINTER(RenderStats)]),
    "qbc_render_views_noalloc": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(Outputs), C.c_int]),
    "qbc_tree_remove_points": (C.c_int, [C.c_void_p, C.c_int, c_float_p, C.c_int64, C.c_float, C.c_int, C.c_int,
                                         C.POINTER(C.c_int32), C.POINTER(C.c_int32), c_int64_p]),
    "qbc_flat_read": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, c_float_p, c_float_p, c_float_p,
                                C.c_int64, c_int64_p, C.POINTER(C.c_int32), C.c_int64, c_int64_p]),
    "qbc_load_flat": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_float,
                                C.c_int, c_int64_p, c_int64_p, C.POINTER(C.c_int32), C.c_int64, c_int64_p]),
    "qbc_autotune": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(Outputs), C.c_int, C.POINTER(RenderOpts), C.c_int,
                               C.POINTER(TuneResult)]),
    "qbc_graph_capture": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(Outputs), C.c_int, C.POINTER(RenderOpts),
                                    C.POINTER(C.c_void_p)]),
    "qbc_graph_capture_dynamic": (C.c_int, [C.c_void_p, C.POINTER(DynamicUpdate), C.POINTER(View),
                                            C.POINTER(Outputs), C.c_int, C.POINTER(RenderOpts),
                                            C.POINTER(C.c_void_p)]),
    "qbc_dynamic_update_run": (C.c_int, [C.c_void_p, C.POINTER(DynamicUpdate)]),
    "qbc_graph_update": (C.c_int, [C.c_void_p, C.POINTER(View), C.c_int]),
    "qbc_graph_launch": (C.c_int, [C.c_void_p]),
    "qbc_graph_destroy": (C.c_int, [C.c_void_p]),
    "qbc_proposal_collect": (C.c_int, [C.c_void_p, C.POINTER(View), C.c_int, c_int64_p]),
    "qbc_proposal_train": (C.c_int, [C.c_void_p, C.POINTER(TrainOpts), C.POINTER(TrainStats)]),
    "qbc_proposal_clear": (C.c_int, [C.c_void_p]),
    "qbc_proposal_get_params": (C.c_int, [C.c_void_p, c_float_p]),
    "qbc_proposal_set_params": (C.c_int, [C.c_void_p, c_float_p]),
    "qbc_proposal_eval": (C.c_int, [C.c_void_p, c_float_p, C.c_int64, c_float_p]),
    "qbc_proposal_gradient": (C.c_int, [C.c_void_p, c_float_p, c_float_p, C.POINTER(C.c_int8), C.c_int64,
                                        c_float_p, c_float_p]),
    "qbc_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "qbc_synchronize": (C.c_int, [C.c_void_p]),
    "qbc_set_option": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qbc_get_option": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "qbc_tree_nodes": (C.c_int, [C.c_void_p, C.c_int, c_int64_p]),
    "qbc_model_points": (C.c_int, [C.c_void_p, C.c_int, c_int64_p]),
    "qbc_launch_count": (C.c_int, [C.c_void_p, c_int64_p]),
    "qbc_build_tree": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.c_float, C.c_int, C.c_int64, C.c_int]),
    "qbc_build_tree_paths": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.c_int, C.c_int64, C.c_int]),
    "qbc_download_tree": (C.c_int, [C.c_void_p, C.c_int, c_int32_p, C.c_int64, c_int64_p]),
    "qbc_octree_create": (C.c_int, [C.c_float, C.c_int, C.POINTER(C.c_void_p)]),
    "qbc_octree_free": (C.c_int, [C.c_void_p]),
    "qbc_octree_reset": (C.c_int, [C.c_void_p]),
    "qbc_octree_insert_points": (C.c_int, [C.c_void_p, c_float_p, C.c_int64, C.c_int64]),
    "qbc_octree_insert_paths": (C.c_int, [C.c_void_p, c_int32_p, C.c_int64, C.c_int64]),
    "qbc_octree_remove_point": (C.c_int, [C.c_void_p, c_float_p, c_int32_p, c_int32_p]),
    "qbc_octree_nodes": (C.c_int, [C.c_void_p, C.POINTER(c_int32_p), c_int64_p]),
    "qbc_scene_generate": (C.c_int, [C.POINTER(SceneDesc), c_float_p, c_float_p, c_float_p]),
}

_LIB = None


OPT_SERVICE_MIN = 1
OPT_PROPOSAL_GATE = 2
OPT_TILE_WIDTH = 3
OPT_BLOCKS_PER_SM = 4
OPT_PROPOSAL_COUNT = 5
OPT_BOX_PRUNE = 6
OPT_PERSISTENT = 7
OPT_PROPOSAL_LEVEL = 8
OPT_SPLIT_TREES = 9


def lib_path() -> str:
    """The in-tree build, or the file named by QBC_LIBRARY (another build of
    the same library, e.g. one compiled with different tuning)."""
    return os.environ.get("QBC_LIBRARY") or _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libqbcuda.so (building it first if asked); raise if unavailable."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build_if_missing and path == _build.LIB:
        _build.build()
    if not os.path.exists(path):
        raise QbcError(-4, f"libqbcuda.so not built at {path}")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        msg = _LIB.qbc_last_error().decode() if _LIB is not None else ""
        raise QbcError(rc, msg)
