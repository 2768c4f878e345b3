"""Host-side mirror of the reference's GL connector for the octree ray-cast
path (src/qubatron/octree_glc.c:65-85), running on libqbcuda.

Names and argument meanings follow the reference:

* ``octree_glc_init(path)``                       -> octree_glc.c:93-247
* ``octree_glc_upload_texbuffer_data(rc, data, type, size, itemsize, start, end, buftype)``
                                                  -> octree_glc.c:361-498
* ``octree_glc_update(rc, width, height, position, angle, lighta, quality, maxlevel, basesize, shoot)``
                                                  -> octree_glc.c:249-352

Differences, all deliberate: there is no window, so ``octree_glc_update``
returns the RGBA8 render target as an (oh, ow, 4) uint8 array with row 0 at
the bottom instead of blitting it; failures raise QbcError where the
reference silently ignores GL errors.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import Outputs, QbcError, View, check

GL_INT = _lib.QBC_GL_INT
GL_FLOAT = _lib.QBC_GL_FLOAT

OCTREE_GLC_BUFFER_STATIC_COLOR = _lib.STATIC_COLOR
OCTREE_GLC_BUFFER_STATIC_NORMAL = _lib.STATIC_NORMAL
OCTREE_GLC_BUFFER_STATIC_OCTREE = _lib.STATIC_OCTREE
OCTREE_GLC_BUFFER_DYNAMIC_COLOR = _lib.DYNAMIC_COLOR
OCTREE_GLC_BUFFER_DYNAMIC_NORMAL = _lib.DYNAMIC_NORMAL
OCTREE_GLC_BUFFER_DYNAMIC_OCTREE = _lib.DYNAMIC_OCTREE


def _f3(v) -> C.Array:
    a = (C.c_float * 3)()
    for k in range(3):
        a[k] = float(v[k])
    return a


def view_setup(width: float, height: float, position, angle, lighta: float, quality: int, maxlevel: int,
               basesize: float, shoot: int = 0, focal: float = 0.0) -> View:
    """Uniforms of one frame (qbc_view_setup)."""
    lib = _lib.load()
    v = View()
    check(lib.qbc_view_setup(width, height, _f3(position), _f3(angle), lighta, int(quality), int(maxlevel),
                             basesize, int(shoot), focal, C.byref(v)))
    return v


class FrameBuffers:
    """Host (numpy) outputs for one view; pass names of the streams wanted."""

    SHAPES = {"rgba8": (4, np.uint8), "rgba32f": (4, np.float32), "flags": (1, np.uint32),
              "leaf": (4, np.int32), "isp": (4, np.float32), "visits": (4, np.uint32)}

    def __init__(self, view: View, streams: Iterable[str] = ("rgba8",)):
        h, w = view.height_px, view.width_px
        self.arrays = {}
        for s in streams:
            comps, dt = self.SHAPES[s]
            shape = (h, w) if comps == 1 else (h, w, comps)
            self.arrays[s] = np.zeros(shape, dtype=dt)

    def outputs(self) -> Outputs:
        o = Outputs()
        for s, a in self.arrays.items():
            setattr(o, s, a.ctypes.data)
        return o

    def __getitem__(self, k: str) -> np.ndarray:
        return self.arrays[k]


class OctreeGLC:
    """octree_glc_t: one libqbcuda context on one GPU."""

    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = C.c_void_p()
        check(self._lib.qbc_create(int(device), C.byref(h)))
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self._lib.qbc_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- octree_glc_upload_texbuffer_data ----
    def upload_texbuffer_data(self, data, type: int, size: int, itemsize: int, start: int, end: int,
                              buftype: int) -> None:
        """`data` is the whole host array (a C-contiguous numpy array or an int
        address); the copy reads bytes [start, end) of it."""
        if isinstance(data, np.ndarray):
            if not data.flags.c_contiguous:
                raise QbcError(-1, "upload data must be C-contiguous")
            if data.nbytes < size:
                raise QbcError(-1, f"upload size {size} exceeds the array's {data.nbytes} bytes")
            ptr = data.ctypes.data
        else:
            ptr = int(data)
        check(self._lib.qbc_upload(self.handle, C.c_void_p(ptr), int(type), int(size), int(itemsize), int(start),
                                   int(end), int(buftype)))

    # ---- octree_glc_update ----
    def update(self, width: float, height: float, position, angle, lighta: float, quality: int, maxlevel: int,
               basesize: float, shoot: int = 0) -> np.ndarray:
        v = view_setup(width, height, position, angle, lighta, quality, maxlevel, basesize, shoot)
        out = np.zeros((v.height_px, v.width_px, 4), dtype=np.uint8)
        check(self._lib.qbc_render(self.handle, width, height, _f3(position), _f3(angle), lighta, int(quality),
                                   int(maxlevel), basesize, int(shoot), C.c_void_p(out.ctypes.data)))
        return out

    def render_views(self, views: Sequence[View], outputs: Sequence[Outputs], on_device: bool) -> None:
        n = len(views)
        varr = (View * n)(*views)
        oarr = (Outputs * n)(*outputs)
        check(self._lib.qbc_render_views(self.handle, varr, oarr, n, 1 if on_device else 0))

    def render_views_ex(self, views: Sequence[View], outputs: Sequence[Outputs], on_device: bool,
                        two_pass: bool = False, proposals: int = 0, log: bool = False, proposal_level: int = 0,
                        seed: int = 0) -> dict:
        """qbc_render_views_ex; returns the render statistics."""
        n = len(views)
        varr = (View * n)(*views)
        oarr = (Outputs * n)(*outputs)
        opts = _lib.RenderOpts(int(two_pass), int(proposals), int(log), int(proposal_level), int(seed))
        st = _lib.RenderStats()
        check(self._lib.qbc_render_views_ex(self.handle, varr, oarr, n, 1 if on_device else 0, C.byref(opts),
                                            C.byref(st)))
        return st.as_dict()

    def render_host_ex(self, views: Sequence[View], streams: Iterable[str] = ("rgba8",), **kw):
        bufs = [FrameBuffers(v, streams) for v in views]
        stats = self.render_views_ex(views, [b.outputs() for b in bufs], False, **kw)
        return bufs, stats

    def remove_points(self, dynamic: bool, points, basesize: float = 1800.0, levels: int = 12):
        """qbc_tree_remove_points on host points: octree_remove_point of each
        point in order, on the device tree. Returns (modind, octind, removed)."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        n = pts.shape[0]
        mod = np.zeros(n, np.int32)
        oct_ = np.zeros(n, np.int32)
        rem = C.c_int64()
        i32 = C.POINTER(C.c_int32)
        check(self._lib.qbc_tree_remove_points(self.handle, 1 if dynamic else 0, pts.ctypes.data_as(_lib.c_float_p), n,
                                               basesize, levels, 0, mod.ctypes.data_as(i32), oct_.ctypes.data_as(i32),
                                               C.byref(rem)))
        return mod, oct_, rem.value

    def load_flat(self, prefix: str, dynamic: bool = False, basesize: float = 1800.0, levels: int = 12) -> dict:
        """qbc_load_flat: read prefix.{pnt,col,nrm,rng}, build the tree on the
        GPU in file order, upload the model; returns counts and ranges."""
        from .flatfile import paths
        p = [s.encode() for s in paths(prefix)]
        n, nodes, nr = C.c_int64(), C.c_int64(), C.c_int64()
        check(self._lib.qbc_flat_read(p[0], p[1], p[2], p[3], None, None, None, 0, C.byref(n), None, 0, C.byref(nr)))
        rng = np.zeros(max(nr.value, 1), np.int32)
        check(self._lib.qbc_load_flat(self.handle, 1 if dynamic else 0, p[0], p[1], p[2], p[3], basesize, levels,
                                      C.byref(n), C.byref(nodes), rng.ctypes.data_as(C.POINTER(C.c_int32)), rng.size,
                                      C.byref(nr)))
        return {"points": n.value, "nodes": nodes.value, "ranges": rng[:nr.value]}

    def autotune(self, views: Sequence[View], outputs: Sequence[Outputs], reps: int = 5, two_pass: bool = False,
                 proposals: int = 0, proposal_level: int = 0, seed: int = 0) -> dict:
        """qbc_autotune: time candidate tuning options on these views (device
        outputs) and leave the fastest set; returns the chosen settings."""
        n = len(views)
        varr = (View * n)(*views)
        oarr = (Outputs * n)(*outputs)
        opts = _lib.RenderOpts(int(two_pass), int(proposals), 0, int(proposal_level), int(seed))
        res = _lib.TuneResult()
        check(self._lib.qbc_autotune(self.handle, varr, oarr, n, C.byref(opts), int(reps), C.byref(res)))
        return res.as_dict()

    def graph_capture(self, views: Sequence[View], outputs: Sequence[Outputs], two_pass: bool = False,
                      proposals: int = 0, proposal_level: int = 0, seed: int = 0) -> "FrameGraph":
        """qbc_graph_capture: the frame (device outputs) as a CUDA graph."""
        n = len(views)
        varr = (View * n)(*views)
        oarr = (Outputs * n)(*outputs)
        opts = _lib.RenderOpts(int(two_pass), int(proposals), 0, int(proposal_level), int(seed))
        h = C.c_void_p()
        check(self._lib.qbc_graph_capture(self.handle, varr, oarr, n, C.byref(opts), C.byref(h)))
        return FrameGraph(self, h, n)

    def dynamic_update(self, update: "_lib.DynamicUpdate") -> None:
        """qbc_dynamic_update_run: skin, rebuild the dynamic tree, take the
        normals, all queued on the context's stream."""
        check(self._lib.qbc_dynamic_update_run(self.handle, C.byref(update)))

    def graph_capture_dynamic(self, update: "_lib.DynamicUpdate", views: Sequence[View],
                              outputs: Sequence[Outputs], two_pass: bool = False, proposals: int = 0,
                              proposal_level: int = 0, seed: int = 0) -> "FrameGraph":
        """qbc_graph_capture_dynamic: the dynamic update and the frame as one
        CUDA graph; write new bones into update.bones before each launch."""
        n = len(views)
        varr = (View * n)(*views)
        oarr = (Outputs * n)(*outputs)
        opts = _lib.RenderOpts(int(two_pass), int(proposals), 0, int(proposal_level), int(seed))
        h = C.c_void_p()
        check(self._lib.qbc_graph_capture_dynamic(self.handle, C.byref(update), varr, oarr, n, C.byref(opts),
                                                  C.byref(h)))
        return FrameGraph(self, h, n)

    def render_views_noalloc(self, views: Sequence[View], outputs: Sequence[Outputs]) -> None:
        """qbc_render_views_noalloc: device outputs only, no allocation in
        the call (the work-queue counters live in static device memory)."""
        n = len(views)
        varr = (View * n)(*views)
        oarr = (Outputs * n)(*outputs)
        check(self._lib.qbc_render_views_noalloc(self.handle, varr, oarr, n))

    def render_host(self, views: Sequence[View], streams: Iterable[str] = ("rgba8",)) -> list:
        """Render views into fresh numpy buffers; returns a FrameBuffers per view."""
        bufs = [FrameBuffers(v, streams) for v in views]
        self.render_views(views, [b.outputs() for b in bufs], on_device=False)
        return bufs

    def trace_rays(self, pos: np.ndarray, dirs: np.ndarray, basecube, maxlevel: int) -> dict:
        """Batched ray queries (qbc_trace_rays) on host arrays -> dict of arrays."""
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        n = pos.shape[0]
        out = {"status": np.zeros(n, np.int32), "leaf": np.zeros((n, 2), np.int32),
               "model": np.zeros((n, 2), np.int32), "isp": np.zeros((n, 4), np.float32),
               "col": np.zeros((n, 4), np.float32), "nrm": np.zeros((n, 4), np.float32),
               "visits": np.zeros((n, 2), np.uint32)}
        h = _lib.RayHits(*[out[k].ctypes.data for k in ("status", "leaf", "model", "isp", "col", "nrm", "visits")])
        bc = (C.c_float * 4)(*[float(x) for x in basecube])
        check(self._lib.qbc_trace_rays(self.handle, C.c_void_p(pos.ctypes.data), C.c_void_p(dirs.ctypes.data), n, bc,
                                       int(maxlevel), C.byref(h), 0))
        return out

    def camera_rays(self, view: View, px: np.ndarray, py: np.ndarray) -> np.ndarray:
        """Camera rays of the pixels (px, py) of a view as the render kernels
        make them (qbc_camera_rays): (n, 4) float32, csv xyz and the cosine of
        its angle to the light."""
        px = np.ascontiguousarray(px, np.int32).ravel()
        py = np.ascontiguousarray(py, np.int32).ravel()
        out = np.zeros((px.size, 4), np.float32)
        check(self._lib.qbc_camera_rays(self.handle, C.byref(view), C.c_void_p(px.ctypes.data),
                                        C.c_void_p(py.ctypes.data), px.size, C.c_void_p(out.ctypes.data), 0))
        return out

    def camera_rays_device(self, view: View, px_ptr: int, py_ptr: int, n: int, out_ptr: int) -> None:
        """qbc_camera_rays on device arrays (int32 px, py; float4 out)."""
        check(self._lib.qbc_camera_rays(self.handle, C.byref(view), C.c_void_p(px_ptr), C.c_void_p(py_ptr), int(n),
                                        C.c_void_p(out_ptr), 1))

    def set_stream(self, stream_ptr: Optional[int]) -> None:
        check(self._lib.qbc_set_stream(self.handle, C.c_void_p(stream_ptr or 0)))

    def build_tree(self, dynamic: bool, points, basesize: float = 1800.0, levels: int = 12,
                   first_index: int = 0, count: bool = True) -> Optional[int]:
        """GPU build of the static or dynamic tree from points (numpy host
        array, or a device pointer with `points=(ptr, n)`); returns the node
        count (count=False: returns None and does not wait for the build)."""
        if isinstance(points, tuple):
            ptr, n, dev = int(points[0]), int(points[1]), 1
        else:
            p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
            ptr, n, dev = p.ctypes.data, p.shape[0], 0
        check(self._lib.qbc_build_tree(self.handle, 1 if dynamic else 0, C.c_void_p(ptr), n, float(basesize),
                                       int(levels), int(first_index), dev))
        return self.tree_nodes(1 if dynamic else 0) if count else None

    def build_tree_paths(self, dynamic: bool, octets, levels: int = 12, first_index: int = 0) -> int:
        if isinstance(octets, tuple):
            ptr, n, dev = int(octets[0]), int(octets[1]), 1
        else:
            o = np.ascontiguousarray(octets, np.int32).reshape(-1, levels)
            ptr, n, dev = o.ctypes.data, o.shape[0], 0
        check(self._lib.qbc_build_tree_paths(self.handle, 1 if dynamic else 0, C.c_void_p(ptr), n, int(levels),
                                             int(first_index), dev))
        return self.tree_nodes(1 if dynamic else 0)

    def download_tree(self, dynamic: bool) -> np.ndarray:
        """The tree in the reference layout, shape (n, 12) int32."""
        n = C.c_int64()
        t = 1 if dynamic else 0
        check(self._lib.qbc_download_tree(self.handle, t, None, 0, C.byref(n)))
        out = np.zeros((n.value, 12), np.int32)
        if n.value:
            check(self._lib.qbc_download_tree(self.handle, t, out.ctypes.data_as(_lib.c_int32_p), n.value,
                                              C.byref(n)))
        return out

    def upload_device(self, ptr: int, type: int, size: int, itemsize: int, start: int, end: int,
                      buftype: int) -> None:
        """qbc_upload_device: the same upload from device memory at ptr."""
        check(self._lib.qbc_upload_device(self.handle, C.c_void_p(int(ptr)), int(type), int(size), int(itemsize),
                                          int(start), int(end), int(buftype)))

    def skin_rigid(self, rest_pts: int, rest_nrm: int, bone: int, n: int, bones: np.ndarray, out_pts: int,
                   out_nrm: int) -> None:
        """qbc_skin_rigid on device pointers; bones is (n_bones, 12) float32."""
        b = np.ascontiguousarray(bones, np.float32).reshape(-1, 12)
        check(self._lib.qbc_skin_rigid(self.handle, C.c_void_p(rest_pts), C.c_void_p(rest_nrm), C.c_void_p(bone),
                                       int(n), b.ctypes.data_as(_lib.c_float_p), b.shape[0], C.c_void_p(out_pts),
                                       C.c_void_p(out_nrm)))

    # ---- occluder-proposal network ----
    def proposal_collect(self, views: Sequence[View]) -> int:
        n = len(views)
        varr = (View * n)(*views)
        cnt = C.c_int64()
        check(self._lib.qbc_proposal_collect(self.handle, varr, n, C.byref(cnt)))
        return cnt.value

    def proposal_train(self, steps: int, batch: int = 4096, lr: float = 2e-3, seed: int = 1) -> dict:
        st = _lib.TrainStats()
        check(self._lib.qbc_proposal_train(self.handle, C.byref(_lib.TrainOpts(int(steps), int(batch), float(lr), 0,
                                                                               int(seed))), C.byref(st)))
        return st.as_dict()

    def proposal_clear(self) -> None:
        check(self._lib.qbc_proposal_clear(self.handle))

    def proposal_params(self) -> np.ndarray:
        out = np.zeros(_lib.PROPOSAL_PARAMS, np.float32)
        check(self._lib.qbc_proposal_get_params(self.handle, out.ctypes.data_as(_lib.c_float_p)))
        return out

    def proposal_set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == _lib.PROPOSAL_PARAMS
        check(self._lib.qbc_proposal_set_params(self.handle, p.ctypes.data_as(_lib.c_float_p)))

    def proposal_eval(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 45)
        out = np.zeros((x.shape[0], 4), np.float32)
        check(self._lib.qbc_proposal_eval(self.handle, x.ctypes.data_as(_lib.c_float_p), x.shape[0],
                                          out.ctypes.data_as(_lib.c_float_p)))
        return out

    def proposal_gradient(self, x: np.ndarray, t: np.ndarray, kind: np.ndarray):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 45)
        t = np.ascontiguousarray(t, np.float32)
        k = np.ascontiguousarray(kind, np.int8)
        loss = C.c_float()
        grad = np.zeros(_lib.PROPOSAL_PARAMS, np.float32)
        check(self._lib.qbc_proposal_gradient(self.handle, x.ctypes.data_as(_lib.c_float_p),
                                              t.ctypes.data_as(_lib.c_float_p), k.ctypes.data_as(C.POINTER(C.c_int8)),
                                              x.shape[0], C.byref(loss), grad.ctypes.data_as(_lib.c_float_p)))
        return loss.value, grad

    def set_option(self, option: int, value: int) -> None:
        check(self._lib.qbc_set_option(self.handle, int(option), int(value)))

    def get_option(self, option: int) -> int:
        v = C.c_int()
        check(self._lib.qbc_get_option(self.handle, int(option), C.byref(v)))
        return v.value

    def synchronize(self) -> None:
        check(self._lib.qbc_synchronize(self.handle))

    def tree_nodes(self, tree: int) -> int:
        n = C.c_int64()
        check(self._lib.qbc_tree_nodes(self.handle, tree, C.byref(n)))
        return n.value

    def model_points(self, model: int) -> int:
        n = C.c_int64()
        check(self._lib.qbc_model_points(self.handle, model, C.byref(n)))
        return n.value

    def launch_count(self) -> int:
        n = C.c_int64()
        check(self._lib.qbc_launch_count(self.handle, C.byref(n)))
        return n.value

    # convenience: whole-array uploads in the reference's call pattern
    def upload_model(self, dynamic: bool, colors: np.ndarray, normals: np.ndarray) -> None:
        colors = np.ascontiguousarray(colors, dtype=np.float32)
        normals = np.ascontiguousarray(normals, dtype=np.float32)
        base = DYNAMIC if dynamic else STATIC
        self.upload_texbuffer_data(colors, GL_FLOAT, colors.nbytes, 12, 0, colors.nbytes, base + 0)
        self.upload_texbuffer_data(normals, GL_FLOAT, normals.nbytes, 12, 0, normals.nbytes, base + 1)

    def upload_octree(self, dynamic: bool, nodes: np.ndarray) -> None:
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        base = DYNAMIC if dynamic else STATIC
        self.upload_texbuffer_data(nodes, GL_INT, nodes.nbytes, 16, 0, nodes.nbytes, base + 2)


STATIC = 0
DYNAMIC = 3


def octree_glc_init(path: Optional[str] = None, device: int = 0) -> OctreeGLC:
    """octree_glc_init: `path` (the shader directory) is accepted and unused."""
    return OctreeGLC(device)


def octree_glc_upload_texbuffer_data(rc: OctreeGLC, data, type: int, size: int, itemsize: int, start: int,
                                     end: int, buftype: int) -> None:
    rc.upload_texbuffer_data(data, type, size, itemsize, start, end, buftype)


def octree_glc_update(rc: OctreeGLC, width: float, height: float, position, angle, lighta: float, quality: int,
                      maxlevel: int, basesize: float, shoot: int = 0) -> np.ndarray:
    return rc.update(width, height, position, angle, lighta, quality, maxlevel, basesize, shoot)


class FrameGraph:
    """qbc_graph: a captured frame; launch() replays it, update(views)
    re-captures it for new uniforms of the same view sizes."""

    def __init__(self, owner: OctreeGLC, handle: C.c_void_p, n: int):
        self._owner = owner  # the context outlives the graph
        self._lib = owner._lib
        self.handle = handle
        self.n = n

    def launch(self) -> None:
        check(self._lib.qbc_graph_launch(self.handle))

    def update(self, views: Sequence[View]) -> None:
        n = len(views)
        varr = (View * n)(*views)
        check(self._lib.qbc_graph_update(self.handle, varr, n))

    def close(self) -> None:
        if self.handle:
            self._lib.qbc_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
