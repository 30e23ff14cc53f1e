"""ctypes binding of the C ABI in include/fclg.h (lib/libfclg.so).

The library is the product path: there is no CPU fallback, and loading fails
loudly when the shared library or a GB300 (sm_103) device is missing.
"""
import ctypes
import os

import numpy as np

from .layout import PAIR_DTYPE, RESULT64_DTYPE, RESULT_DTYPE, SHAPE_DTYPE

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("FCLG_LIB") or os.path.join(PKG, "lib", "libfclg.so")

FCLG_REQ_BOOLEAN_ONLY = 1
FCLG_REQ_NO_EPA = 2
FCLG_REQ_WARM_START = 4
FCLG_REQ_GJK_BOOLEAN = 8
FCLG_REQ_NO_ANALYTIC = 16
FCLG_REQ_INCREMENTAL = 32
FCLG_STATUS_DIRECTED = 1 << 18
FCLG_STATUS_INCREMENTAL = 1 << 19

# Every symbol include/fclg.h declares (checked by tests/test_abi.py).
EXPORTS = [
    "fclg_create", "fclg_destroy", "fclg_last_error", "fclg_version", "fclg_built_arch",
    "fclg_set_shapes", "fclg_set_shapes_device",
    "fclg_distance", "fclg_distance_device", "fclg_distance_device_static", "fclg_collide", "fclg_collide_device",
    "fclg_distance64", "fclg_distance64_device",
    "fclg_set_launch", "fclg_set_tuning", "fclg_get_tuning", "fclg_launch_count", "fclg_set_profiling",
    "fclg_pass_times", "fclg_bvh_build", "fclg_bvh_node_sizes", "fclg_mesh_create", "fclg_mesh_destroy", "fclg_mesh_info", "fclg_mesh_export",
    "fclg_mesh_collide", "fclg_mesh_collide_device", "fclg_mesh_traffic",
    "fclg_warmstart_create", "fclg_warmstart_destroy", "fclg_warmstart_last_error", "fclg_warmstart_param_count",
    "fclg_warmstart_get_params", "fclg_warmstart_set_params", "fclg_warmstart_predict", "fclg_warmstart_forward",
    "fclg_warmstart_gradient", "fclg_warmstart_train", "fclg_set_warmstart", "fclg_warmstart_status",
    "fclg_autotune", "fclg_graph_create", "fclg_graph_launch", "fclg_graph_destroy",
    "fclg_collide_directed", "fclg_collide_directed_device", "fclg_hull_graph",
    "fclg_mesh_shape_collide", "fclg_mesh_shape_collide_device",
    "fclg_broadphase", "fclg_broadphase_device", "fclg_object_pairs_device", "fclg_broadphase_cross_device",
    "fclg_translational_ccd", "fclg_translational_ccd_device",
    "fclg_mesh_shape_contacts", "fclg_mesh_shape_contacts_device",
]

# translational CCD (fclg_displacement, fclg_ccd_request, fclg_ccd_result)
DISP_DTYPE = np.dtype([("axis", "<f4", (3,)), ("distance", "<f4")])
CCD_RESULT_DTYPE = np.dtype([("collide", "<u4"), ("status", "<u4"), ("toc_lower", "<f4"), ("toc_upper", "<f4")])
FCLG_TOC_NONE, FCLG_TOC_BOX, FCLG_TOC_SAMPLE = 0, 1, 2


class CcdRequest(ctypes.Structure):
    _fields_ = [("toc_type", ctypes.c_uint32), ("max_gjk_iterations", ctypes.c_int32),
                ("gjk_tolerance", ctypes.c_float), ("reserved", ctypes.c_uint32),
                ("zero_movement_tolerance", ctypes.c_double)]

STATIC_MAX_PAIRS = 16384  # FCLG_STATIC_MAX_PAIRS

MESH_NODE_DTYPE = np.dtype([("axis", "<f4", (9,)), ("center", "<f4", (3,)), ("extent", "<f4", (3,)),
                            ("child", "<i4")])
assert MESH_NODE_DTYPE.itemsize == 64


class FclgError(RuntimeError):
    pass


class Tuning(ctypes.Structure):
    _fields_ = [("bucketing", ctypes.c_int32), ("gjk_lanes_small", ctypes.c_int32),
                ("gjk_lanes_large", ctypes.c_int32), ("large_hull_vertices", ctypes.c_int32),
                ("gjk_ctas_per_sm", ctypes.c_int32), ("epa_ctas_per_sm", ctypes.c_int32),
                ("support_walk", ctypes.c_int32), ("gjk_refill", ctypes.c_int32), ("epa_resume", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("gjk_max_iterations", ctypes.c_uint32), ("epa_max_faces", ctypes.c_uint32),
                ("epa_max_iterations", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("gjk_tolerance", ctypes.c_float), ("epa_tolerance", ctypes.c_float),
                ("warm_gap", ctypes.c_float), ("warm_probe", ctypes.c_uint32)]


class Request64(ctypes.Structure):
    """fclg_request64: the parameters of the FP64 separation distance."""
    _fields_ = [("gjk_tolerance", ctypes.c_double), ("gjk_max_iterations", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


_lib = None


def load_library(path=LIB_PATH):
    """Loads lib/libfclg.so and declares the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FclgError("libfclg.so not built (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    lib.fclg_create.argtypes = [ctypes.POINTER(vp), i32]
    lib.fclg_create.restype = i32
    lib.fclg_destroy.argtypes = [vp]
    lib.fclg_destroy.restype = None
    lib.fclg_last_error.argtypes = [vp]
    lib.fclg_last_error.restype = ctypes.c_char_p
    lib.fclg_version.restype = i32
    lib.fclg_built_arch.restype = i32
    lib.fclg_set_shapes.argtypes = [vp, vp, u32, vp, u64]
    lib.fclg_set_shapes.restype = i32
    lib.fclg_set_shapes_device.argtypes = [vp, vp, u32, vp, u64]
    lib.fclg_set_shapes_device.restype = i32
    for name in ("fclg_distance", "fclg_collide", "fclg_distance64"):
        getattr(lib, name).argtypes = [vp, vp, u32, vp, vp]
        getattr(lib, name).restype = i32
    for name in ("fclg_distance_device", "fclg_distance_device_static", "fclg_collide_device",
                 "fclg_distance64_device"):
        getattr(lib, name).argtypes = [vp, vp, u32, vp, vp, vp]
        getattr(lib, name).restype = i32
    lib.fclg_set_launch.argtypes = [vp, i32, i32]
    lib.fclg_set_launch.restype = i32
    lib.fclg_set_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.fclg_set_tuning.restype = i32
    lib.fclg_get_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.fclg_get_tuning.restype = i32
    lib.fclg_launch_count.argtypes = [vp]
    lib.fclg_launch_count.restype = u64
    lib.fclg_set_profiling.argtypes = [vp, i32]
    lib.fclg_set_profiling.restype = i32
    lib.fclg_pass_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(u64), i32]
    lib.fclg_pass_times.restype = i32
    lib.fclg_bvh_build.argtypes = [vp, u32, vp, u32, vp, vp]
    lib.fclg_bvh_build.restype = i32
    lib.fclg_bvh_node_sizes.argtypes = [vp, u32, vp, u32, vp, ctypes.POINTER(u32)]
    lib.fclg_bvh_node_sizes.restype = i32
    lib.fclg_mesh_create.argtypes = [vp, vp, u32, vp, u32, ctypes.POINTER(vp)]
    lib.fclg_mesh_create.restype = i32
    lib.fclg_mesh_destroy.argtypes = [vp]
    lib.fclg_mesh_destroy.restype = None
    lib.fclg_mesh_info.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    lib.fclg_mesh_info.restype = i32
    lib.fclg_mesh_export.argtypes = [vp, vp, vp]
    lib.fclg_mesh_export.restype = i32
    lib.fclg_mesh_collide.argtypes = [vp, vp, vp, vp, u32, u32, vp, vp, vp, vp]
    lib.fclg_mesh_collide.restype = i32
    lib.fclg_mesh_collide_device.argtypes = [vp, vp, vp, vp, u32, u32, vp, vp, vp, vp, vp]
    lib.fclg_mesh_collide_device.restype = i32
    lib.fclg_mesh_traffic.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64), i32]
    lib.fclg_mesh_traffic.restype = i32
    lib.fclg_warmstart_create.argtypes = [i32, u32, u32, ctypes.POINTER(vp)]
    lib.fclg_warmstart_create.restype = i32
    lib.fclg_warmstart_destroy.argtypes = [vp]
    lib.fclg_warmstart_destroy.restype = None
    lib.fclg_warmstart_last_error.argtypes = [vp]
    lib.fclg_warmstart_last_error.restype = ctypes.c_char_p
    lib.fclg_warmstart_param_count.argtypes = [vp]
    lib.fclg_warmstart_param_count.restype = u64
    for name in ("fclg_warmstart_get_params", "fclg_warmstart_set_params"):
        getattr(lib, name).argtypes = [vp, vp, u64]
        getattr(lib, name).restype = i32
    lib.fclg_warmstart_predict.argtypes = [vp, vp, u32, vp, u32, vp]
    lib.fclg_warmstart_status.argtypes = [vp]
    lib.fclg_warmstart_status.restype = i32
    lib.fclg_warmstart_predict.restype = i32
    lib.fclg_warmstart_forward.argtypes = [vp, vp, u32, vp, vp]
    lib.fclg_warmstart_forward.restype = i32
    lib.fclg_warmstart_gradient.argtypes = [vp, vp, vp, u32, vp, vp]
    lib.fclg_warmstart_gradient.restype = i32
    lib.fclg_warmstart_train.argtypes = [vp, vp, vp, u32, ctypes.POINTER(TrainConfig), vp]
    lib.fclg_warmstart_train.restype = i32
    lib.fclg_set_warmstart.argtypes = [vp, vp]
    lib.fclg_set_warmstart.restype = i32
    lib.fclg_collide_directed.argtypes = [vp, vp, u32, vp, vp, vp]
    lib.fclg_collide_directed.restype = i32
    lib.fclg_collide_directed_device.argtypes = [vp, vp, u32, vp, vp, vp, vp]
    lib.fclg_collide_directed_device.restype = i32
    lib.fclg_autotune.argtypes = [vp, vp, u32, vp, vp, i32, ctypes.POINTER(Tuning), ctypes.POINTER(ctypes.c_float)]
    lib.fclg_autotune.restype = i32
    lib.fclg_graph_create.argtypes = [vp, vp, u32, vp, vp, i32, ctypes.POINTER(vp)]
    lib.fclg_graph_create.restype = i32
    lib.fclg_graph_launch.argtypes = [vp, vp, vp]
    lib.fclg_graph_launch.restype = i32
    lib.fclg_graph_destroy.argtypes = [vp]
    lib.fclg_graph_destroy.restype = None
    lib.fclg_hull_graph.argtypes = [vp, u32, vp, vp, vp, u32, ctypes.POINTER(u32)]
    lib.fclg_hull_graph.restype = i32
    lib.fclg_mesh_shape_collide.argtypes = [vp, vp, vp, vp, u32, u32, vp, vp, vp, vp]
    lib.fclg_mesh_shape_collide.restype = i32
    lib.fclg_mesh_shape_collide_device.argtypes = [vp, vp, vp, vp, u32, u32, vp, vp, vp, vp, vp]
    lib.fclg_mesh_shape_collide_device.restype = i32
    lib.fclg_broadphase.argtypes = [vp, vp, vp, u32, vp, u32, ctypes.POINTER(u32), vp]
    lib.fclg_broadphase.restype = i32
    lib.fclg_broadphase_device.argtypes = [vp, vp, vp, u32, vp, u32, vp, vp, vp, vp]
    lib.fclg_broadphase_device.restype = i32
    lib.fclg_object_pairs_device.argtypes = [vp, vp, vp, vp, u32, vp, vp]
    lib.fclg_object_pairs_device.restype = i32
    lib.fclg_broadphase_cross_device.argtypes = [vp, vp, vp, u32, vp, vp, u32, vp, u32, vp, vp]
    lib.fclg_broadphase_cross_device.restype = i32
    lib.fclg_mesh_shape_contacts.argtypes = [vp, vp, vp, vp, u32, u32, vp, vp, vp, vp, vp]
    lib.fclg_mesh_shape_contacts.restype = i32
    lib.fclg_mesh_shape_contacts_device.argtypes = [vp, vp, vp, vp, u32, u32, vp, vp, vp, vp, vp, vp]
    lib.fclg_mesh_shape_contacts_device.restype = i32
    lib.fclg_translational_ccd.argtypes = [vp, vp, u32, vp, vp, vp]
    lib.fclg_translational_ccd.restype = i32
    lib.fclg_translational_ccd_device.argtypes = [vp, vp, u32, vp, vp, vp, vp]
    lib.fclg_translational_ccd_device.restype = i32
    _lib = lib
    return lib


class TrainConfig(ctypes.Structure):
    _fields_ = [("epochs", ctypes.c_uint32), ("batch", ctypes.c_uint32), ("lr", ctypes.c_float),
                ("lr_final", ctypes.c_float), ("seed", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def make_request64(gjk_tol=0.0, gjk_max_iter=0):
    r = Request64()
    r.gjk_tolerance = gjk_tol
    r.gjk_max_iterations = gjk_max_iter
    return r


def make_request(flags=0, gjk_tol=0.0, epa_tol=0.0, gjk_max_iter=0, epa_max_faces=0, epa_max_iter=0,
                 warm_gap=0.0, warm_probe=0):
    r = Request()
    r.flags = flags
    r.warm_gap = warm_gap
    r.warm_probe = warm_probe
    r.gjk_tolerance = gjk_tol
    r.epa_tolerance = epa_tol
    r.gjk_max_iterations = gjk_max_iter
    r.epa_max_faces = epa_max_faces
    r.epa_max_iterations = epa_max_iter
    return r


class Context:
    """One fclg_context on a device: shapes plus batched collide / distance."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.fclg_create(ctypes.byref(h), device)
        if rc != 0:
            raise FclgError("fclg_create(device=%d) failed with %d (needs an sm_103 GPU)" % (device, rc))
        self.h = h
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.fclg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise FclgError("%s failed (%d): %s" % (what, rc, self.lib.fclg_last_error(self.h).decode()))

    def set_shapes(self, shapes, vertices):
        s = np.ascontiguousarray(shapes, SHAPE_DTYPE)
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 4)
        self._check(self.lib.fclg_set_shapes(self.h, _ptr(s), len(s), _ptr(v), len(v)), "fclg_set_shapes")

    def set_shapes_device(self, d_shapes, d_vertices):
        """d_shapes / d_vertices: CUDA tensors (uint8 or any dtype) holding the packed arrays."""
        n_s = d_shapes.numel() * d_shapes.element_size() // SHAPE_DTYPE.itemsize
        n_v = d_vertices.numel() * d_vertices.element_size() // 16
        self._keep = [d_shapes, d_vertices]
        self._check(self.lib.fclg_set_shapes_device(self.h, ctypes.c_void_p(d_shapes.data_ptr()), n_s,
                                                    ctypes.c_void_p(d_vertices.data_ptr()), n_v),
                    "fclg_set_shapes_device")

    def set_batch(self, batch):
        self.set_shapes(batch.shapes, batch.vertices)

    def _host_query(self, fn, pairs, request, out):
        p = np.ascontiguousarray(pairs, PAIR_DTYPE)
        if out is None:
            out = np.zeros(len(p), RESULT_DTYPE)
        req = ctypes.byref(request) if request is not None else None
        self._check(fn(self.h, _ptr(p), len(p), req, _ptr(out)), fn.__name__)
        return out

    def distance(self, pairs, request=None, out=None):
        """Signed distance per pair (host arrays in and out)."""
        return self._host_query(self.lib.fclg_distance, pairs, request, out)

    def distance64(self, pairs, request=None, out=None):
        """The GJK path of GJKSolver<double>::shapeDistance per pair in FP64 on the GPU
        (RESULT64_DTYPE out; request: a Request64 or None)."""
        if out is None:
            out = np.zeros(len(pairs), RESULT64_DTYPE)
        return self._host_query(self.lib.fclg_distance64, pairs, request, out)

    def distance64_device(self, d_pairs, n, d_results, request=None, stream=0):
        """Asynchronous FP64 separation distance on device pointers (fclg_result64 out)."""
        self._dev_query(self.lib.fclg_distance64_device, d_pairs, n, d_results, request, stream)

    def collide(self, pairs, request=None, out=None):
        """fcl::collide per pair (host arrays in and out)."""
        return self._host_query(self.lib.fclg_collide, pairs, request, out)

    def _dev_query(self, fn, d_pairs, n, d_results, request, stream):
        req = ctypes.byref(request) if request is not None else None
        st = ctypes.c_void_p(stream) if stream else None
        self._check(fn(self.h, ctypes.c_void_p(d_pairs), n, req, ctypes.c_void_p(d_results), st), fn.__name__)

    def distance_device(self, d_pairs, n, d_results, request=None, stream=0):
        """Asynchronous signed distance on device pointers (ints) on a CUDA stream handle."""
        self._dev_query(self.lib.fclg_distance_device, d_pairs, n, d_results, request, stream)

    def distance_device_static(self, d_pairs, n, d_results, request=None, stream=0):
        """distance_device without allocation in the call (at most STATIC_MAX_PAIRS pairs)."""
        self._dev_query(self.lib.fclg_distance_device_static, d_pairs, n, d_results, request, stream)

    def collide_device(self, d_pairs, n, d_results, request=None, stream=0):
        self._dev_query(self.lib.fclg_collide_device, d_pairs, n, d_results, request, stream)

    def set_launch(self, gjk_lanes=0, epa_ctas_per_sm=0):
        self._check(self.lib.fclg_set_launch(self.h, gjk_lanes, epa_ctas_per_sm), "fclg_set_launch")

    def set_tuning(self, **kw):
        """Fields of fclg_tuning by name; unspecified ones keep their value."""
        t = Tuning()
        for k, v in kw.items():
            if k in ("bucketing", "support_walk", "gjk_refill", "epa_resume") and isinstance(v, bool):
                v = 1 if v else -1
            setattr(t, k, int(v))
        self._check(self.lib.fclg_set_tuning(self.h, ctypes.byref(t)), "fclg_set_tuning")

    def get_tuning(self):
        t = Tuning()
        self._check(self.lib.fclg_get_tuning(self.h, ctypes.byref(t)), "fclg_get_tuning")
        return {name: getattr(t, name) for name, _ in Tuning._fields_}

    def set_profiling(self, enable=True):
        self._check(self.lib.fclg_set_profiling(self.h, int(enable)), "fclg_set_profiling")

    def pass_times(self, reset=True):
        """(gjk_ms, epa_ms, queries) summed since the last reset."""
        g, e, q = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
        self._check(self.lib.fclg_pass_times(self.h, ctypes.byref(g), ctypes.byref(e), ctypes.byref(q), int(reset)),
                    "fclg_pass_times")
        return g.value, e.value, q.value

    def mesh_traffic(self, reset=True):
        """(node pairs, triangle pairs) tested by mesh-mesh queries run while
        profiling was on, since the last reset."""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self.lib.fclg_mesh_traffic(self.h, ctypes.byref(a), ctypes.byref(b), int(reset)),
                    "fclg_mesh_traffic")
        return a.value, b.value

    @property
    def launch_count(self):
        return int(self.lib.fclg_launch_count(self.h))

    def collide_directed(self, pairs, dirs, request=None):
        """fcl::collide, directed penetration mode, host arrays: dirs float[n][3] (unit,
        shape b's escape direction in shape a's frame); with FCLG_REQ_INCREMENTAL in the
        request's flags the incremental minimum-distance mode from dirs as hints, and with
        FCLG_REQ_INCREMENTAL | FCLG_REQ_WARM_START from the context's model's directions
        (dirs None)."""
        p = np.ascontiguousarray(pairs, PAIR_DTYPE)
        d = None
        if dirs is not None:
            d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
            assert len(d) == len(p)
        out = np.zeros(len(p), RESULT_DTYPE)
        req = ctypes.byref(request) if request is not None else None
        self._check(self.lib.fclg_collide_directed(self.h, _ptr(p), len(p), _ptr(d) if d is not None else None,
                                                   req, _ptr(out)), "fclg_collide_directed")
        return out

    def translational_ccd(self, pairs, disp, toc_type=FCLG_TOC_NONE, max_gjk_iterations=0, gjk_tolerance=0.0,
                          zero_movement_tolerance=0.0, out=None):
        """fcl::translational_ccd on every pair, host arrays: disp = DISP_DTYPE rows or
        float[n][4] (unit axis in shape a's frame, distance); CCD_RESULT_DTYPE out (or
        written into `out`, e.g. a pinned array)."""
        p = np.ascontiguousarray(pairs, PAIR_DTYPE)
        d = np.ascontiguousarray(disp, np.float32).reshape(-1, 4) if not isinstance(disp, np.ndarray) or \
            disp.dtype != DISP_DTYPE else np.ascontiguousarray(disp).view(np.float32).reshape(-1, 4)
        assert len(d) == len(p)
        if out is None:
            out = np.zeros(len(p), CCD_RESULT_DTYPE)
        assert out.dtype == CCD_RESULT_DTYPE and len(out) == len(p) and out.flags.c_contiguous
        req = CcdRequest(toc_type, max_gjk_iterations, gjk_tolerance, 0, zero_movement_tolerance)
        self._check(self.lib.fclg_translational_ccd(self.h, _ptr(p), len(p), _ptr(d), ctypes.byref(req), _ptr(out)),
                    "fclg_translational_ccd")
        return out

    def translational_ccd_device(self, d_pairs, n, d_disp, d_results, toc_type=FCLG_TOC_NONE, stream=None):
        """The device entry on device pointers (stream: a CUDA stream handle or None)."""
        req = CcdRequest(toc_type, 0, 0.0, 0, 0.0)
        self._check(self.lib.fclg_translational_ccd_device(self.h, ctypes.c_void_p(d_pairs), n, ctypes.c_void_p(d_disp),
                                                           ctypes.byref(req), ctypes.c_void_p(d_results),
                                                           ctypes.c_void_p(stream) if stream else None),
                    "fclg_translational_ccd_device")

    def autotune(self, d_pairs, n, d_results, request=None, distance=True):
        """Times candidate launch shapes on the batch, keeps the fastest; returns (tuning dict, ms)."""
        t = Tuning()
        ms = ctypes.c_float()
        req = ctypes.byref(request) if request is not None else None
        self._check(self.lib.fclg_autotune(self.h, ctypes.c_void_p(d_pairs), n, req, ctypes.c_void_p(d_results),
                                           int(distance), ctypes.byref(t), ctypes.byref(ms)), "fclg_autotune")
        return {name: getattr(t, name) for name, _ in Tuning._fields_}, ms.value

    def graph(self, d_pairs, n, d_results, request=None, distance=True):
        """A CUDA graph of one query on these device buffers (QueryGraph)."""
        return QueryGraph(self, d_pairs, n, d_results, request, distance)

    def set_warmstart(self, model):
        """Model for queries with FCLG_REQ_WARM_START (None: none)."""
        self._check(self.lib.fclg_set_warmstart(self.h, model.h if model is not None else None),
                    "fclg_set_warmstart")
        self._warmstart = model


class QueryGraph:
    """fclg_graph_*: one captured query, replayed with launch()."""

    def __init__(self, ctx, d_pairs, n, d_results, request=None, distance=True):
        self.ctx = ctx
        h = ctypes.c_void_p()
        req = ctypes.byref(request) if request is not None else None
        ctx._check(ctx.lib.fclg_graph_create(ctx.h, ctypes.c_void_p(d_pairs), n, req, ctypes.c_void_p(d_results),
                                             int(distance), ctypes.byref(h)), "fclg_graph_create")
        self.h = h

    def launch(self, stream=0):
        st = ctypes.c_void_p(stream) if stream else None
        self.ctx._check(self.ctx.lib.fclg_graph_launch(self.ctx.h, self.h, st), "fclg_graph_launch")

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.fclg_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WarmStart:
    """The learned GJK warm-start model (fclg_warmstart_*) on one device.

    Device buffers are passed as integer pointers (e.g. torch tensors'
    data_ptr()): pairs fclg_pair[n], labels / outputs float32[n][3]."""

    def __init__(self, n_classes, seed=0, device=0):
        self.lib = load_library()
        self.n_classes = n_classes
        h = ctypes.c_void_p()
        rc = self.lib.fclg_warmstart_create(device, n_classes, seed, ctypes.byref(h))
        if rc != 0:
            raise FclgError("fclg_warmstart_create failed (%d)" % rc)
        self.h = h
        self.n_params = int(self.lib.fclg_warmstart_param_count(h))

    def _check(self, rc, what):
        if rc != 0:
            raise FclgError("%s failed (%d): %s" % (what, rc, self.lib.fclg_warmstart_last_error(self.h).decode()))

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        self._check(self.lib.fclg_warmstart_get_params(self.h, _ptr(p), self.n_params), "fclg_warmstart_get_params")
        return p

    def set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        self._check(self.lib.fclg_warmstart_set_params(self.h, _ptr(p), len(p)), "fclg_warmstart_set_params")

    def predict(self, d_pairs, n, d_out, normalize=True, mma_sync=False, stream=0):
        """Directions (or raw outputs) by the tcgen05 kernel, or the mma.sync one."""
        st = ctypes.c_void_p(stream) if stream else None
        flags = (1 if normalize else 0) | (2 if mma_sync else 0)
        self._check(self.lib.fclg_warmstart_predict(self.h, ctypes.c_void_p(d_pairs), n, ctypes.c_void_p(d_out),
                                                    flags, st), "fclg_warmstart_predict")

    def status(self):
        self._check(self.lib.fclg_warmstart_status(self.h), "fclg_warmstart_status")

    def forward(self, d_pairs, n, d_y, stream=0):
        st = ctypes.c_void_p(stream) if stream else None
        self._check(self.lib.fclg_warmstart_forward(self.h, ctypes.c_void_p(d_pairs), n, ctypes.c_void_p(d_y), st),
                    "fclg_warmstart_forward")

    def gradient(self, d_pairs, d_labels, n):
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.fclg_warmstart_gradient(self.h, ctypes.c_void_p(d_pairs), ctypes.c_void_p(d_labels), n,
                                                     _ptr(g), ctypes.byref(loss)), "fclg_warmstart_gradient")
        return loss.value, g

    def train(self, d_pairs, d_labels, n, epochs=4, batch=4096, lr=1e-3, lr_final=0.0, seed=0):
        cfg = TrainConfig(epochs, batch, lr, lr_final, seed, 0)
        losses = np.zeros(epochs, np.float32)
        self._check(self.lib.fclg_warmstart_train(self.h, ctypes.c_void_p(d_pairs), ctypes.c_void_p(d_labels), n,
                                                  ctypes.byref(cfg), _ptr(losses)), "fclg_warmstart_train")
        return losses

    def close(self):
        if getattr(self, "h", None):
            self.lib.fclg_warmstart_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def direction_labels(results):
    """Training targets from plain query results (RESULT_DTYPE): the unit vector
    p_a - p_b, i.e. the direction GJK's search ends at (its guess); rows
    without a valid answer get zeros and should be dropped."""
    v = results["p_a"].astype(np.float64) - results["p_b"].astype(np.float64)
    n = np.linalg.norm(v, axis=1, keepdims=True)
    ok = (results["ok"] == 1) & (n[:, 0] > 1e-9)
    u = np.where(ok[:, None], v / np.maximum(n, 1e-30), 0.0)
    return u.astype(np.float32), ok


class GpuMesh:
    """A triangle mesh with its OBB hierarchy on the context's device."""

    def __init__(self, ctx, vertices, triangles):
        self.ctx = ctx
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
        h = ctypes.c_void_p()
        ctx._check(ctx.lib.fclg_mesh_create(ctx.h, _ptr(v), len(v), _ptr(t), len(t), ctypes.byref(h)),
                   "fclg_mesh_create")
        self.h = h
        nn, nt = ctypes.c_uint32(), ctypes.c_uint32()
        ctx.lib.fclg_mesh_info(h, ctypes.byref(nn), ctypes.byref(nt))
        self.n_nodes, self.n_tris = nn.value, nt.value

    def export(self):
        """(nodes [n_nodes] MESH_NODE_DTYPE, triangles float32 [n_tris, 3, 4])."""
        nodes = np.zeros(self.n_nodes, MESH_NODE_DTYPE)
        tris = np.zeros((self.n_tris, 3, 4), np.float32)
        assert self.ctx.lib.fclg_mesh_export(self.h, _ptr(nodes), _ptr(tris)) == 0
        return nodes, tris

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.fclg_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def broadphase(ctx, shape_ids, poses, cap=None):
    """Overlapping object pairs (fclg_broadphase): objects = (shape of the
    context's set, world pose [12]).  Returns (pairs [m, 2] uint32 with i < j,
    aabbs [n, 6] float32 lo / hi); retries with room for every pair."""
    ids = np.ascontiguousarray(shape_ids, np.uint32)
    p = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = len(p)
    cap = 4 * n if cap is None else cap
    aabbs = np.zeros((n, 6), np.float32)
    while True:
        pairs = np.zeros((max(cap, 1), 2), np.uint32)
        m = ctypes.c_uint32(0)
        ctx._check(ctx.lib.fclg_broadphase(ctx.h, _ptr(ids), _ptr(p), n, _ptr(pairs), cap, ctypes.byref(m),
                                           _ptr(aabbs)), "fclg_broadphase")
        if m.value <= cap:
            return pairs[:m.value], aabbs
        cap = m.value


def mesh_shape_collide(ctx, mesh, shape_ids, poses, max_contacts=1):
    """fcl::collide(mesh, shape) per query, penetration off: shapes of the
    context's shape set, poses [n, 12] in the mesh frame.  Returns (flags,
    counts, tri_ids [n, max_contacts], status)."""
    ids = np.ascontiguousarray(shape_ids, np.uint32)
    p = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = len(p)
    flags = np.zeros(n, np.uint8)
    counts = np.zeros(n, np.uint32)
    tris = np.full((n, max_contacts), -1, np.int32)
    status = np.zeros(n, np.uint32)
    ctx._check(ctx.lib.fclg_mesh_shape_collide(ctx.h, mesh.h, _ptr(ids), _ptr(p), n, max_contacts, _ptr(flags),
                                               _ptr(counts), _ptr(tris), _ptr(status)), "fclg_mesh_shape_collide")
    return flags, counts, tris, status


def mesh_shape_contacts(ctx, mesh, shape_ids, poses, max_contacts=1):
    """fcl::collide(mesh, shape) per query with penetration on.  Returns
    (flags, counts, tri_ids [n, max_contacts], contacts [n, max_contacts, 8]
    float32 = pos, normal, depth, status bits (view the last column as
    uint32), status)."""
    ids = np.ascontiguousarray(shape_ids, np.uint32)
    p = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = len(p)
    flags = np.zeros(n, np.uint8)
    counts = np.zeros(n, np.uint32)
    tris = np.full((n, max_contacts), -1, np.int32)
    con = np.zeros((n, max_contacts, 8), np.float32)
    status = np.zeros(n, np.uint32)
    ctx._check(ctx.lib.fclg_mesh_shape_contacts(ctx.h, mesh.h, _ptr(ids), _ptr(p), n, max_contacts, _ptr(flags),
                                                _ptr(counts), _ptr(tris), _ptr(con), _ptr(status)),
               "fclg_mesh_shape_contacts")
    return flags, counts, tris, con, status


def mesh_collide(ctx, mesh_a, mesh_b, poses, max_contacts=1):
    """Boolean mesh-mesh collision per pose (host arrays): (flags, counts, pairs, status)."""
    p = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = len(p)
    flags = np.zeros(n, np.uint8)
    counts = np.zeros(n, np.uint32)
    pairs = np.full((n, max_contacts, 2), -1, np.int32)
    status = np.zeros(n, np.uint32)
    ctx._check(ctx.lib.fclg_mesh_collide(ctx.h, mesh_a.h, mesh_b.h, _ptr(p), n, max_contacts, _ptr(flags),
                                         _ptr(counts), _ptr(pairs), _ptr(status)), "fclg_mesh_collide")
    return flags, counts, pairs, status


def hull_graph(points):
    """Edge graph of the convex hull of ``points`` [n, 3 or 4] (fclg_hull_graph,
    host work): (starts[6], first[n + 1], adj), rows of adj ascending; None when
    the points span no volume."""
    lib = load_library()
    p = np.asarray(points, np.float32)
    n = len(p)
    xyzw = np.zeros((n, 4), np.float32)
    xyzw[:, :p.shape[1]] = p[:, :4]
    starts = np.zeros(6, np.uint32)
    first = np.zeros(n + 1, np.uint32)
    m = ctypes.c_uint32(0)
    rc = lib.fclg_hull_graph(_ptr(xyzw), n, _ptr(starts), _ptr(first), None, 0, ctypes.byref(m))
    if rc != 0:
        return None
    adj = np.zeros(max(m.value, 1), np.uint32)
    rc = lib.fclg_hull_graph(_ptr(xyzw), n, _ptr(starts), _ptr(first), _ptr(adj), len(adj), ctypes.byref(m))
    if rc != 0:
        raise FclgError("fclg_hull_graph failed (%d)" % rc)
    return starts, first, adj[:m.value]


def bvh_node_sizes(vertices, triangles):
    """Host-only: each node's FP64 |extent|^2 (the traversal's descend key) and
    the tree depth."""
    lib = load_library()
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    sizes = np.zeros(2 * len(t) - 1)
    depth = ctypes.c_uint32(0)
    rc = lib.fclg_bvh_node_sizes(_ptr(v), len(v), _ptr(t), len(t), _ptr(sizes), ctypes.byref(depth))
    if rc != 0:
        raise FclgError("fclg_bvh_node_sizes failed (%d)" % rc)
    return sizes, depth.value


def bvh_build(vertices, triangles):
    """Host-only BVH build: (nodes [2 nt - 1] MESH_NODE_DTYPE, triangles float32 [nt, 3, 4])."""
    lib = load_library()
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    nodes = np.zeros(2 * len(t) - 1, MESH_NODE_DTYPE)
    soup = np.zeros((len(t), 3, 4), np.float32)
    rc = lib.fclg_bvh_build(_ptr(v), len(v), _ptr(t), len(t), _ptr(nodes), _ptr(soup))
    if rc != 0:
        raise FclgError("fclg_bvh_build failed (%d)" % rc)
    return nodes, soup
