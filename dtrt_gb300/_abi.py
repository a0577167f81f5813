"""ctypes mirror of include/dtrt_gb300.h and the loader of the CUDA library.

The structures here are the plain-C scene description every entry point of
``libdtrt_gb300.so`` consumes. The loader fails loudly when the library is
missing: there is no CPU fallback for the render path.
"""
import ctypes
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libdtrt_gb300.so")

c_float_p = ctypes.POINTER(ctypes.c_float)
c_int_p = ctypes.POINTER(ctypes.c_int)

(DTRT_OK, DTRT_ERR_INVALID, DTRT_ERR_CUDA, DTRT_ERR_OVERFLOW, DTRT_ERR_UNSUPPORTED, DTRT_ERR_IO, DTRT_ERR_STEP_CAP,
 DTRT_ERR_NO_DEVICE) = range(8)
STATUS_NAMES = {
    0: "OK", 1: "INVALID", 2: "CUDA", 3: "OVERFLOW", 4: "UNSUPPORTED", 5: "IO", 6: "STEP_CAP", 7: "NO_DEVICE",
}

BSDF_NULL, BSDF_DIFFUSE, BSDF_PHONG, BSDF_ROUGHDIELECTRIC = 0, 1, 2, 3
PHASE_ISOTROPIC, PHASE_HG = 0, 1
EMITTER_AREA, EMITTER_AREA_EX = 0, 1
MEDIUM_HOMOGENEOUS, MEDIUM_HETEROGENEOUS = 0, 1

MODE_EMISSION = 0x01
MODE_SURFACE_MAIN = 0x02
MODE_SURFACE_BOUNDARY = 0x04
MODE_VOLUME_MAIN = 0x08
MODE_VOLUME_BOUNDARY1 = 0x10
MODE_VOLUME_BOUNDARY2 = 0x20
MODE_ALL = 0x3F


class CameraDesc(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("cam_to_world", c_float_p), ("cam_to_ndc", c_float_p),
        ("clip_near", ctypes.c_float), ("med_id", ctypes.c_int),
        ("velocities", c_float_p),
        ("crop_offset_x", ctypes.c_int), ("crop_offset_y", ctypes.c_int),
        ("crop_width", ctypes.c_int), ("crop_height", ctypes.c_int),
    ]


class ShapeDesc(ctypes.Structure):
    _fields_ = [
        ("vertices", c_float_p), ("indices", c_int_p), ("uvs", c_float_p), ("normals", c_float_p),
        ("num_vertices", ctypes.c_int), ("num_triangles", ctypes.c_int),
        ("light_id", ctypes.c_int), ("bsdf_id", ctypes.c_int),
        ("med_int_id", ctypes.c_int), ("med_ext_id", ctypes.c_int),
        ("velocities", c_float_p),
    ]


class BsdfDesc(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int),
        ("diffuse", ctypes.c_float * 3), ("specular", ctypes.c_float * 3), ("exponent", ctypes.c_float),
        ("alpha", ctypes.c_float), ("int_ior", ctypes.c_float), ("ext_ior", ctypes.c_float),
        ("d_diffuse", c_float_p), ("d_specular", c_float_p), ("d_exponent", c_float_p),
        ("d_alpha", c_float_p), ("d_eta", c_float_p),
    ]


class EmitterDesc(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int), ("shape_id", ctypes.c_int), ("intensity", ctypes.c_float * 3),
        ("two_sided", ctypes.c_int), ("kappa", ctypes.c_float),
        ("d_intensity", c_float_p), ("d_kappa", c_float_p),
    ]


class PhaseDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("g", ctypes.c_float), ("d_g", c_float_p)]


class MediumDesc(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int), ("phase_id", ctypes.c_int),
        ("sigma_t", ctypes.c_float), ("albedo", ctypes.c_float * 3),
        ("d_sigma_t", c_float_p), ("d_albedo", c_float_p),
        ("density_file", ctypes.c_char_p), ("density", c_float_p), ("res", ctypes.c_int * 3),
        ("vol_min", ctypes.c_float * 3), ("vol_max", ctypes.c_float * 3),
        ("albedo_file", ctypes.c_char_p), ("albedo_grid", c_float_p), ("albedo_res", ctypes.c_int * 3),
        ("albedo_min", ctypes.c_float * 3), ("albedo_max", ctypes.c_float * 3),
        ("to_world", ctypes.c_float * 16), ("density_scale", ctypes.c_float),
        ("d_density_scale", c_float_p), ("trans_velocities", c_float_p), ("rot_velocities", c_float_p),
    ]


class SceneDesc(ctypes.Structure):
    _fields_ = [
        ("nder", ctypes.c_int),
        ("camera", CameraDesc),
        ("num_shapes", ctypes.c_int), ("shapes", ctypes.POINTER(ShapeDesc)),
        ("num_bsdfs", ctypes.c_int), ("bsdfs", ctypes.POINTER(BsdfDesc)),
        ("num_emitters", ctypes.c_int), ("emitters", ctypes.POINTER(EmitterDesc)),
        ("num_phases", ctypes.c_int), ("phases", ctypes.POINTER(PhaseDesc)),
        ("num_media", ctypes.c_int), ("media", ctypes.POINTER(MediumDesc)),
        ("edge_weights", c_float_p),
    ]


class RenderOptions(ctypes.Structure):
    _fields_ = [
        ("seed", ctypes.c_uint64), ("spp", ctypes.c_int), ("max_bounces", ctypes.c_int),
        ("sppe", ctypes.c_int), ("sppse", ctypes.c_int), ("quiet", ctypes.c_int),
        ("mode", ctypes.c_int), ("ddist_coeff", ctypes.c_float),
    ]


class RenderStats(ctypes.Structure):
    _fields_ = [
        ("camera_paths", ctypes.c_uint64), ("edge_records", ctypes.c_uint64), ("edge_samples", ctypes.c_uint64),
        ("lins_records", ctypes.c_uint64), ("primary_edge_samples", ctypes.c_uint64),
        ("li_tasks", ctypes.c_uint64), ("rays", ctypes.c_uint64), ("node_visits", ctypes.c_uint64),
        ("tri_tests", ctypes.c_uint64), ("grid_lookups", ctypes.c_uint64), ("batches", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
        ("k_rays", ctypes.c_uint64 * 5), ("k_node_visits", ctypes.c_uint64 * 5),
        ("k_tri_tests", ctypes.c_uint64 * 5), ("k_grid_lookups", ctypes.c_uint64 * 5),
        ("ms_total", ctypes.c_double), ("ms_camera", ctypes.c_double), ("ms_edge", ctypes.c_double),
        ("ms_li", ctypes.c_double), ("ms_primary", ctypes.c_double), ("ms_setup", ctypes.c_double),
        ("counters_enabled", ctypes.c_int), ("camera_schedule", ctypes.c_int),
        ("light_samples", ctypes.c_uint64), ("k_light_samples", ctypes.c_uint64 * 5),
        ("camera_state_bytes", ctypes.c_uint64),
    ]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if isinstance(v, ctypes.Array) else v
        return d


BVH_AUTO, BVH_HOST, BVH_DEVICE = 0, 1, 2
BVH_DEVICE_MIN_TRIS = 65536


class BvhInfo(ctypes.Structure):
    _fields_ = [("builder", ctypes.c_int), ("refit", ctypes.c_int), ("num_nodes", ctypes.c_int),
                ("max_depth", ctypes.c_int), ("ms_build", ctypes.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


BATCH_MAX_ITEMS, BATCH_MAX_TRIALS = 256, 16
BATCH_AUTOTUNE, BATCH_GRAPH, BATCH_TUNE_FULL, BATCH_WAVEFRONT = 1, 2, 4, 8


class BatchItem(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("opts", RenderOptions), ("d_image", ctypes.c_void_p),
                ("image", ctypes.c_void_p), ("d_density", ctypes.c_void_p), ("d_vertices", ctypes.c_void_p)]


class BatchStats(ctypes.Structure):
    _fields_ = [
        ("num_items", ctypes.c_int), ("total_paths", ctypes.c_uint64), ("grid_blocks", ctypes.c_int),
        ("blocks_per_sm", ctypes.c_int), ("schedule", ctypes.c_int), ("streams", ctypes.c_int),
        ("chunk_paths", ctypes.c_int), ("order_longest_first", ctypes.c_int),
        ("graph", ctypes.c_int), ("num_trials", ctypes.c_int),
        ("trial_chunk", ctypes.c_int * BATCH_MAX_TRIALS), ("trial_order", ctypes.c_int * BATCH_MAX_TRIALS),
        ("trial_ms", ctypes.c_float * BATCH_MAX_TRIALS), ("tune_sample_stride", ctypes.c_int64),
        ("full_ms", ctypes.c_float * 4),
        ("item_ms_estimate", ctypes.c_double * BATCH_MAX_ITEMS), ("order", ctypes.c_int * BATCH_MAX_ITEMS),
        ("full_ms_wavefront", ctypes.c_float), ("wave_capacity", ctypes.c_int64), ("vertex_items", ctypes.c_int),
    ]

    def as_dict(self):
        n, t = self.num_items, self.num_trials
        names = {0: "persistent", 1: "per_item_launches", 2: "wavefront"}

        def trial(c):
            return "per_item_launches" if c < 0 else "wavefront" if c == 0 else "persistent"
        return {"num_items": n, "total_paths": self.total_paths, "grid_blocks": self.grid_blocks,
                "blocks_per_sm": self.blocks_per_sm,
                "schedule": names.get(self.schedule, "?"), "streams": self.streams,
                "chunk_paths": self.chunk_paths,
                "order_longest_first": bool(self.order_longest_first), "graph": bool(self.graph),
                "trials": [{"schedule": trial(self.trial_chunk[i]),
                            "chunk": max(self.trial_chunk[i], 0), "streams": max(-self.trial_chunk[i], 1),
                            "order": "longest_first" if self.trial_order[i] == 0 else "input",
                            "ms": self.trial_ms[i]} for i in range(t)],
                "tune_sample_stride": self.tune_sample_stride,
                "full_size_ms": {"persistent": self.full_ms[0], "per_item_1": self.full_ms[1],
                                 "per_item_2": self.full_ms[2], "per_item_4": self.full_ms[3],
                                 "wavefront": self.full_ms_wavefront},
                "wave_capacity": self.wave_capacity, "vertex_items": self.vertex_items,
                "item_ms_estimate": list(self.item_ms_estimate[:min(n, BATCH_MAX_ITEMS)]),
                "order": list(self.order[:min(n, BATCH_MAX_ITEMS)])}


UPDATE_REBUILD_BVH = 1
CAMERA_AUTO, CAMERA_MEGAKERNEL, CAMERA_WAVEFRONT = 0, 1, 2


class UpdateStats(ctypes.Structure):
    _fields_ = [("bvh_refit", ctypes.c_int), ("buffers_reused", ctypes.c_int), ("buffers_allocated", ctypes.c_int),
                ("sah_ratio", ctypes.c_float), ("host_ms", ctypes.c_double), ("ms_bvh", ctypes.c_double),
                ("ms_arrays", ctypes.c_double), ("ms_device", ctypes.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# Every C-ABI symbol declared in include/dtrt_gb300.h, with its ctypes signature.
EST_SCATTER_SEGMENT_FROM_ORIGIN = 1

_SIGNATURES = {
    "dtrt_abi_version": (ctypes.c_int, []),
    "dtrt_device_count": (ctypes.c_int, []),
    "dtrt_nder_supported": (ctypes.c_int, [ctypes.c_int]),
    "dtrt_last_error": (ctypes.c_char_p, []),
    "dtrt_scene_create": (ctypes.c_int, [ctypes.POINTER(SceneDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "dtrt_scene_set_edge_weights": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_int]),
    "dtrt_scene_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dtrt_release_cached_memory": (ctypes.c_int, []),
    "dtrt_scene_update": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SceneDesc), ctypes.c_uint,
                                         ctypes.POINTER(UpdateStats)]),
    "dtrt_render_fwd": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptions), ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_void_p]),
    "dtrt_render_fwd_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptions), ctypes.c_void_p,
                                               ctypes.c_int, ctypes.c_void_p]),
    "dtrt_render_primal": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptions), ctypes.c_void_p,
                                          ctypes.c_int, ctypes.c_void_p]),
    "dtrt_scene_enable_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dtrt_scene_last_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderStats)]),
    "dtrt_scene_set_queue_capacity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "dtrt_scene_set_tracking_cap": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dtrt_scene_set_camera_schedule": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dtrt_scene_set_estimator_flags": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint]),
    "dtrt_scene_gradient_sizes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                                 ctypes.POINTER(ctypes.c_int64)]),
    "dtrt_scene_set_density": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p]),
    "dtrt_scene_set_density_derivatives": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p]),
    "dtrt_render_adjoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptions), ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p]),
    "dtrt_batch_create": (ctypes.c_int, [ctypes.POINTER(BatchItem), ctypes.c_int, ctypes.c_uint, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "dtrt_batch_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dtrt_batch_stats_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchStats)]),
    "dtrt_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dtrt_trace_closest": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_int, c_int_p, c_float_p]),
    "dtrt_vol_read": (ctypes.c_int, [ctypes.c_char_p, c_int_p, c_int_p, c_float_p, c_float_p, c_float_p]),
    "dtrt_set_bvh_builder": (ctypes.c_int, [ctypes.c_int]),
    "dtrt_scene_bvh_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BvhInfo)]),
    "dtrt_rng_sequence": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_uint32), c_float_p, ctypes.POINTER(ctypes.c_double)]),
}

_lib = None


class DtrtError(RuntimeError):
    """A non-zero status from the C ABI, with its dtrt_last_error() message."""

    def __init__(self, status, message):
        super().__init__(f"dtrt status {status} ({STATUS_NAMES.get(status, '?')}): {message}")
        self.status = status


def load(path=None):
    """Load libdtrt_gb300.so (built by __graft_entry__.build()). Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("DTRT_GB300_LIB", LIB_PATH)
    if not os.path.exists(p):
        raise ImportError(
            f"dtrt_gb300 CUDA library not found at {p}; build it with "
            "`python -c \"import __graft_entry__ as g; g.build()\"` (no CPU fallback exists)")
    lib = ctypes.CDLL(p)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.dtrt_abi_version() != 1:
        raise ImportError("dtrt_gb300 ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def check(status):
    if status != DTRT_OK:
        msg = _lib.dtrt_last_error().decode() if _lib is not None else "?"
        raise DtrtError(status, msg)
    return status


def declared_symbols(header=None):
    """Function names declared in include/dtrt_gb300.h (for the export test)."""
    import re
    h = header or os.path.join(os.path.dirname(_HERE), "include", "dtrt_gb300.h")
    text = open(h).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(dtrt_\w+)\s*\(", text, re.M)))


if __name__ == "__main__":  # pragma: no cover
    print(declared_symbols(), file=sys.stderr)
