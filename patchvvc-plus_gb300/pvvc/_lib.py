"""Loads libpvvc_gb300.so (built in-tree next to this package) and declares
the C ABI of include/pvvc_gb300.h for ctypes.  There is no fallback: if the
library is missing, importing the decoder raises."""
from __future__ import annotations

import ctypes as C
import os

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_ROOT, "libpvvc_gb300.so")

u8p = C.POINTER(C.c_uint8)
f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u32p = C.POINTER(C.c_uint32)
i64p = C.POINTER(C.c_int64)
u64p = C.POINTER(C.c_uint64)
vp = C.c_void_p

STATUS = {
    0: "PVVC_OK", 1: "PVVC_ERR_ARG", 2: "PVVC_ERR_OVERRUN", 3: "PVVC_ERR_GEOMETRY", 4: "PVVC_ERR_SIZE",
    5: "PVVC_ERR_NO_REFERENCE", 6: "PVVC_ERR_BAD_SLICE", 7: "PVVC_ERR_NOMEM", 8: "PVVC_ERR_CUDA", 9: "PVVC_ERR_ZSTD",
    10: "PVVC_ERR_FORMAT", 11: "PVVC_ERR_CAPACITY", 12: "PVVC_ERR_TREE",
}


class BatchDesc(C.Structure):
    _fields_ = [("nslices", C.c_int32), ("slot", i32p), ("type", u8p), ("size", u32p), ("qp", u8p), ("mv", f32p),
                ("geo_off", u64p), ("geo_size", u32p), ("col_off", u64p), ("col_size", u32p), ("out_off", u64p)]


class Tune(C.Structure):
    _fields_ = [("group_ctas_per_sm", C.c_int32), ("min_group", C.c_int32), ("rlgr_block", C.c_int32),
                ("rlgr_long_ctas", C.c_int32), ("rlgr_mid_pct", C.c_int32), ("rlgr_long_lanes", C.c_int32)]


class PlanInfo(C.Structure):
    _fields_ = [("nslices", C.c_int32), ("nintra", C.c_int32), ("groups_a", C.c_int32), ("groups_b", C.c_int32),
                ("singles_a", C.c_int32), ("singles_b", C.c_int32), ("kernels", C.c_int32), ("group_ctas", C.c_int32),
                ("tune", Tune), ("clear_bytes", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_leaves", C.c_int32), ("max_nodes", C.c_int32),
                ("max_batch_points", C.c_uint64), ("ring_points", C.c_uint64), ("inflight", C.c_int32),
                ("max_batch_frames", C.c_int32), ("tune", Tune)]


class Completion(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("handle", C.c_uint64), ("stream_id", C.c_int32), ("status", C.c_int32),
                ("npoints", C.c_uint64), ("xyz", C.c_void_p), ("rgb", C.c_void_p), ("submit_us", C.c_double),
                ("launch_us", C.c_double), ("done_us", C.c_double), ("batch_id", C.c_int32), ("batch_frames", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("frames", C.c_uint64), ("points", C.c_uint64), ("slices", C.c_uint64),
                ("slots_total", C.c_uint64), ("slots_free", C.c_uint64), ("streams_open", C.c_uint64),
                ("reserved_bytes", C.c_uint64), ("gpu_busy_us", C.c_double)]


class IcpParams(C.Structure):
    _fields_ = [("max_corr_dist", C.c_float), ("max_iter", C.c_int32), ("fitness_eps", C.c_float),
                ("transform_eps", C.c_float), ("mse_abs_eps", C.c_float)]


class SynthConfig(C.Structure):
    _fields_ = [("grid_bits", C.c_int32), ("nprims", C.c_int32), ("axis_min", C.c_float), ("axis_max", C.c_float),
                ("target_points", C.c_int32), ("nframes", C.c_int32), ("gof", C.c_int32), ("size_mode", C.c_int32),
                ("size_a", C.c_float), ("size_b", C.c_float), ("size_min", C.c_float), ("size_max", C.c_float),
                ("qp_i", C.c_uint8), ("qp_p", C.c_uint8), ("rot_deg", C.c_float), ("trans_vox", C.c_float),
                ("jitter", C.c_float), ("color_noise", C.c_float), ("seed", C.c_uint64), ("nthreads", C.c_int32),
                ("zstd_level", C.c_int32)]


# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("pvvc_status_string", C.c_char_p, [C.c_int]),
    ("pvvc_state_create", C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(vp)]),
    ("pvvc_state_destroy", C.c_int, [vp]),
    ("pvvc_state_reset", C.c_int, [vp, vp]),
    ("pvvc_plan_create", C.c_int, [C.POINTER(BatchDesc), C.POINTER(vp)]),
    ("pvvc_plan_destroy", C.c_int, [vp]),
    ("pvvc_plan_query", C.c_int, [vp, u64p, u64p]),
    ("pvvc_plan_create_tuned", C.c_int, [C.POINTER(BatchDesc), C.POINTER(Tune), C.POINTER(vp)]),
    ("pvvc_plan_host_times", C.c_int, [vp, C.POINTER(C.c_double), C.c_int32]),
    ("pvvc_plan_info_get", C.c_int, [vp, C.POINTER(PlanInfo)]),
    ("pvvc_plan_autotune", C.c_int, [C.POINTER(BatchDesc), vp, vp, C.c_int32, vp, C.POINTER(Tune), f32p]),
    ("pvvc_graph_create", C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, C.c_uint64, C.POINTER(vp)]),
    ("pvvc_graph_launch", C.c_int, [vp, vp]),
    ("pvvc_graph_destroy", C.c_int, [vp]),
    ("pvvc_decode", C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, C.c_uint64, vp]),
    ("pvvc_decode_profiled", C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, C.c_uint64, vp, C.POINTER(vp)]),
    ("pvvc_decode_frames_host", C.c_int, [vp, C.c_int32, C.POINTER(u8p), u64p, f32p, u8p, C.c_uint64, u64p, i32p,
                                          C.c_int32, vp]),
    ("pvvc_host_stage_times", C.c_int, [C.POINTER(C.c_double), C.c_int32]),
    ("pvvc_zstd_inflate_batch", C.c_int, [C.c_int32, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("pvvc_zstd_content_size", C.c_int, [u8p, C.c_uint64, u64p]),
    ("pvvc_zstd_inflate_host", C.c_int, [u8p, C.c_uint64, u8p, C.c_uint64, u64p]),
    ("pvvc_launch_cudaProcess", C.c_int, [C.c_int, C.c_int, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                          C.c_int, vp]),
    ("pvvc_encode_patch_gop", C.c_int, [f32p, C.c_uint32, f32p, C.c_int32, u8p, u8p, C.c_uint64, u64p, u8p,
                                        C.c_uint64, u64p, u32p]),
    ("pvvc_rlgr_encode", C.c_int64, [i64p, C.c_uint64, u8p, C.c_uint64]),
    ("pvvc_patch_leaf_yuv", C.c_int, [f32p, C.c_uint32, f32p, C.c_int32, u8p, C.c_uint64, u64p, f32p, C.c_uint64,
                                      C.POINTER(C.c_uint32)]),
    ("pvvc_encoder_create", C.c_int, [C.POINTER(vp)]),
    ("pvvc_encoder_destroy", C.c_int, [vp]),
    ("pvvc_encode_colors", C.c_int, [vp, C.POINTER(BatchDesc), vp, vp, vp, vp, u64p, C.POINTER(C.c_uint32), vp, vp, vp]),
    ("pvvc_rlgr_decode_host", C.c_int, [u8p, C.c_uint64, C.c_uint64, i64p]),
    ("pvvc_icp_workspace_size", C.c_int, [C.c_int32, C.c_uint64, C.c_uint64, u64p]),
    ("pvvc_icp_batch", C.c_int, [C.c_int32, vp, vp, vp, vp, vp, C.POINTER(IcpParams), vp, vp, vp, vp, vp, C.c_uint64,
                                 C.c_uint64, C.c_uint64, vp]),
    ("pvvc_icp_batch_noalloc", C.c_int, [C.c_int32, vp, vp, vp, vp, vp, C.POINTER(IcpParams), vp, vp, vp, vp,
                                         C.c_uint64, vp]),
    ("pvvc_cloud_mse_batch", C.c_int, [C.c_int32, vp, vp, vp, vp, vp, vp, vp, C.c_uint64, C.c_uint64, C.c_uint64, vp]),
    ("pvvc_fitter_create", C.c_int, [C.POINTER(vp)]),
    ("pvvc_fitter_destroy", C.c_int, [vp]),
    ("pvvc_fitting_clouds", C.c_int, [vp, C.c_int32, i32p, u32p, f32p, u32p, C.c_float, C.c_float, C.c_int32, f32p,
                                      C.c_uint64, u64p, i32p, vp]),
    ("pvvc_cloud_quality_workspace_size", C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("pvvc_cloud_quality", C.c_int, [C.c_uint64, vp, vp, C.c_uint64, vp, vp, vp, vp, C.c_uint64, vp]),
    ("pvvc_knn_colors_workspace_size", C.c_int, [C.c_int32, C.c_uint64, u64p]),
    ("pvvc_knn_colors_batch", C.c_int, [C.c_int32, vp, vp, vp, vp, vp, vp, C.c_int32, vp, vp, vp, vp, vp, C.c_uint64,
                                        C.c_uint64, vp]),
    ("pvvc_gemm_bf16", C.c_int, [C.c_int32, C.c_int32, C.c_int32, vp, C.c_int64, vp, C.c_int64, vp, C.c_int64, vp, vp,
                                 C.c_int64, C.c_int32, C.c_int32, vp]),
    ("pvvc_device_error_take", C.c_int, [i32p]),
    ("pvvc_regnet_param_count", C.c_int, []),
    ("pvvc_regnet_create", C.c_int, [C.c_uint64, C.POINTER(vp)]),
    ("pvvc_regnet_destroy", C.c_int, [vp]),
    ("pvvc_regnet_get_params", C.c_int, [vp, f32p, C.c_int64]),
    ("pvvc_regnet_set_params", C.c_int, [vp, f32p, C.c_int64]),
    ("pvvc_regnet_train_step", C.c_int, [vp, C.c_int32, vp, vp, vp, vp, vp, vp, vp, C.c_uint64, vp, vp, vp]),
    ("pvvc_regnet_grad", C.c_int, [vp, C.c_int32, vp, vp, C.c_float, vp, vp, vp]),
    ("pvvc_propose", C.c_int, [vp, C.c_int32, vp, vp, vp, vp, C.c_uint64, vp, vp]),
    ("pvvc_regnet_outputs", C.c_int, [vp, C.c_int32, vp, vp]),
    ("pvvc_server_create", C.c_int, [C.POINTER(ServerConfig), C.POINTER(vp)]),
    ("pvvc_server_destroy", C.c_int, [vp]),
    ("pvvc_server_open_stream", C.c_int, [vp, C.c_int32, i32p]),
    ("pvvc_server_close_stream", C.c_int, [vp, C.c_int32]),
    ("pvvc_server_submit", C.c_int, [vp, C.c_int32, vp, C.c_uint64, C.c_uint64]),
    ("pvvc_server_poll", C.c_int, [vp, C.POINTER(Completion), C.c_int32, i32p, C.c_int32]),
    ("pvvc_server_read", C.c_int, [vp, C.c_uint64, f32p, u8p]),
    ("pvvc_server_release", C.c_int, [vp, C.c_uint64]),
    ("pvvc_server_stats_get", C.c_int, [vp, C.POINTER(ServerStats)]),
    # synthetic sequences (not part of the drop-in boundary)
    ("pvvc_synth_create", C.c_int, [C.POINTER(SynthConfig), C.POINTER(vp)]),
    ("pvvc_synth_destroy", None, [vp]),
    ("pvvc_synth_gof_count", C.c_int32, [vp]),
    ("pvvc_synth_patch_count", C.c_int32, [vp, C.c_int32]),
    ("pvvc_synth_patch", C.c_int, [vp, C.c_int32, C.c_int32, f32p, f32p, f32p, u32p, i32p]),
    ("pvvc_synth_encode", C.c_int, [vp]),
    ("pvvc_synth_frame", C.c_int, [vp, C.c_int32, C.POINTER(u8p), u64p]),
    ("pvvc_synth_frame_points", C.c_uint64, [vp, C.c_int32]),
]

_LIB = None


def lib():
    """The loaded library.  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it first (python patchvvc-plus_gb300/build.py)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class PvvcError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)} ({lib().pvvc_status_string(status).decode()})")


def check(status: int, what: str = "") -> None:
    if status != 0:
        raise PvvcError(status, what)


def build_library(verbose: bool = False) -> str:
    """Compile libpvvc_gb300.so in-tree (patchvvc-plus_gb300/build.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("pvvc_gb300_build", os.path.join(_PKG_ROOT, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose)
