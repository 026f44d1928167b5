"""ctypes binding of libasv.so (include/asv.h, include/asv_host.h).

The library is built in-tree by `_build.build()`; loading never falls back to
anything else: a missing or stale library is an error.
"""
import ctypes
import os

from . import _build

c_int, c_float, c_size_t, c_void_p, c_char_p = (ctypes.c_int, ctypes.c_float, ctypes.c_size_t,
                                                ctypes.c_void_p, ctypes.c_char_p)
P = ctypes.POINTER

ASV_OK = 0
ASV_ERR_BAD_ARG = 1
ASV_ERR_OOM = 2
ASV_ERR_OVER_BUDGET = 3
ASV_ERR_TIMEOUT = 4
ASV_ERR_CUDA = 5
ASV_ERR_STATE = 6
ASV_ERR_NO_DEVICE = 7
REQ_CLIP = 0
REQ_WINDOW = 1
VARIANT_PLAIN = 0
VARIANT_STREAM = 1


class Config(ctypes.Structure):
    _fields_ = [("variant", c_int), ("lloyd_iters", c_int), ("full_ladder", c_int),
                ("middlebury", c_int), ("density_adjust", c_int), ("device", c_int),
                ("stream", c_void_p), ("hbm_budget", c_size_t), ("use_graph", c_int),
                ("instrument", c_int), ("jfa_zrun", c_int), ("jfa_tile_blocks", c_int)]


class Info(ctypes.Structure):
    _fields_ = [("W", c_int), ("H", c_int), ("D", c_int), ("K", c_int), ("Kp", c_int),
                ("s", c_int), ("ratio", c_float), ("passes", c_int), ("steps", c_int * 32),
                ("dead", c_int), ("neg_count", c_int), ("final_label_num", c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("jfa_ms", ctypes.c_double), ("jfa_launches", c_int),
                ("centroid_ms", ctypes.c_double), ("metric_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("launches", c_int), ("window_ms", ctypes.c_double)]


class StreamInfo(ctypes.Structure):
    _fields_ = [(n, c_int) for n in ("blocks", "next_block", "block_start", "block_end",
                                     "frames_needed", "seeds_placed", "block_Kp")]


class Request(ctypes.Structure):
    _fields_ = [("kind", c_int), ("session", c_int), ("W", c_int), ("H", c_int), ("D", c_int),
                ("K", c_int), ("rgb", c_void_p), ("fwd", c_void_p), ("bwd", c_void_p),
                ("labels_out", c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("failed", ctypes.c_longlong), ("queued", ctypes.c_longlong),
                ("running", ctypes.c_longlong), ("bytes_in_use", c_size_t), ("budget", c_size_t),
                ("slots", c_int), ("sessions", c_int)]


class Eval(ctypes.Structure):
    _fields_ = [("undersegmentation", ctypes.c_double), ("segmentation_accuracy", ctypes.c_double),
                ("boundary_recall", ctypes.c_double), ("mean_duration", ctypes.c_double),
                ("supervoxels", c_int), ("truth_segments", c_int), ("truth_boundary", ctypes.c_longlong),
                ("recalled", ctypes.c_longlong)]


class SynthParams(ctypes.Structure):
    _fields_ = [("W", c_int), ("H", c_int), ("frame0", c_int), ("nframes", c_int),
                ("n_ellipses", c_int), ("noise_sigma", c_float), ("vmax", c_float),
                ("jitter", c_float), ("drift_amp", c_float), ("drift_period", c_float),
                ("seed", ctypes.c_uint64)]


# name -> (restype, argtypes); every function declared in include/asv*.h
class RenderOptions(ctypes.Structure):
    _fields_ = [(n, c_int) for n in ("lloyd_iters", "write_txt", "write_render", "connectivity", "device",
                                     "verbose")]


SIGNATURES = {
    "asv_config_default": (None, [P(Config)]),
    "asv_create": (c_int, [P(Config), P(c_void_p)]),
    "asv_destroy": (c_int, [c_void_p]),
    "asv_last_error": (c_char_p, [c_void_p]),
    "asv_status_string": (c_char_p, [c_int]),
    "asv_version": (c_int, []),
    "asv_init_gpu": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int]),
    "asv_init_gpu_bgr": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int]),
    "asv_upload_flow": (c_int, [c_void_p, c_void_p, c_void_p]),
    "asv_initialization": (c_int, [c_void_p]),
    "asv_compute_flow": (c_int, [c_void_p]),
    "asv_seed_matrix": (c_int, [c_void_p]),
    "asv_rgb2lab": (c_int, [c_void_p]),
    "asv_ld_first_init": (c_int, [c_void_p]),
    "asv_flood": (c_int, [c_void_p, c_int]),
    "asv_centroids_next_seeds": (c_int, [c_void_p, c_int]),
    "asv_ld_next_seeds_matrix": (c_int, [c_void_p, c_int]),
    "asv_check_dead_seeds": (c_int, [c_void_p, c_void_p]),
    "asv_run_lloyd": (c_int, [c_void_p]),
    "asv_enforce_connectivity": (c_int, [c_void_p, c_int, c_void_p, P(c_int)]),
    "asv_enforce_connectivity_labels": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p,
                                                P(c_int)]),
    "asv_autotune": (c_int, [c_void_p, P(c_int)]),
    "asv_segment_clip": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int,
                                 c_int, c_void_p]),
    "asv_get_info": (c_int, [c_void_p, P(Info)]),
    "asv_get_labels": (c_int, [c_void_p, c_void_p]),
    "asv_get_raw_labels": (c_int, [c_void_p, c_void_p]),
    "asv_get_flow": (c_int, [c_void_p, c_void_p, c_void_p]),
    "asv_evaluate": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p]),
    "asv_get_seeds": (c_int, [c_void_p, c_void_p]),
    "asv_set_seeds": (c_int, [c_void_p, c_void_p, c_int]),
    "asv_get_lab": (c_int, [c_void_p, c_void_p]),
    "asv_get_sums": (c_int, [c_void_p, c_void_p]),
    "asv_check_dead_seeds_host": (c_int, [c_void_p, c_void_p, c_void_p]),
    "asv_jfa_pass_host": (c_int, [c_void_p, c_int, c_float, c_void_p, c_void_p]),
    "asv_get_stats": (c_int, [c_void_p, P(Stats)]),
    "asv_get_stream": (c_int, [c_void_p, P(c_void_p)]),
    "asv_synchronize": (c_int, [c_void_p]),
    "asv_clip_bytes": (c_size_t, [c_int, c_int, c_int, c_int]),
    "asv_check_dead_seeds_noalloc": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                             c_void_p]),
    "asv_batch_init": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "asv_batch_upload": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "asv_batch_get_labels": (c_int, [c_void_p, c_int, c_void_p]),
    "asv_batch_get_info": (c_int, [c_void_p, c_int, P(Info)]),
    "asv_batch_bytes": (c_size_t, [c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "asv_server_create": (c_int, [P(Config), c_int, c_size_t, P(c_void_p)]),
    "asv_server_destroy": (c_int, [c_void_p]),
    "asv_server_open_session": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, P(c_int)]),
    "asv_server_submit": (c_int, [c_void_p, c_void_p, P(ctypes.c_longlong)]),
    "asv_server_wait": (c_int, [c_void_p, ctypes.c_longlong, P(ctypes.c_double), P(ctypes.c_double),
                                P(c_int)]),
    "asv_server_poll": (c_int, [c_void_p, ctypes.c_longlong, P(c_int)]),
    "asv_server_get_stats": (c_int, [c_void_p, c_void_p]),
    "asv_stream_begin": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int]),
    "asv_stream_info_get": (c_int, [c_void_p, c_void_p]),
    "asv_stream_push": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, P(c_int)]),
    "asv_stream_block": (c_int, [c_void_p, c_int, P(c_int), P(c_int), P(c_int)]),
    "asv_stream_feed": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "asv_stream_feed_bgr": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "asv_stream_push_fed": (c_int, [c_void_p, c_void_p, P(c_int)]),
    "asv_stream_push_fed_async": (c_int, [c_void_p, c_void_p]),
    "asv_stream_wait": (c_int, [c_void_p, P(c_int), P(c_int)]),
    # include/asv_host.h
    "asv_synth_clip": (c_int, [P(SynthParams), c_void_p, c_void_p, c_void_p]),
    "asv_synth_truth": (c_int, [P(SynthParams), c_void_p]),
    "asv_preprocess_frame": (c_int, [c_void_p, c_int, c_int, c_void_p]),
    "asv_write_labels_txt": (c_int, [c_char_p, c_void_p, c_int, c_int, c_int]),
    "asv_write_render_ppm": (c_int, [c_char_p, c_void_p, c_int, c_int, c_int, c_int]),
    "asv_png_info": (c_int, [c_char_p, P(c_int), P(c_int)]),
    "asv_png_read_bgr": (c_int, [c_char_p, c_void_p, c_int, c_int]),
    "asv_png_read_frames_bgr": (c_int, [P(c_char_p), c_int, c_int, c_int, c_void_p]),
    "asv_png_write_rgb": (c_int, [c_char_p, c_void_p, c_int, c_int]),
    "asv_render_rgb": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p]),
    "asv_write_render_png": (c_int, [c_char_p, c_void_p, c_int, c_int, c_int, c_int, c_int]),
    "asv_frame_info": (c_int, [c_char_p, P(c_int), P(c_int)]),
    "asv_frame_read_bgr": (c_int, [c_char_p, c_void_p, c_int, c_int]),
    "asv_frames_read_bgr": (c_int, [P(c_char_p), c_int, c_int, c_int, c_void_p]),
    "asv_render_options_default": (None, [P(RenderOptions)]),
    "asv_render_run": (c_int, [c_char_p, c_char_p, c_char_p, c_char_p, c_int, c_float, P(RenderOptions)]),
    "asv_render_stream_run": (c_int, [c_char_p, c_char_p, c_char_p, c_char_p, c_int, c_float, P(RenderOptions)]),
}

_LIB = None


def load(build=True):
    """Loads libasv.so (building it first when asked and stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("libasv.so is not built; run __graft_entry__.build()")
    lib = ctypes.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class AsvError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status
