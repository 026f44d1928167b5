"""Python mirror of the reference's Image/Render operator surface over libasv.

`Image` has one method per method of the reference's `Image` class
(GPU-AS/Image.h:73-88), each a thin call into the C ABI; `Render.run` is the
plain per-clip pipeline of `Render::run` (GPU-AS/Render.cpp:100-350) with
host buffers in and labels out.  Everything runs on the CUDA path of
libasv.so; there is no CPU fallback.
"""
import collections
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import AsvError, Config, Info, Stats, SynthParams


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def synth_clip(W, H, D, n_ellipses=12, noise_sigma=5.0, vmax=3.0, jitter=0.0, drift_amp=0.0,
               drift_period=60.0, seed=1, frame0=0):
    """Seeded synthetic clip (rgb uint8 [D,H,W,3], fwd/bwd float32 [D,H,W,2])."""
    lib = _lib.load()
    rgb = np.empty((D, H, W, 3), np.uint8)
    fwd = np.empty((D, H, W, 2), np.float32)
    bwd = np.empty((D, H, W, 2), np.float32)
    p = SynthParams(W, H, frame0, D, n_ellipses, noise_sigma, vmax, jitter, drift_amp,
                    drift_period, seed)
    if lib.asv_synth_clip(ctypes.byref(p), _ptr(rgb), _ptr(fwd), _ptr(bwd)) != 0:
        raise ValueError("bad synthetic clip parameters")
    return rgb, fwd, bwd


def synth_truth(W, H, D, n_ellipses=12, noise_sigma=5.0, vmax=3.0, jitter=0.0, drift_amp=0.0,
                drift_period=60.0, seed=1, frame0=0):
    """Ground-truth ids [D,H,W] int32 of synth_clip with the same arguments:
    the ellipse on top of each pixel, n_ellipses for the background."""
    lib = _lib.load()
    ids = np.empty((D, H, W), np.int32)
    p = SynthParams(W, H, frame0, D, n_ellipses, noise_sigma, vmax, jitter, drift_amp,
                    drift_period, seed)
    if lib.asv_synth_truth(ctypes.byref(p), _ptr(ids)) != 0:
        raise ValueError("bad synthetic clip parameters")
    return ids


def config(variant=_lib.VARIANT_PLAIN, lloyd_iters=20, full_ladder=0, middlebury=0,
           density_adjust=1, device=0, stream=None, hbm_budget=0, use_graph=1, instrument=0,
           jfa_zrun=0, jfa_tile_blocks=0):
    c = Config()
    _lib.load().asv_config_default(ctypes.byref(c))
    c.variant, c.lloyd_iters, c.full_ladder, c.middlebury = variant, lloyd_iters, full_ladder, middlebury
    c.density_adjust, c.device, c.stream, c.hbm_budget = density_adjust, device, stream, hbm_budget
    c.use_graph, c.instrument, c.jfa_zrun, c.jfa_tile_blocks = use_graph, instrument, jfa_zrun, jfa_tile_blocks
    return c


class Image:
    """One clip on the GPU; methods follow the reference's Image class."""

    def __init__(self, cfg=None, **kw):
        self.lib = _lib.load()
        self.cfg = cfg if cfg is not None else config(**kw)
        h = ctypes.c_void_p()
        st = self.lib.asv_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if st != _lib.ASV_OK:
            raise AsvError(st, self.lib.asv_status_string(st).decode())
        self.h = h
        self.shape = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.asv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        if st != _lib.ASV_OK:
            raise AsvError(st, self.lib.asv_last_error(self.h).decode())

    # --- reference Image methods ------------------------------------------
    def init_gpu(self, rgb, K):
        rgb = np.ascontiguousarray(rgb, np.uint8)
        D, H, W, _ = rgb.shape
        self._ck(self.lib.asv_init_gpu(self.h, _ptr(rgb), W, H, D, K))
        self.shape = (D, H, W)

    def init_gpu_bgr(self, bgr, K):
        """init_gpu for raw BGR frames [D,H,W,3] (top row first): blur, BGR->RGB
        and flip on the device (Render::cvMat2TexureInput)."""
        bgr = np.ascontiguousarray(bgr, np.uint8)
        D, H, W, _ = bgr.shape
        self._ck(self.lib.asv_init_gpu_bgr(self.h, _ptr(bgr), W, H, D, K))
        self.shape = (D, H, W)

    def upload_flow(self, fwd, bwd):
        fwd = np.ascontiguousarray(fwd, np.float32)
        bwd = np.ascontiguousarray(bwd, np.float32)
        self._ck(self.lib.asv_upload_flow(self.h, _ptr(fwd), _ptr(bwd)))

    def compute_flow(self):
        """forward_backward_flow on the device (asv_compute_flow), instead of upload_flow"""
        self._ck(self.lib.asv_compute_flow(self.h))

    def flow(self):
        """(fwd, bwd) flow volumes [D,H,W,2] of a one-clip context"""
        D, H, W = self.shape
        fwd = np.empty((D, H, W, 2), np.float32)
        bwd = np.empty((D, H, W, 2), np.float32)
        self._ck(self.lib.asv_get_flow(self.h, _ptr(fwd), _ptr(bwd)))
        return fwd, bwd

    def initialization(self):
        self._ck(self.lib.asv_initialization(self.h))

    def seed_matrix(self):
        self._ck(self.lib.asv_seed_matrix(self.h))

    def RGB2LAB(self):
        self._ck(self.lib.asv_rgb2lab(self.h))

    def Ld_first_init(self):
        self._ck(self.lib.asv_ld_first_init(self.h))

    def flood(self, it):
        self._ck(self.lib.asv_flood(self.h, it))

    def centroids_next_seeds(self, it):
        self._ck(self.lib.asv_centroids_next_seeds(self.h, it))

    def Ld_next_seeds_matrix(self, it):
        self._ck(self.lib.asv_ld_next_seeds_matrix(self.h, it))

    def check_dead_seeds(self):
        out = np.empty(self.shape, np.int32)
        self._ck(self.lib.asv_check_dead_seeds(self.h, _ptr(out)))
        return out

    def run_lloyd(self):
        self._ck(self.lib.asv_run_lloyd(self.h))

    def enforce_connectivity(self, supsz=0):
        """Image::enforce_connectivity_3d on the last JFA labels; returns
        (labels, number of labels).  supsz 0: W*H*D / K."""
        out = np.empty(self.shape, np.int32)
        n = ctypes.c_int()
        self._ck(self.lib.asv_enforce_connectivity(self.h, supsz, _ptr(out), ctypes.byref(n)))
        return out, n.value

    def enforce_connectivity_labels(self, labels, supsz):
        """Render::label_connected3D / EnforceLabelConnectivity3D on a label
        volume [D,H,W]; returns (labels, number of labels)."""
        labels = np.ascontiguousarray(labels, np.int32)
        D, H, W = labels.shape
        out = np.empty_like(labels)
        n = ctypes.c_int()
        self._ck(self.lib.asv_enforce_connectivity_labels(self.h, _ptr(labels), W, H, D, int(supsz), _ptr(out),
                                                          ctypes.byref(n)))
        return out, n.value

    def evaluate(self, labels, truth):
        """asv_evaluate: LIBSVX-style measures of labels [D,H,W] against truth ids;
        returns a dict."""
        labels = np.ascontiguousarray(labels, np.int32)
        truth = np.ascontiguousarray(truth, np.int32)
        D, H, W = labels.shape
        e = _lib.Eval()
        self._ck(self.lib.asv_evaluate(self.h, _ptr(labels), _ptr(truth), W, H, D, ctypes.byref(e)))
        return {k: getattr(e, k) for k, _ in _lib.Eval._fields_}

    def autotune(self):
        """asv_autotune: times the Lloyd loop at JFA tile depths 4..32, keeps the
        fastest; returns it."""
        z = ctypes.c_int()
        self._ck(self.lib.asv_autotune(self.h, ctypes.byref(z)))
        return z.value

    # --- state ---------------------------------------------------------------
    def info(self):
        i = Info()
        self._ck(self.lib.asv_get_info(self.h, ctypes.byref(i)))
        return i

    def labels(self):
        out = np.empty(self.shape, np.int32)
        self._ck(self.lib.asv_get_labels(self.h, _ptr(out)))
        return out

    def raw_labels(self):
        out = np.empty(self.shape, np.int32)
        self._ck(self.lib.asv_get_raw_labels(self.h, _ptr(out)))
        return out

    def seeds(self):
        out = np.empty((self.info().Kp, 12), np.float32)
        self._ck(self.lib.asv_get_seeds(self.h, _ptr(out)))
        return out

    def set_seeds(self, seeds):
        seeds = np.ascontiguousarray(seeds, np.float32)
        self._ck(self.lib.asv_set_seeds(self.h, _ptr(seeds), seeds.shape[0]))

    def lab(self):
        out = np.empty(self.shape + (4,), np.uint8)
        self._ck(self.lib.asv_get_lab(self.h, _ptr(out)))
        return out

    def sums(self):
        out = np.empty((self.info().Kp + 1, 7), np.int64)
        self._ck(self.lib.asv_get_sums(self.h, _ptr(out)))
        return out

    def check_dead_seeds_host(self, raw):
        raw = np.ascontiguousarray(raw, np.int32)
        out = np.empty_like(raw)
        self._ck(self.lib.asv_check_dead_seeds_host(self.h, _ptr(raw), _ptr(out)))
        return out

    def jfa_pass(self, labels_in, step, ratio):
        labels_in = np.ascontiguousarray(labels_in, np.int32)
        out = np.empty_like(labels_in)
        self._ck(self.lib.asv_jfa_pass_host(self.h, step, ratio, _ptr(labels_in), _ptr(out)))
        return out

    def stats(self):
        s = Stats()
        self._ck(self.lib.asv_get_stats(self.h, ctypes.byref(s)))
        return s

    def stream(self):
        p = ctypes.c_void_p()
        self._ck(self.lib.asv_get_stream(self.h, ctypes.byref(p)))
        return p.value

    def synchronize(self):
        self._ck(self.lib.asv_synchronize(self.h))

    def segment(self, rgb, fwd, bwd, K):
        """Render::run's plain per-clip sequence; returns post-processed labels."""
        self.init_gpu(rgb, K)
        self.upload_flow(fwd, bwd)
        self.initialization()
        self.seed_matrix()
        self.RGB2LAB()
        self.run_lloyd()
        return self.labels()

    def segment_folder(self, folder, K):
        """Render::run from a folder of PNG, BMP or PNM frames (GPU-AS/Render.cpp:151-243):
        the sorted frames decoded on the host, preprocessing and optical flow
        on the device, then the plain sequence.  Returns post-processed labels."""
        self.init_gpu_bgr(read_frames(list_frames(folder)), K)
        self.compute_flow()
        self.initialization()
        self.seed_matrix()
        self.RGB2LAB()
        self.run_lloyd()
        return self.labels()


class Batch(Image):
    """Many clips of uneven size in one context: every stage one launch over all
    clips, the Lloyd loop one CUDA graph (asv_batch_*)."""

    def __init__(self, dims, **kw):
        """dims: list of (W, H, D, K) per clip."""
        super().__init__(**kw)
        arr = [np.ascontiguousarray([d[i] for d in dims], np.int32) for i in range(4)]
        self._dims = arr
        self._ck(self.lib.asv_batch_init(self.h, len(dims), *[_ptr(a) for a in arr]))
        self.shapes = [(int(d[2]), int(d[1]), int(d[0])) for d in dims]

    def upload(self, i, rgb, fwd, bwd):
        rgb = np.ascontiguousarray(rgb, np.uint8)
        fwd = np.ascontiguousarray(fwd, np.float32)
        bwd = np.ascontiguousarray(bwd, np.float32)
        if rgb.shape[:3] != self.shapes[i]:
            raise ValueError(f"clip {i} is {self.shapes[i]}, got {rgb.shape[:3]}")
        self._ck(self.lib.asv_batch_upload(self.h, i, _ptr(rgb), _ptr(fwd), _ptr(bwd)))

    def prepare(self):
        """initialization + seed_matrix + RGB2LAB for every clip."""
        self.initialization()
        self.seed_matrix()
        self.RGB2LAB()

    def clip_labels(self, i):
        out = np.empty(self.shapes[i], np.int32)
        self._ck(self.lib.asv_batch_get_labels(self.h, i, _ptr(out)))
        return out

    def clip_info(self, i):
        inf = Info()
        self._ck(self.lib.asv_batch_get_info(self.h, i, ctypes.byref(inf)))
        return inf


class Stream(Image):
    """The reference's streaming form (streamGPU-AS/Render.cpp:100-569) on the
    device: `push` takes a block's new frames and returns the video-wide labels
    of the frames that block finishes."""

    def __init__(self, W, H, D_all, K_video=0, seeds_num_100=0, block_size=30, **kw):
        super().__init__(**kw)
        self._ck(self.lib.asv_stream_begin(self.h, W, H, D_all, K_video, seeds_num_100, block_size))
        self.W, self.H = W, H
        self._fed = {}       # block -> the fed arrays, alive until that block's push returns
        self._inflight = collections.deque()   # (block, first frame, labels out) of enqueued blocks

    def info(self):
        i = _lib.StreamInfo()
        self._ck(self.lib.asv_stream_info_get(self.h, ctypes.byref(i)))
        return i

    def push(self, rgb, fwd=None, bwd=None, out=None):
        """rgb [n,H,W,3] uint8, fwd/bwd [n,H,W,2] float32: the next block's new frames
        (fwd and bwd None: the block's flow is computed on the device).
        `out`: where the labels go, an int32 C-contiguous array of at least
        [block frames, H, W]; a buffer reused for every block (e.g. pinned)
        takes block_size + block_size // 3 frames, the longest block (the
        last block absorbs the remainder of the video); a new array when None.
        Returns (first frame index, labels [done,H,W] int32, a view of `out`)."""
        inf = self.info()
        rgb = np.ascontiguousarray(rgb, np.uint8)
        if fwd is not None:
            fwd = np.ascontiguousarray(fwd, np.float32)
            bwd = np.ascontiguousarray(bwd, np.float32)
        if rgb.shape[0] != inf.frames_needed:
            raise ValueError(f"block {inf.next_block} needs {inf.frames_needed} new frames")
        D = inf.block_end - inf.block_start
        if out is None:
            out = np.empty((D, self.H, self.W), np.int32)
        elif (out.dtype != np.int32 or not out.flags.c_contiguous or out.ndim != 3
              or out.shape[0] < D or out.shape[1:] != (self.H, self.W)):
            raise ValueError(f"out must be C-contiguous int32 of at least ({D}, {self.H}, {self.W})")
        done = ctypes.c_int()
        self._ck(self.lib.asv_stream_push(self.h, _ptr(rgb), _ptr(fwd), _ptr(bwd), _ptr(out),
                                          ctypes.byref(done)))
        return inf.block_start, out[:done.value]

    def block(self, b):
        """(block_start, block_end, frames_needed) of block b"""
        a, e, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._ck(self.lib.asv_stream_block(self.h, b, ctypes.byref(a), ctypes.byref(e), ctypes.byref(n)))
        return a.value, e.value, n.value

    def feed(self, rgb, fwd=None, bwd=None, bgr=False):
        """Queue the upload of the next unfed block's new frames (asv_stream_feed):
        it runs on the device while the block before it computes.  bgr=True:
        the frames as decoded (BGR, top row first), preprocessed on the device
        (asv_stream_feed_bgr).  Returns the block's index.  The arrays must stay
        unchanged until that block's push_fed returns (they are kept alive here
        until then)."""
        b = max([self.info().next_block] + [k + 1 for k in self._fed])
        if b >= self.info().blocks:
            raise ValueError("every block of the video is fed")
        n = self.block(b)[2]
        rgb = np.ascontiguousarray(rgb, np.uint8)
        if fwd is not None:
            fwd = np.ascontiguousarray(fwd, np.float32)
            bwd = np.ascontiguousarray(bwd, np.float32)
        if rgb.shape[0] != n:
            raise ValueError(f"block {b} needs {n} new frames")
        call = self.lib.asv_stream_feed_bgr if bgr else self.lib.asv_stream_feed
        self._ck(call(self.h, _ptr(rgb), _ptr(fwd), _ptr(bwd)))
        self._fed[b] = (rgb, fwd, bwd)
        return b

    def push_fed(self, out=None):
        """asv_stream_push_fed: the next block, whose frames were fed ahead.
        `out` and the return value as in push."""
        inf = self.info()
        D = inf.block_end - inf.block_start
        if out is None:
            out = np.empty((D, self.H, self.W), np.int32)
        elif (out.dtype != np.int32 or not out.flags.c_contiguous or out.ndim != 3
              or out.shape[0] < D or out.shape[1:] != (self.H, self.W)):
            raise ValueError(f"out must be C-contiguous int32 of at least ({D}, {self.H}, {self.W})")
        done = ctypes.c_int()
        self._ck(self.lib.asv_stream_push_fed(self.h, _ptr(out), ctypes.byref(done)))
        self._fed.pop(inf.next_block, None)
        return inf.block_start, out[:done.value]

    def push_fed_async(self, out):
        """asv_stream_push_fed_async: enqueue the next (fed) block and return;
        `wait` gives its labels, in `out` (kept here until then).  Returns the
        block's index."""
        inf = self.info()
        D = inf.block_end - inf.block_start
        if (out.dtype != np.int32 or not out.flags.c_contiguous or out.ndim != 3
                or out.shape[0] < D or out.shape[1:] != (self.H, self.W)):
            raise ValueError(f"out must be C-contiguous int32 of at least ({D}, {self.H}, {self.W})")
        self._ck(self.lib.asv_stream_push_fed_async(self.h, _ptr(out)))
        self._inflight.append((inf.next_block, inf.block_start, out))
        return inf.next_block

    def wait(self):
        """asv_stream_wait: the oldest block in flight, as
        (first frame index, labels [done,H,W] int32, a view of its `out`)."""
        blk, done = ctypes.c_int(), ctypes.c_int()
        try:
            self._ck(self.lib.asv_stream_wait(self.h, ctypes.byref(blk), ctypes.byref(done)))
        finally:
            b, f0, out = self._inflight.popleft() if self._inflight else (None, 0, None)
            self._fed.pop(b, None)
        return f0, out[:done.value]


class Server:
    """Request pool on one GPU (asv_server_*): clip requests admitted first-fit
    under an HBM budget, each on its own slot stream, plus streaming sessions
    whose windows run in order.  `submit_*` returns a request id; `wait` gives
    (labels, latency_ms, queue_ms)."""

    def __init__(self, max_slots=4, hbm_budget=0, **kw):
        self.lib = _lib.load()
        self.cfg = config(**kw)
        h = ctypes.c_void_p()
        st = self.lib.asv_server_create(ctypes.byref(self.cfg), max_slots, hbm_budget, ctypes.byref(h))
        if st != _lib.ASV_OK:
            raise AsvError(st, self.lib.asv_status_string(st).decode())
        self.h = h
        self._live = {}      # id -> (arrays kept alive, labels out, session W/H)
        self._sessions = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.asv_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        if st != _lib.ASV_OK:
            raise AsvError(st, self.lib.asv_status_string(st).decode())

    def open_session(self, W, H, D_all, K_video=0, seeds_num_100=0, block_size=30):
        sid = ctypes.c_int()
        self._ck(self.lib.asv_server_open_session(self.h, W, H, D_all, K_video, seeds_num_100,
                                                  block_size, ctypes.byref(sid)))
        self._sessions[sid.value] = (W, H, block_size or 30)
        return sid.value

    def _submit(self, req, keep, out):
        rid = ctypes.c_longlong()
        self._ck(self.lib.asv_server_submit(self.h, ctypes.byref(req), ctypes.byref(rid)))
        self._live[rid.value] = (keep, out, req.kind == _lib.REQ_WINDOW)
        return rid.value

    def submit_clip(self, rgb, fwd, bwd, K):
        """fwd and bwd None: the clip's flow is computed on the device"""
        rgb = np.ascontiguousarray(rgb, np.uint8)
        if fwd is not None:
            fwd = np.ascontiguousarray(fwd, np.float32)
            bwd = np.ascontiguousarray(bwd, np.float32)
        D, H, W = rgb.shape[:3]
        out = np.empty((D, H, W), np.int32)
        req = _lib.Request(_lib.REQ_CLIP, 0, W, H, D, K, _ptr(rgb).value,
                           _ptr(fwd).value if fwd is not None else None,
                           _ptr(bwd).value if bwd is not None else None, _ptr(out).value)
        return self._submit(req, (rgb, fwd, bwd), out)

    def submit_window(self, session, rgb, fwd=None, bwd=None):
        """the next block's new frames of a session (asv_stream_push semantics;
        fwd and bwd None: the block's flow is computed on the device)"""
        W, H, block = self._sessions[session]
        rgb = np.ascontiguousarray(rgb, np.uint8)
        if fwd is not None:
            fwd = np.ascontiguousarray(fwd, np.float32)
            bwd = np.ascontiguousarray(bwd, np.float32)
        # the last block of a video can reach block_size + block_size/3 - 1 frames
        out = np.empty((block + block // 3, H, W), np.int32)
        req = _lib.Request(_lib.REQ_WINDOW, session, W, H, rgb.shape[0], 0, _ptr(rgb).value,
                           _ptr(fwd).value if fwd is not None else None,
                           _ptr(bwd).value if bwd is not None else None, _ptr(out).value)
        return self._submit(req, (rgb, fwd, bwd), out)

    def wait(self, rid):
        lat, qms, done = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        st = self.lib.asv_server_wait(self.h, rid, ctypes.byref(lat), ctypes.byref(qms),
                                      ctypes.byref(done))
        keep, out, window = self._live.pop(rid)
        self._ck(st)
        if window:
            out = out[:done.value]
        return out, lat.value, qms.value

    def poll(self, rid):
        d = ctypes.c_int()
        self._ck(self.lib.asv_server_poll(self.h, rid, ctypes.byref(d)))
        return bool(d.value)

    def stats(self):
        s = _lib.ServerStats()
        self._ck(self.lib.asv_server_get_stats(self.h, ctypes.byref(s)))
        return s


def write_labels_txt(path, labels):
    D, H, W = labels.shape
    lab = np.ascontiguousarray(labels, np.int32)
    if _lib.load().asv_write_labels_txt(path.encode(), _ptr(lab), W, H, D) != 0:
        raise OSError(f"cannot write {path}")


def write_render_ppm(prefix, labels, n_labels):
    D, H, W = labels.shape
    lab = np.ascontiguousarray(labels, np.int32)
    if _lib.load().asv_write_render_ppm(prefix.encode(), _ptr(lab), W, H, D, n_labels) != 0:
        raise OSError(f"cannot write {prefix}*.ppm")


_PNG_ERRORS = {-1: "bad argument", -2: "file I/O error", -3: "malformed PNG", -4: "unsupported PNG",
               -5: "frame size differs"}


def _png_ck(st, what):
    if st != 0:
        raise (OSError if st == -2 else ValueError)(f"{what}: {_PNG_ERRORS.get(st, st)}")


def png_info(path):
    """(W, H) from a PNG file's header"""
    W, H = ctypes.c_int(), ctypes.c_int()
    _png_ck(_lib.load().asv_png_info(os.fsencode(path), ctypes.byref(W), ctypes.byref(H)), path)
    return W.value, H.value


def read_png(path):
    """cv::imread(path, 1) of a PNG frame: [H, W, 3] uint8 BGR, top row first."""
    W, H = png_info(path)
    out = np.empty((H, W, 3), np.uint8)
    _png_ck(_lib.load().asv_png_read_bgr(os.fsencode(path), _ptr(out), W, H), path)
    return out


FRAME_EXTENSIONS = (".png", ".bmp", ".ppm", ".pgm", ".pnm")


def list_frames(folder):
    """The frame files (PNG, BMP, PNM) of a folder in sorted order
    (Render::run sorts the file list, GPU-AS/Render.cpp:151-153)."""
    names = sorted(f for f in os.listdir(folder) if f.lower().endswith(FRAME_EXTENSIONS))
    if not names:
        raise ValueError(f"no frames in {folder}")
    return [os.path.join(folder, f) for f in names]


def frame_info(path):
    """(W, H) of a PNG, BMP or PNM frame file"""
    W, H = ctypes.c_int(), ctypes.c_int()
    _png_ck(_lib.load().asv_frame_info(os.fsencode(path), ctypes.byref(W), ctypes.byref(H)), path)
    return W.value, H.value


def read_frame(path):
    """cv::imread(path, 1) of a PNG, BMP or PNM frame: [H, W, 3] uint8 BGR, top row first."""
    W, H = frame_info(path)
    out = np.empty((H, W, 3), np.uint8)
    _png_ck(_lib.load().asv_frame_read_bgr(os.fsencode(path), _ptr(out), W, H), path)
    return out


def read_frames(paths, out=None):
    """Frames of one size (PNG, BMP or PNM) decoded on all host threads:
    [D, H, W, 3] uint8 BGR (into `out`, e.g. a pinned buffer, when given)."""
    paths = list(paths)
    W, H = frame_info(paths[0])
    if out is None:
        out = np.empty((len(paths), H, W, 3), np.uint8)
    elif out.shape != (len(paths), H, W, 3) or out.dtype != np.uint8 or not out.flags.c_contiguous:
        raise ValueError(f"out must be a contiguous uint8 array of shape {(len(paths), H, W, 3)}")
    arr = (ctypes.c_char_p * len(paths))(*[os.fsencode(p) for p in paths])
    _png_ck(_lib.load().asv_frames_read_bgr(arr, len(paths), W, H, _ptr(out)), "frames")
    return out


def write_png(path, rgb):
    """8-bit RGB image [H, W, 3], top row first."""
    rgb = np.ascontiguousarray(rgb, np.uint8)
    H, W, _ = rgb.shape
    _png_ck(_lib.load().asv_png_write_rgb(os.fsencode(path), _ptr(rgb), W, H), path)


def render_rgb(labels, n_labels):
    """Pseudo-colour frames of print_render: [D, H, W, 3] RGB, top row first."""
    D, H, W = labels.shape
    lab = np.ascontiguousarray(labels, np.int32)
    out = np.empty((D, H, W, 3), np.uint8)
    _png_ck(_lib.load().asv_render_rgb(_ptr(lab), W, H, D, n_labels, _ptr(out)), "render")
    return out


def write_render_png(prefix, labels, n_labels, start_index=-1):
    """The pseudo-colour frames as PNG files: <prefix>NNNNN.png (from 1), or
    <prefix>SSSSS_NNNNN.png for a streaming window starting at start_index."""
    D, H, W = labels.shape
    lab = np.ascontiguousarray(labels, np.int32)
    _png_ck(_lib.load().asv_write_render_png(os.fsencode(prefix), _ptr(lab), W, H, D, n_labels, start_index),
            prefix)


def preprocess_frame(bgr):
    """Render::cvMat2TexureInput on one BGR frame stored top row first."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    H, W, _ = bgr.shape
    out = np.empty_like(bgr)
    if _lib.load().asv_preprocess_frame(_ptr(bgr), W, H, _ptr(out)) != 0:
        raise ValueError("bad frame")
    return out


def render_run(dataset_path, save_path, dbname, vdname, seeds_num, compactness=8.0, stream=False, **opts):
    """Render::run of the plain (or, stream=True, the streaming) program:
    <dataset_path>/<vdname> PNG frames in, <save_path><dbname>/AS/<vdname>/
    <seeds_num>.txt and <seeds_num>_NNNNN.png out (asv_render_run /
    asv_render_stream_run).  opts: lloyd_iters, write_txt, write_render,
    connectivity, device, verbose.  Returns the library's code (0 = done)."""
    lib = _lib.load()
    o = _lib.RenderOptions()
    lib.asv_render_options_default(ctypes.byref(o))
    for k, v in opts.items():
        setattr(o, k, int(v))
    fn = lib.asv_render_stream_run if stream else lib.asv_render_run
    return fn(os.fsencode(dataset_path), os.fsencode(save_path), dbname.encode(), vdname.encode(), int(seeds_num),
              float(compactness), ctypes.byref(o))
