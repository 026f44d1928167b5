"""GB300-native supervoxel engine: the JFA + Lloyd hot path of
dongxiao0401/anisotropic_supervoxel behind a C ABI (include/asv.h).

Python here is a thin host mirror over libasv.so (ctypes); the compute runs
in the CUDA kernels of csrc/.
"""
from ._lib import AsvError, load  # noqa: F401
from .image import (Batch, Image, Server, Stream, config, frame_info, list_frames, png_info, preprocess_frame,  # noqa: F401
                    read_frame, read_frames, read_png, render_rgb, render_run, synth_clip, synth_truth, write_labels_txt, write_png,
                    write_render_png, write_render_ppm)
