/*
 * asv_host.h -- host pipeline around the C ABI (libasv.so): synthetic clip
 * source, frame preprocessing and the reference's output writers.
 *
 * These replace the host parts of the reference's Render class that sit
 * either side of the supervoxel path (GPU-AS/Render.cpp, GPU-AS/Image.cpp
 * print_sv_txt / print_render); they run on the CPU as in the reference.
 */
#ifndef ASV_HOST_H
#define ASV_HOST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Seeded synthetic video: linear-gradient background plus moving ellipses
 * of uniform-random LAB colour, additive Gaussian noise, and the exact
 * generating motion as forward/backward flow.  Frames are produced in
 * texture orientation (y up), i.e. directly in the layout asv_init_gpu
 * takes.  Frame f of a video depends only on (seed, f), so windows of a
 * long video can be generated independently. */
typedef struct asv_synth_params {
    int W, H;
    int frame0;         /* first frame index to generate */
    int nframes;        /* frames to generate */
    int n_ellipses;
    float noise_sigma;  /* Gaussian noise on uint8 */
    float vmax;         /* speed drawn uniformly in [0, vmax] px/frame */
    float jitter;       /* per-frame velocity jitter, uniform in [-jitter, jitter] */
    float drift_amp;    /* background drift amplitude in px (0 = static) */
    float drift_period; /* background drift period in frames */
    uint64_t seed;
} asv_synth_params;

/* rgb: nframes*H*W*3; fwd, bwd: nframes*H*W*2 (either may be NULL). */
int asv_synth_clip(const asv_synth_params *p, uint8_t *rgb, float *fwd, float *bwd);

/* Ground truth of the same frames: per pixel the index of the ellipse on
 * top, n_ellipses for the background (nframes*H*W int32). */
int asv_synth_truth(const asv_synth_params *p, int32_t *ids);

/* Render::cvMat2TexureInput (GPU-AS/Render.cpp:354-359): 3x3 Gaussian blur
 * (sigma 0 -> [1,2,1]/4 separable, border reflect-101, rounded half up),
 * BGR -> RGB and vertical flip, for one frame stored top row first. */
int asv_preprocess_frame(const uint8_t *bgr, int W, int H, uint8_t *rgb_tex);

/* Image::print_sv_txt (GPU-AS/Image.cpp:1780-1806): frames in order, rows
 * from y = H-1 down to 0, each label left-aligned in 4 columns plus a
 * space, a newline per row and two blank lines per frame. */
int asv_write_labels_txt(const char *path, const int32_t *labels, int W, int H, int D);

/* Image::print_render (GPU-AS/Image.cpp:1883-1935): one colour per label
 * from rand() % 256 (C library generator in its default state), -1 black,
 * written as binary PPM frames <prefix>NNNNN.ppm, top row first. */
int asv_write_render_ppm(const char *prefix, const int32_t *labels, int W, int H, int D,
                         int n_labels);

/* ---- PNG frames (PNG / zlib RFC 1950 / DEFLATE RFC 1951, no codec library).
 * Return 0, or -1 bad argument, -2 file I/O, -3 malformed file (signature,
 * chunk CRC, zlib stream, Adler-32, filter type, palette index), -4
 * unsupported (unknown critical chunk, more than 2^28 pixels), -5 the image
 * is not W x H. */

/* Width and height from a PNG file's header. */
int asv_png_info(const char *path, int *W, int *H);

/* cv::imread(path, 1) of Render::run (GPU-AS/Render.cpp:151-157, 229-238)
 * for a PNG frame: W*H*3 bytes BGR, top row first.  Every colour type, bit
 * depth and Adam7 interlacing; grey replicated, alpha dropped, 16-bit
 * samples reduced to their high byte, 1/2/4-bit grey scaled to 0..255. */
int asv_png_read_bgr(const char *path, uint8_t *bgr, int W, int H);

/* n frames of one size, decoded on all host threads, into n*W*H*3 bytes
 * (the clip layout asv_init_gpu_bgr takes).  Returns the error of the
 * first frame that failed. */
int asv_png_read_frames_bgr(const char *const *paths, int n, int W, int H, uint8_t *bgr);

/* Any supported frame file, the format taken from its first bytes: PNG, BMP
 * (1/4/8-bit palette, 16/24/32-bit, bit fields; RLE refused as -4) or
 * binary PNM (P5 grey, P6 colour; maxval 255 or 65535).  Same pixels and
 * return codes as the PNG calls above: imread(path, 1)'s BGR, top row first. */
int asv_frame_info(const char *path, int *W, int *H);
int asv_frame_read_bgr(const char *path, uint8_t *bgr, int W, int H);
/* n frames of one size of any supported format, on all host threads */
int asv_frames_read_bgr(const char *const *paths, int n, int W, int H, uint8_t *bgr);

/* 8-bit RGB PNG (W*H*3 bytes, top row first). */
int asv_png_write_rgb(const char *path, const uint8_t *rgb, int W, int H);

/* The pseudo-colour frames of asv_write_render_ppm in memory: D*W*H*3
 * bytes RGB, top row first. */
int asv_render_rgb(const int32_t *labels, int W, int H, int D, int n_labels, uint8_t *rgb);

/* The same frames as PNG files: <prefix>NNNNN.png numbered from 1
 * (print_render, GPU-AS/Image.cpp:1930-1932) when start_index < 0, else
 * <prefix>SSSSS_NNNNN.png with S = start_index and N = start_index + 1 + t
 * (output_render_all, streamGPU-AS/Render.cpp:819-821). */
int asv_write_render_png(const char *prefix, const int32_t *labels, int W, int H, int D,
                         int n_labels, int start_index);

/* ---- the reference's host programs ------------------------------------ */

/* Options of asv_render_run / asv_render_stream_run. */
typedef struct asv_render_options {
    int lloyd_iters;    /* 0: 20, the reference's Lloyd_max_iter (GPU-AS/Render.cpp:11) */
    int write_txt;      /* the label txt file (the reference's output_label) */
    int write_render;   /* the pseudo-colour frames as PNG files */
    int connectivity;   /* plain form: post-processing 6.2, 3D connectivity enforcement
                           (GPU-AS/Render.cpp:323-341), instead of 6.1 */
    int device;         /* CUDA device ordinal */
    int verbose;        /* progress lines on stdout, as the reference's cout */
} asv_render_options;

/* defaults: 20 iterations, txt and renders written, 6.1 post-processing,
 * device 0, quiet */
void asv_render_options_default(asv_render_options *opt);

#define ASV_RENDER_ERR_ARG (-1)     /* NULL argument or seeds_num < 1 */
#define ASV_RENDER_ERR_IO (-2)      /* no frames, unreadable folder, unwritable output */
#define ASV_RENDER_ERR_DECODE (-3)  /* a frame is not a readable PNG file */
#define ASV_RENDER_ERR_SIZE (-4)    /* frames of different sizes */
#define ASV_RENDER_ERR_GPU (-5)     /* a C ABI call failed (message on stderr) */

/* Render::run of the plain program (GPU-AS/Render.cpp:100-350, called by
 * GPU-AS/main.cpp:49-86 with the same arguments): the sorted frames of
 * <dataset_path>/<vdname> (PNG), preprocessing and optical flow on the
 * device, seeds (K = seeds_num), metric, LAB, the Lloyd loop and
 * check_dead_seeds; writes <save_path><dbname>/AS/<vdname>/<seeds_num>.txt
 * (print_sv_txt) and <seeds_num>_NNNNN.png pseudo-colour frames
 * (print_render, numbered from 1).  compactness is accepted and, as in the
 * reference (Image::init_variables, GPU-AS/Image.cpp:1050), 8 is used.
 * opt NULL: asv_render_options_default.  Returns 0 or ASV_RENDER_ERR_*. */
int asv_render_run(const char *dataset_path, const char *save_path, const char *dbname, const char *vdname,
                   int seeds_num, float compactness, const asv_render_options *opt);

/* Render::run of the streaming program (streamGPU-AS/Render.cpp:100-303):
 * seeds_num over the whole video (seeds_num_100 = seeds_num * 100 / frames),
 * blocks of 30 frames overlapping by 10, each block's flow computed on the
 * device; writes the video-wide labels as <seeds_num>.txt
 * (output_label_all, :741-764) and <seeds_num>_NNNNN.png
 * (output_render_all, :766-826) in the same folder layout.  Compactness 6
 * (streamGPU-AS/Image.cpp:968). */
int asv_render_stream_run(const char *dataset_path, const char *save_path, const char *dbname,
                          const char *vdname, int seeds_num, float compactness, const asv_render_options *opt);

#ifdef __cplusplus
}
#endif
#endif
