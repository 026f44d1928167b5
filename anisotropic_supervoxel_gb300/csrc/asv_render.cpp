// asv_render.cpp -- the reference's Render::run host programs as a drop-in
// over the C ABI: the plain per-clip form (GPU-AS/Render.cpp:100-350) and
// the streaming form (streamGPU-AS/Render.cpp:100-303, outputs :741-826).
//
// Both read the sorted frames of <dataset_path>/<vdname>, segment them on
// the GPU (preprocessing, optical flow, seeds, metric, LAB, the Lloyd loop,
// post-processing) and write, under <save_path><dbname>/AS/<vdname>/, the
// txt label file <seeds_num>.txt (print_sv_txt / output_label_all) and the
// pseudo-colour frames <seeds_num>_NNNNN.png (print_render /
// output_render_all, whose per-frame imwrite the reference leaves commented
// out).  No GL context, window or OpenCV: frames are PNG, BMP or PNM files
// decoded by this library.
#include "asv.h"
#include "asv_host.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <thread>
#include <vector>

namespace {

namespace fs = std::filesystem;

// Render::getFiles + sort (GPU-AS/Render.cpp:148-150): every regular file of
// the folder, full paths sorted as strings
int list_frames(const std::string &dir, std::vector<std::string> &files)
{
    std::error_code ec;
    files.clear();
    for (const auto &e : fs::directory_iterator(dir, ec)) {
        if (e.is_regular_file(ec)) files.push_back(e.path().string());
    }
    if (ec) return ASV_RENDER_ERR_IO;
    std::sort(files.begin(), files.end());
    return files.empty() ? ASV_RENDER_ERR_IO : 0;
}

// save_path + dbname + "/AS/" + vdname + "/" created (mkdir -p), then + seeds_num
int out_stem(const char *save_path, const char *dbname, const char *vdname, int seeds_num, std::string &stem)
{
    std::string dir = std::string(save_path) + dbname + "/AS/" + vdname + "/";
    std::error_code ec;
    fs::create_directories(dir, ec);
    if (ec) return ASV_RENDER_ERR_IO;
    stem = dir + std::to_string(seeds_num);
    return 0;
}

int say(const asv_render_options &o, const char *fmt, const char *a, long long b)
{
    if (o.verbose) {
        std::printf(fmt, a, b);
        std::fflush(stdout);
    }
    return 0;
}

struct Ctx {
    asv_ctx *c = nullptr;
    ~Ctx() { if (c) asv_destroy(c); }
};

int asv_fail(asv_ctx *c, asv_status st, const char *what)
{
    std::fprintf(stderr, "asv_render: %s: %s (%s)\n", what, asv_status_string(st), c ? asv_last_error(c) : "");
    return ASV_RENDER_ERR_GPU;
}

int read_png_frames(const std::vector<std::string> &files, int f0, int n, int W, int H, std::vector<uint8_t> &bgr)
{
    std::vector<const char *> paths;
    for (int i = f0; i < f0 + n; i++) paths.push_back(files[i].c_str());
    bgr.resize((size_t)n * W * H * 3);
    const int e = asv_frames_read_bgr(paths.data(), n, W, H, bgr.data());
    if (e == -5) return ASV_RENDER_ERR_SIZE;
    return e ? ASV_RENDER_ERR_DECODE : 0;
}

int write_outputs(const asv_render_options &o, const std::string &stem, const int32_t *labels, int W, int H, int D,
                  int n_labels)
{
    if (o.write_txt && asv_write_labels_txt((stem + ".txt").c_str(), labels, W, H, D) != 0) return ASV_RENDER_ERR_IO;
    if (o.write_render && asv_write_render_png((stem + "_").c_str(), labels, W, H, D, n_labels, -1) != 0)
        return ASV_RENDER_ERR_IO;
    return 0;
}

} // namespace

extern "C" void asv_render_options_default(asv_render_options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->lloyd_iters = 20;
    o->write_txt = 1;
    o->write_render = 1;
}

extern "C" int asv_render_run(const char *dataset_path, const char *save_path, const char *dbname, const char *vdname,
                              int seeds_num, float compactness, const asv_render_options *opt)
{
    (void)compactness;                       // Image::init_variables sets it to 8 (GPU-AS/Image.cpp:1050)
    if (!dataset_path || !save_path || !dbname || !vdname || seeds_num < 1) return ASV_RENDER_ERR_ARG;
    asv_render_options o;
    if (opt) o = *opt; else asv_render_options_default(&o);
    std::vector<std::string> files;
    if (list_frames(std::string(dataset_path) + "/" + vdname, files) != 0) return ASV_RENDER_ERR_IO;
    std::string stem;
    if (out_stem(save_path, dbname, vdname, seeds_num, stem) != 0) return ASV_RENDER_ERR_IO;
    say(o, "%s,%lld:\n", vdname, seeds_num);
    int W = 0, H = 0;
    if (asv_frame_info(files[0].c_str(), &W, &H) != 0) return ASV_RENDER_ERR_DECODE;
    const int D = (int)files.size();
    std::vector<uint8_t> bgr;
    int e = read_png_frames(files, 0, D, W, H, bgr);
    if (e) return e;

    asv_config cfg;
    asv_config_default(&cfg);
    cfg.variant = ASV_VARIANT_PLAIN;
    cfg.lloyd_iters = o.lloyd_iters > 0 ? o.lloyd_iters : 20;
    cfg.device = o.device;
    Ctx c;
    asv_status st = asv_create(&cfg, &c.c);
    if (st != ASV_OK) return asv_fail(nullptr, st, "asv_create");
    // Render::run steps 1-5 (GPU-AS/Render.cpp:255-293)
    if ((st = asv_init_gpu_bgr(c.c, bgr.data(), W, H, D, seeds_num)) != ASV_OK) return asv_fail(c.c, st, "init_gpu");
    if ((st = asv_compute_flow(c.c)) != ASV_OK) return asv_fail(c.c, st, "forward_backward_flow");
    if ((st = asv_initialization(c.c)) != ASV_OK) return asv_fail(c.c, st, "initialization");
    if ((st = asv_seed_matrix(c.c)) != ASV_OK) return asv_fail(c.c, st, "seed_matrix");
    if ((st = asv_rgb2lab(c.c)) != ASV_OK) return asv_fail(c.c, st, "RGB2LAB");
    if ((st = asv_run_lloyd(c.c)) != ASV_OK) return asv_fail(c.c, st, "Lloyd loop");
    // 6.1 check_dead_seeds (the loop's post-processing), or 6.2 connectivity
    std::vector<int32_t> labels((size_t)W * H * D);
    int n_labels = 0;
    if (o.connectivity) {
        if ((st = asv_enforce_connectivity(c.c, 0, labels.data(), &n_labels)) != ASV_OK)
            return asv_fail(c.c, st, "enforce_connectivity_3d");
    } else {
        if ((st = asv_get_labels(c.c, labels.data())) != ASV_OK) return asv_fail(c.c, st, "labels");
        asv_info info;
        if ((st = asv_get_info(c.c, &info)) != ASV_OK) return asv_fail(c.c, st, "info");
        n_labels = info.final_label_num;
    }
    e = write_outputs(o, stem, labels.data(), W, H, D, n_labels);
    say(o, "%sdone, %lld frames\n", "", D);
    return e;
}

extern "C" int asv_render_stream_run(const char *dataset_path, const char *save_path, const char *dbname,
                                     const char *vdname, int seeds_num, float compactness,
                                     const asv_render_options *opt)
{
    (void)compactness;                       // streamGPU-AS/Image.cpp:968 sets it to 6
    if (!dataset_path || !save_path || !dbname || !vdname || seeds_num < 1) return ASV_RENDER_ERR_ARG;
    asv_render_options o;
    if (opt) o = *opt; else asv_render_options_default(&o);
    std::vector<std::string> files;
    if (list_frames(std::string(dataset_path) + "/" + vdname, files) != 0) return ASV_RENDER_ERR_IO;
    std::string stem;
    if (out_stem(save_path, dbname, vdname, seeds_num, stem) != 0) return ASV_RENDER_ERR_IO;
    say(o, "%s,%lld:\n", vdname, seeds_num);
    int W = 0, H = 0;
    if (asv_frame_info(files[0].c_str(), &W, &H) != 0) return ASV_RENDER_ERR_DECODE;
    const int D_all = (int)files.size();

    asv_config cfg;
    asv_config_default(&cfg);
    cfg.variant = ASV_VARIANT_STREAM;
    cfg.lloyd_iters = o.lloyd_iters > 0 ? o.lloyd_iters : 20;
    cfg.device = o.device;
    Ctx c;
    asv_status st = asv_create(&cfg, &c.c);
    if (st != ASV_OK) return asv_fail(nullptr, st, "asv_create");
    // seeds_num_100 = seeds_num * 100 / depth_all (streamGPU-AS/Render.cpp:156-158), blocks of 30
    if ((st = asv_stream_begin(c.c, W, H, D_all, seeds_num, 0, 30)) != ASV_OK) return asv_fail(c.c, st, "blocks");
    std::vector<int32_t> labels((size_t)W * H * D_all, -1);
    asv_stream_info inf;
    if ((st = asv_stream_info_get(c.c, &inf)) != ASV_OK) return asv_fail(c.c, st, "stream info");
    const int nb = inf.blocks;
    // the block's new frames as imread gives them (streamGPU-AS/Render.cpp:
    // 696-702), into buffer b % 2; cvMat2TexureInput runs on the device
    std::vector<uint8_t> bgr[2];
    auto decode = [&](int b) -> int {
        int a = 0, e = 0, n = 0;
        if (asv_stream_block(c.c, b, &a, &e, &n) != ASV_OK) return ASV_RENDER_ERR_GPU;
        return read_png_frames(files, e - n, n, W, H, bgr[b % 2]);
    };
    int e = decode(0);
    if (e) return e;
    if ((st = asv_stream_feed_bgr(c.c, bgr[0].data(), nullptr, nullptr)) != ASV_OK) return asv_fail(c.c, st, "feed");
    for (int b = 0; b < nb; b++) {
        // block b+1 is decoded on the host threads while block b runs on the
        // device; buffer (b+1) % 2 last held block b-1, whose push has returned
        int e_next = 0;
        std::thread worker([&] { if (b + 1 < nb) e_next = decode(b + 1); });
        if ((st = asv_stream_info_get(c.c, &inf)) != ASV_OK) { worker.join(); return asv_fail(c.c, st, "stream info"); }
        int done = 0;
        // flow computed on the device per block, as the streaming program does
        st = asv_stream_push_fed(c.c, labels.data() + (size_t)W * H * inf.block_start, &done);
        worker.join();
        if (st != ASV_OK) return asv_fail(c.c, st, "block_segment");
        say(o, "%sblock done, %lld frames\n", "", done);
        if (b + 1 < nb) {
            if (e_next) return e_next;
            if ((st = asv_stream_feed_bgr(c.c, bgr[(b + 1) % 2].data(), nullptr, nullptr)) != ASV_OK)
                return asv_fail(c.c, st, "feed");
        }
    }
    if ((st = asv_stream_info_get(c.c, &inf)) != ASV_OK) return asv_fail(c.c, st, "stream info");
    // labels_all with label_num_all = seeds_num_placed (streamGPU-AS/Render.cpp:289-292)
    return write_outputs(o, stem, labels.data(), W, H, D_all, inf.seeds_placed);
}
