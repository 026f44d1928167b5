// A host program calling the library's Render::run drop-in the way the
// reference's GPU-AS/main.cpp:49-86 calls Render::run: one video folder,
// one seed count.  Built by tests/test_gpu_render.py with g++ against
// libasv.so.
//   render_main <plain|stream> <dataset_path> <save_path> <dbname> <vdname> <seeds_num> <lloyd_iters>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "asv_host.h"

int main(int argc, char **argv)
{
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s plain|stream dataset_path save_path dbname vdname seeds_num iters\n", argv[0]);
        return 2;
    }
    asv_render_options opt;
    asv_render_options_default(&opt);
    opt.lloyd_iters = std::atoi(argv[7]);
    const float compactness = 8.0f;
    const bool stream = std::strcmp(argv[1], "stream") == 0;
    const int r = stream ? asv_render_stream_run(argv[2], argv[3], argv[4], argv[5], std::atoi(argv[6]), compactness, &opt)
                         : asv_render_run(argv[2], argv[3], argv[4], argv[5], std::atoi(argv[6]), compactness, &opt);
    if (r != 0) std::fprintf(stderr, "render failed: %d\n", r);
    return r == 0 ? 0 : 1;
}
