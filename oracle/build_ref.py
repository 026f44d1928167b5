"""Compiles the reference's own GLSL shaders as C++ into
oracle/_ref/libref_shaders.so, against which the CPU restatement's shader
maths are pinned.  GLSL's vector types and swizzles come from a small header this
project writes (not from a third-party math library).

TEST INFRASTRUCTURE ONLY.  The shader files are read where they lie under
the reference tree; the transformed C++ and the library go to oracle/_ref/
(git-ignored, never committed).  The transform is textual and mechanical:
drop `#version` and `layout(...)` qualifiers, turn `in`/`out`/`uniform`
declarations into namespace globals, interface blocks into structs, and
`main` into `shader_main`.  The harness below (this project's code) supplies
GL's builtins: `texture()` as nearest-texel sampling with clamp-to-edge,
`gl_Position`, `gl_Layer`, `gl_in`, `EmitVertex`, `EndPrimitive`.  GLSL
float literals are single precision: compiled with -fsingle-precision-constant;
no FMA contraction (-ffp-contract=off); pow() is taken correctly rounded.
"""
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_shaders.so")
# the reference checkout: ASV_REFERENCE_ROOT, else a directory `reference`
# beside the repository's root directory; absent -> the builds return None
REF = os.environ.get("ASV_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                            "reference")
SHADERS = os.path.join(REF, "GPU-AS", "shaders")

PROGRAMS = {
    "rgb2lab": ["RGB2LAB.vs", "RGB2LAB.gs", "RGB2LAB.fs"],
    "derivative": ["derivative_t.vs", "derivative_t.gs"],
    "flood": ["flood.vs", "flood.gs"],
    "centroids": ["centroids.vs"],
    "aver": ["aver_exception.vs"],
    "label_replace": ["label_replace.vs", "label_replace.gs"],
}


def glsl_to_cpp(src, stage):
    s = re.sub(r"//[^\n]*", "", src)
    s = re.sub(r"/\*.*?\*/", "", s, flags=re.S)
    s = re.sub(r"#version[^\n]*", "", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*(in|out)\s*;", "", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*", "", s)

    def block(m):
        kind, name, body, inst, arr = m.group(1), m.group(2), m.group(3), m.group(4), m.group(5)
        t = f"{name}_{kind}"
        return f"struct {t} {{{body}}}; {t} {inst}{'[1]' if arr else ''};"

    s = re.sub(r"\b(in|out)\s+(\w+)\s*\{([^}]*)\}\s*(\w+)\s*(\[\s*\])?\s*;", block, s)
    s = re.sub(r"\bflat\s+", "", s)
    s = re.sub(r"\buniform\s+sampler3D\b", "Sampler3D", s)
    s = re.sub(r"\buniform\s+", "", s)
    s = re.sub(r"^(\s*)(in|out)\s+(?=\w+\s+\w+\s*;)", r"\1", s, flags=re.M)
    s = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", s)
    s = re.sub(r"\.(xyz|rgb|xy)\b(?!\s*\()", r".\1()", s)
    return s


HARNESS = r"""
#include <cmath>
#include <cstdint>
#include <cstring>

// GLSL float vectors: non-template operators, so int operands convert to
// float as GLSL's implicit conversion does; swizzles .xy/.xyz/.rgb are
// accessor proxies (the transform rewrites `.xyz` as `.xyz()`).
struct vec2 {
    union { float x; float r; };
    union { float y; float g; };
    vec2() : x(0), y(0) {}
    vec2(float a, float b) : x(a), y(b) {}
};
struct vec3 {
    union { float x; float r; };
    union { float y; float g; };
    union { float z; float b; };
    vec3() : x(0), y(0), z(0) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3 &operator+=(vec3 o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3 &operator+=(float o) { x = x + o; y = y + o; z = z + o; return *this; }
    vec3 &operator-=(float o) { x = x - o; y = y - o; z = z - o; return *this; }
    vec3 &operator*=(float o) { x = x * o; y = y * o; z = z * o; return *this; }
    vec3 &operator/=(float o) { x = x / o; y = y / o; z = z / o; return *this; }
    struct Swz2 xy();
};
struct ivec3 { int x, y, z; ivec3() : x(0), y(0), z(0) {} ivec3(int a, int b, int c) : x(a), y(b), z(c) {} };
struct Swz2 { float &a, &b; operator vec2() const { return vec2(a, b); } };
struct Swz3 {
    float &a, &b, &c;
    operator vec3() const { return vec3(a, b, c); }
    Swz3 &operator=(vec3 v) { a = v.x; b = v.y; c = v.z; return *this; }
    Swz3 &operator/=(float o) { a = a / o; b = b / o; c = c / o; return *this; }
    Swz3 &operator*=(float o) { a = a * o; b = b * o; c = c * o; return *this; }
};
struct vec4 {
    union { float x; float r; };
    union { float y; float g; };
    union { float z; float b; };
    union { float w; float a; };
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float p, float q, float s, float t) : x(p), y(q), z(s), w(t) {}
    vec4(vec2 v, float s, float t) : x(v.x), y(v.y), z(s), w(t) {}
    vec4(vec3 v, float t) : x(v.x), y(v.y), z(v.z), w(t) {}
    Swz3 xyz() { return Swz3{x, y, z}; }
    Swz3 rgb() { return Swz3{x, y, z}; }
    Swz2 xy() { return Swz2{x, y}; }
};
inline Swz2 vec3::xy() { return Swz2{x, y}; }
static inline vec2 operator*(float s, vec2 v) { return vec2(s * v.x, s * v.y); }
static inline vec2 operator-(vec2 v, float s) { return vec2(v.x - s, v.y - s); }
static inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline vec3 operator+(vec3 a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
static inline vec3 operator-(vec3 a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
static inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
static inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
static inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
static inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float floor(float v) { return std::floor(v); }
static inline vec3 floor(vec3 v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
static inline vec3 abs(vec3 v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }

struct Sampler3D { const float *data = nullptr; int W = 1, H = 1, D = 1, C = 4; };

static inline vec4 texture(const Sampler3D &s, vec3 uv)
{
    int x = (int)std::floor(uv.x * (float)s.W), y = (int)std::floor(uv.y * (float)s.H),
        z = (int)std::floor(uv.z * (float)s.D);
    x = x < 0 ? 0 : (x >= s.W ? s.W - 1 : x);
    y = y < 0 ? 0 : (y >= s.H ? s.H - 1 : y);
    z = z < 0 ? 0 : (z >= s.D ? s.D - 1 : z);
    const float *p = s.data + (((size_t)z * s.H + y) * s.W + x) * s.C;
    return vec4(p[0], s.C > 1 ? p[1] : 0.0f, s.C > 2 ? p[2] : 0.0f, s.C > 3 ? p[3] : 1.0f);
}

#define GL_BUILTINS                                                                 \
    struct gl_PerVertex { vec4 gl_Position; };                                      \
    static gl_PerVertex gl_in[1];                                                   \
    static vec4 gl_Position;                                                        \
    static int gl_Layer;                                                            \
    static inline void EmitVertex() {}                                              \
    static inline void EndPrimitive() {}                                            \
    static inline float pow(float a, float b) { return (float)std::pow((double)a, (double)b); }
"""

WRAPPERS = r"""
static float wr_of(int n) { return (float)(1.0 / (float)n); }   // width_ratio = 1.0 / width_f (Image.cpp:329-331)

extern "C" void ref_rgb2lab(const uint8_t *rgb, long n, float *out3)
{
    for (long i = 0; i < n; i++) {
        rgb2lab_fs::f_color = vec3((float)rgb[3 * i] / 255.0f, (float)rgb[3 * i + 1] / 255.0f,
                                   (float)rgb[3 * i + 2] / 255.0f);
        rgb2lab_fs::shader_main();
        out3[3 * i] = rgb2lab_fs::FragColor.x;
        out3[3 * i + 1] = rgb2lab_fs::FragColor.y;
        out3[3 * i + 2] = rgb2lab_fs::FragColor.z;
    }
}

// rgbf: unorm texel values (c / 255), 3 per voxel
extern "C" void ref_derivative(const float *rgbf, int W, int H, int D, float *out)
{
    Sampler3D s; s.data = rgbf; s.W = W; s.H = H; s.D = D; s.C = 3;
    derivative_vs::width_ratio = derivative_gs::width_ratio = wr_of(W);
    derivative_vs::height_ratio = derivative_gs::height_ratio = wr_of(H);
    derivative_vs::depth_ratio = derivative_gs::depth_ratio = wr_of(D);
    derivative_gs::texels = s;
    for (int z = 0; z < D; z++) for (int y = 0; y < H; y++) for (int x = 0; x < W; x++) {
        derivative_vs::aPos = ivec3(x, y, z);
        derivative_vs::shader_main();
        derivative_gs::gs_in[0].gLayer = derivative_vs::vs_out.gLayer;
        derivative_gs::gs_in[0].gTex = derivative_vs::vs_out.gTex;
        derivative_gs::shader_main();
        out[((size_t)z * H + y) * W + x] = derivative_gs::gradient_t;
    }
}

// labels, scolor, mf3, ml3: RGBA32F volumes (4 floats / voxel); image: LAB, 3 floats / voxel
extern "C" void ref_flood(const float *labels, const float *scolor, const float *mf3, const float *ml3,
                          const float *image, int W, int H, int D, float step, float ratio, float *out4)
{
    Sampler3D t; t.W = W; t.H = H; t.D = D;
    flood_gs::texels = t; flood_gs::texels.data = labels;
    flood_gs::sColorImage = t; flood_gs::sColorImage.data = scolor;
    flood_gs::seedMatrixFirst3 = t; flood_gs::seedMatrixFirst3.data = mf3;
    flood_gs::seedMatrixLast3 = t; flood_gs::seedMatrixLast3.data = ml3;
    flood_gs::image = t; flood_gs::image.data = image; flood_gs::image.C = 3;
    flood_vs::width_ratio = flood_gs::width_ratio = wr_of(W);
    flood_vs::height_ratio = flood_gs::height_ratio = wr_of(H);
    flood_vs::depth_ratio = flood_gs::depth_ratio = wr_of(D);
    flood_gs::step = step;
    flood_gs::ratio = ratio;
    for (int z = 0; z < D; z++) for (int y = 0; y < H; y++) for (int x = 0; x < W; x++) {
        flood_vs::aPos = ivec3(x, y, z);
        flood_vs::shader_main();
        flood_gs::gs_in[0].gPos = flood_vs::vs_out.gPos;
        flood_gs::gs_in[0].gTex = flood_vs::vs_out.gTex;
        flood_gs::shader_main();
        float *o = out4 + 4 * (((size_t)z * H + y) * W + x);
        o[0] = flood_gs::f_color.x; o[1] = flood_gs::f_color.y; o[2] = flood_gs::f_color.z; o[3] = flood_gs::f_color.w;
    }
}

// the render-target texel a voxel labelled `id` adds into (id < 0 -> the slot after the seeds)
extern "C" void ref_centroid_target(float id, int W, int H, float ac_seeds_num, int *tx, int *ty)
{
    static float lab[4];
    lab[0] = lab[1] = lab[2] = 0.5f; lab[3] = id;
    static float img[3] = {0, 0, 0};
    Sampler3D t; t.data = lab; t.W = t.H = t.D = 1;
    centroids_vs::texels = t;
    centroids_vs::image = t; centroids_vs::image.data = img; centroids_vs::image.C = 3;
    centroids_vs::width_ratio = wr_of(W);
    centroids_vs::height_ratio = wr_of(H);
    centroids_vs::depth_ratio = 1.0f;
    centroids_vs::ac_seeds_num = ac_seeds_num;
    centroids_vs::aPos = ivec3(0, 0, 0);
    centroids_vs::shader_main();
    vec4 p = centroids_vs::gl_Position;
    *tx = (int)std::floor((p.x + 1.0f) * 0.5f * (float)W);   // viewport transform
    *ty = (int)std::floor((p.y + 1.0f) * 0.5f * (float)H);
}

// one label_replace pass (Image.cpp:1650-1672): labels4 is the RGBA32F flood
// volume (the label in .w); texels labelled last_seed_index take
// dead_seed_index
extern "C" void ref_label_replace(const float *labels4, int W, int H, int D, int dead_seed_index,
                                  int last_seed_index, float *out4)
{
    Sampler3D t; t.data = labels4; t.W = W; t.H = H; t.D = D;
    label_replace_vs::width_ratio = wr_of(W);
    label_replace_vs::height_ratio = wr_of(H);
    label_replace_vs::depth_ratio = wr_of(D);
    label_replace_gs::texels = t;
    label_replace_gs::dead_seed_index = dead_seed_index;
    label_replace_gs::last_seed_index = last_seed_index;
    for (int z = 0; z < D; z++) for (int y = 0; y < H; y++) for (int x = 0; x < W; x++) {
        label_replace_vs::aPos = ivec3(x, y, z);
        label_replace_vs::shader_main();
        label_replace_gs::gs_in[0].gPos = label_replace_vs::vs_out.gPos;
        label_replace_gs::gs_in[0].gTex = label_replace_vs::vs_out.gTex;
        label_replace_gs::shader_main();
        float *o = out4 + 4 * (((size_t)z * H + y) * W + x);
        vec4 c = label_replace_gs::f_color;
        o[0] = c.x; o[1] = c.y; o[2] = c.z; o[3] = c.w;
    }
}

// sum_pos, sum_color: RGBA32F W x H x D volumes (slice 0 holds the sums);
// image: LAB 3 floats / voxel.  For seed `id`: centroid position (x, y, z, id)
// and colour.
extern "C" void ref_aver_exception(const float *sum_pos, const float *sum_color, const float *image,
                                   int W, int H, int D, int id, float *pos4, float *col3)
{
    Sampler3D t; t.W = W; t.H = H; t.D = D;
    aver_vs::sum_pos = t; aver_vs::sum_pos.data = sum_pos;
    aver_vs::sum_color = t; aver_vs::sum_color.data = sum_color;
    aver_vs::image = t; aver_vs::image.data = image; aver_vs::image.C = 3;
    aver_vs::width = (float)W; aver_vs::height = (float)H; aver_vs::depth = (float)D;
    // seeds_index vertex attributes (Image.cpp:108-125)
    int slice = W * H;
    float tex_x = (float)((float)(id % W) + 0.5), tex_y = (float)((float)(id / W) + 0.5),
          tex_z = (float)((float)(id / slice) + 0.5);
    aver_vs::texPos = vec3(tex_x * wr_of(W), tex_y * wr_of(H), tex_z * wr_of(D));
    aver_vs::seedId = (float)id;
    aver_vs::shader_main();
    vec4 c = aver_vs::vs_out.gCentroidPos;
    pos4[0] = c.x; pos4[1] = c.y; pos4[2] = c.z; pos4[3] = c.w;
    vec3 k = aver_vs::vs_out.gCentroidColor;
    col3[0] = k.x; col3[1] = k.y; col3[2] = k.z;
}
"""


def build(force=False):
    """Transforms and compiles the reference shaders; returns the library path,
    or None when the reference tree is not present."""
    if not os.path.isdir(SHADERS):
        return None
    srcs = [os.path.join(SHADERS, f) for p in PROGRAMS.values() for f in p]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            [os.path.getmtime(f) for f in srcs] + [os.path.getmtime(__file__)]):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    parts = [HARNESS]
    for prog, files in PROGRAMS.items():
        for f in files:
            stage = f.rsplit(".", 1)[1]
            ns = f"{prog}_{stage}"
            body = glsl_to_cpp(open(os.path.join(SHADERS, f)).read(), stage)
            parts.append(f"namespace {ns} {{\nGL_BUILTINS\n{body}\n}}\n")
    parts.append(WRAPPERS)
    cpp = os.path.join(OUT, "ref_shaders.cpp")
    with open(cpp, "w") as fh:
        fh.write("\n".join(parts))
    tmp = LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-fsingle-precision-constant",
           "-ffp-contract=off", "-w", "-o", tmp, cpp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("reference shader build failed:\n" + p.stderr[-6000:])
    os.replace(tmp, LIB)
    return LIB


# ---------------------------------------------------------------------------
# Host functions of the reference compiled from its C++ files: the function
# text is cut out where it lies (comments dropped, `Class::` removed) and
# placed in a struct that supplies the class members it reads.
# ---------------------------------------------------------------------------
HOST_LIB = os.path.join(OUT, "libref_host.so")
HOST_FUNCS = [
    # (file, signature start, shim struct, members, stop marker): a function is
    # cut whole, or up to the stop marker (the first GL call that follows its
    # host arithmetic) and closed there.  A member `cout` shadows std::cout so
    # the functions' progress messages stay out of the test output.
    ("GPU-AS/Image.cpp", "void Image::EnforceLabelConnectivity3D(", "ImageShim",
     "int texel_num, depth, height, width, slice_num;", None),
    ("streamGPU-AS/Render.cpp", "void Render::label_connected3D(", "RenderShim",
     "int width, height, depth_all;", None),
    # Image::init_seeds (GPU-AS/Image.cpp:20-92): the regular seed grid
    ("GPU-AS/Image.cpp", "void Image::init_seeds(", "SeedShim",
     "int texel_num, seeds_num, width, height, depth, s, max_s, ac_seeds_num, dNum, wNum, hNum;\n"
     "    string dbname; vector<float> seeds_lsc; ostringstream cout;", "glGenVertexArrays"),
    # Image::sequence_label (GPU-AS/Image.cpp:1727-1778): the > 3 dead-seed remap
    # and the raster-order fill of label -1
    ("GPU-AS/Image.cpp", "void Image::sequence_label(", "SequenceShim",
     "int texel_num; ostringstream cout;", None),
    # Image::initialization (GPU-AS/Image.cpp:350-620): its host code before the
    # first GL call (cell ranges, the cell-id grid) and after the readback of
    # the density sums (the redistribution); the GL part in between is the
    # two density shaders, pinned on their own, and is replaced by the glue
    # INIT_GLUE, which keeps the grid and supplies the sums as `res`
    ("GPU-AS/Image.cpp", "void Image::initialization(", "InitShim",
     "int texel_num, slice_num, width, height, depth, ac_seeds_num, dNum, hNum, wNum;\n"
     "    vector<float> seeds_lsc, seeds_lsc_adjust; float *grid_out; const float *res_in;\n"
     "    ostringstream cout;", ("glBindFramebuffer", "vector<float> seed_density;")),
    # Image::init_variables (the ratio), reset_variables and flood
    # (GPU-AS/Image.cpp:1048-1190): compiled whole against the GL stubs of
    # HOST_PRELUDE, the recording Shader returns the step and ratio of every pass
    ("GPU-AS/Image.cpp", "void Image::init_variables(", "FloodShim",
     "int s, texel_num, current_buffer, seed_range, flood_iter; float compactness, ratio, step_length;\n"
     "    float width_ratio, height_ratio, depth_ratio; GLuint frameBuffer_flood, VAO_all_t;\n"
     "    GLuint texture_flood[5], texture_image[4]; GLenum buffers_flood[5]; ostringstream cout;\n"
     "    @void Image::reset_variables(@void Image::flood(", None),
    # the streaming program's per-window grid and density placement
    # (streamGPU-AS/Image.cpp:26-120, 321-595): the same host code shapes
    ("streamGPU-AS/Image.cpp", "void Image::initialization_grid(", "StreamGridShim",
     "int texel_num, seeds_num, width, height, depth, s, max_s, ac_seeds_num, dNum, wNum, hNum;\n"
     "    vector<float> seeds_lsc, seeds_lsc_adjust; ostringstream cout;", "glGenVertexArrays"),
    # Image::print_sv_txt (GPU-AS/Image.cpp:1780-1806): the txt label file
    ("GPU-AS/Image.cpp", "void Image::print_sv_txt(", "TxtShim",
     "int depth, height, width, slice_num; ostringstream cout;", None),
    ("streamGPU-AS/Image.cpp", "void Image::initialization_adjust(", "StreamInitShim",
     "int texel_num, slice_num, width, height, depth, ac_seeds_num, dNum, hNum, wNum;\n"
     "    vector<float> seeds_lsc, seeds_lsc_adjust; float *grid_out; const float *res_in;\n"
     "    ostringstream cout;", ("glBindFramebuffer", "vector<float> seed_density;")),
]

HOST_PRELUDE = """#include <cmath>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <utility>
#include <vector>
using namespace std;
// GL calls of the compiled functions, as no-ops (no context exists here), and
// the shader program type as a recorder of the float uniforms set on it
typedef unsigned int GLuint;
typedef unsigned int GLenum;
enum { GL_FRAMEBUFFER, GL_COLOR_BUFFER_BIT, GL_TEXTURE_3D, GL_POINTS, GL_TEXTURE0, GL_TEXTURE1, GL_TEXTURE2,
       GL_TEXTURE3, GL_TEXTURE4 };
static inline void glBindFramebuffer(GLenum, GLuint) {}
static inline void glDrawBuffers(int, const GLenum *) {}
static inline void glClearColor(float, float, float, float) {}
static inline void glClear(GLenum) {}
static inline void glActiveTexture(GLenum) {}
static inline void glBindTexture(GLenum, GLuint) {}
static inline void glBindVertexArray(GLuint) {}
static inline void glDrawArrays(GLenum, int, int) {}
struct Shader {
    vector<pair<string, float>> floats;
    void use() {}
    void setInt(const string &, int) {}
    void setFloat(const string &name, float v) { floats.push_back(make_pair(name, v)); }
};
"""

INIT_GLUE = """
    memcpy(grid_out, grid, sizeof(float) * texel_num);
    delete[] grid;
    float *res = new float[4 * ac_seeds_num];
    for (int q = 0; q < ac_seeds_num; q++) res[4 * q] = res_in[q];
"""

HOST_WRAPPERS = r"""
extern "C" int ref_enforce_connectivity(const int *labels, int W, int H, int D, int supsz, int *out)
{
    ImageShim s;
    s.width = W; s.height = H; s.depth = D; s.slice_num = W * H; s.texel_num = W * H * D;
    int *nl = out;
    int num = 0;
    s.EnforceLabelConnectivity3D(const_cast<int *>(labels), nl, num, supsz);
    return num;
}

extern "C" int ref_label_connected3D(const int *labels, int W, int H, int D, int supsz, int *out)
{
    RenderShim s;
    s.width = W; s.height = H; s.depth_all = D;
    int num = 0;
    s.label_connected3D(const_cast<int *>(labels), out, num, supsz);
    return num;
}

// the seed grid: (x, y, z, id) per seed into out (room for cap seeds), and
// s, dNum, hNum, wNum, ac_seeds_num into g5; returns the seeds placed
extern "C" int ref_init_seeds(int W, int H, int D, int K, int middlebury, float *out, int cap, int *g5)
{
    SeedShim s;
    s.width = W; s.height = H; s.depth = D; s.seeds_num = K; s.texel_num = W * H * D;
    s.dbname = middlebury ? "MiddleburyFlow" : "";
    s.init_seeds();
    const int n = (int)(s.seeds_lsc.size() / 4);
    for (int i = 0; i < n && i < cap; i++)
        for (int k = 0; k < 4; k++) out[4 * i + k] = s.seeds_lsc[4 * i + k];
    g5[0] = s.s; g5[1] = s.dNum; g5[2] = s.hNum; g5[3] = s.wNum; g5[4] = s.ac_seeds_num;
    return n;
}

// check_dead_seeds' map (GPU-AS/Image.cpp:1597-1617: live seeds numbered in
// seed order, from their voxel counts), then sequence_label on the labels
// Image::init_seeds, then the host parts of Image::initialization with the
// density sums given (one per grid cell); writes the cell-id grid (W*H*D)
// and the redistributed seeds (x, y, z, id), returns how many
extern "C" int ref_initialization(int W, int H, int D, int K, int middlebury, const float *density,
                                  float *grid_out, float *seeds_out, int cap)
{
    SeedShim g;
    g.width = W; g.height = H; g.depth = D; g.seeds_num = K; g.texel_num = W * H * D;
    g.dbname = middlebury ? "MiddleburyFlow" : "";
    g.init_seeds();
    InitShim s;
    s.width = W; s.height = H; s.depth = D; s.texel_num = W * H * D; s.slice_num = W * H;
    s.ac_seeds_num = g.ac_seeds_num; s.dNum = g.dNum; s.hNum = g.hNum; s.wNum = g.wNum;
    s.seeds_lsc = g.seeds_lsc; s.grid_out = grid_out; s.res_in = density;
    Shader a, b;
    s.initialization(a, b);
    const int n = (int)(s.seeds_lsc_adjust.size() / 4);
    for (int i = 0; i < n && i < cap; i++)
        for (int k = 0; k < 4; k++) seeds_out[4 * i + k] = s.seeds_lsc_adjust[4 * i + k];
    return n;
}

// the streaming program's window grid and density placement, as above
extern "C" int ref_stream_initialization(int W, int H, int D, int K, const float *density, float *grid_out,
                                         float *seeds_out, int cap, int *g5)
{
    StreamGridShim g;
    g.width = W; g.height = H; g.depth = D; g.seeds_num = K; g.texel_num = W * H * D;
    int kp = 0;
    g.initialization_grid(kp);
    g5[0] = g.s; g5[1] = g.dNum; g5[2] = g.hNum; g5[3] = g.wNum; g5[4] = kp;
    if (!density) {                                      // the grid alone
        const int n = (int)(g.seeds_lsc.size() / 4);
        for (int i = 0; i < n && i < cap; i++)
            for (int k = 0; k < 4; k++) seeds_out[4 * i + k] = g.seeds_lsc[4 * i + k];
        return n;
    }
    StreamInitShim s;
    s.width = W; s.height = H; s.depth = D; s.texel_num = W * H * D; s.slice_num = W * H;
    s.ac_seeds_num = g.ac_seeds_num; s.dNum = g.dNum; s.hNum = g.hNum; s.wNum = g.wNum;
    s.seeds_lsc = g.seeds_lsc; s.grid_out = grid_out; s.res_in = density;
    Shader a, b;
    s.initialization_adjust(a, b);
    const int n = (int)(s.seeds_lsc_adjust.size() / 4);
    for (int i = 0; i < n && i < cap; i++)
        for (int k = 0; k < 4; k++) seeds_out[4 * i + k] = s.seeds_lsc_adjust[4 * i + k];
    return n;
}

// the JFA passes of one Lloyd iteration for base step s: Image::init_variables
// (compactness 8, ratio), then Image::flood with the uniforms recorded; writes
// each pass's step and ratio, returns the pass count, *ratio_out the ratio
extern "C" int ref_flood_ladder(int s_, float *steps, float *ratios, int cap, float *ratio_out)
{
    FloodShim f;
    f.s = s_; f.texel_num = 1; f.current_buffer = 0;
    f.init_variables();
    Shader sh;
    f.flood(sh, 1);
    int n = 0;
    for (size_t i = 0; i + 1 < sh.floats.size(); i++)
        if (sh.floats[i].first == "step" && sh.floats[i + 1].first == "ratio") {
            if (n < cap) { steps[n] = sh.floats[i].second; ratios[n] = sh.floats[i + 1].second; }
            n++;
        }
    *ratio_out = f.ratio;
    return n;
}

// Image::print_sv_txt with output_label = true: writes <path_stem>.txt
extern "C" void ref_print_sv_txt(int *labels, int W, int H, int D, const char *path_stem)
{
    TxtShim s;
    s.width = W; s.height = H; s.depth = D; s.slice_num = W * H;
    s.print_sv_txt(labels, string(path_stem), true, false);
}

extern "C" void ref_sequence_label(int *labels, long n, const long long *counts, int Kp, int dead_seed)
{
    map<int, int> m;
    int valid = 0;
    for (int i = 0; i < Kp; i++)
        if (int(float(counts[i])) >= 1) m.insert(pair<int, int>(i, valid++));
    SequenceShim s;
    s.texel_num = (int)n;
    s.sequence_label(labels, m, dead_seed != 0);
}
"""


# Host code that lies inside a longer function of the reference: the text
# between two markers is cut out and placed in a wrapper of this project's
# (the shim supplies the surrounding function's locals and members).
SNIPPETS = [
    # the block partition of the streaming Render::run (streamGPU-AS/Render.cpp:199-241)
    ("streamGPU-AS/Render.cpp", "int Render::run(", "block_size = 30;", "block_num = block_interval.size() / 2;",
     "struct StreamBlocksShim {\n    int block_size, block_num, depth_all; ostringstream cout;\n"
     "    int run(int D, int *out, int cap) {\n        depth_all = D;\n@SNIPPET@\n"
     "        for (int i = 0; i < (int)block_interval.size() && i < cap; i++) out[i] = block_interval[i];\n"
     "        return block_num;\n    }\n};\n"
     "extern \"C\" int ref_stream_blocks(int D, int *out, int cap) { StreamBlocksShim s; return s.run(D, out, cap); }\n"),
    # the kept seeds of post_and_next (streamGPU-AS/Render.cpp:519-540)
    ("streamGPU-AS/Render.cpp", "void Render::post_and_next(", "int sind = 0;", "sind += 4;",
     "struct KeepShim {\n    int block_size, kept_seeds_num; vector<float> kept_seeds; ostringstream cout;\n"
     "    int run(const float *info, int n, int bs, float *out) {\n        block_size = bs;\n"
     "        vector<float> seeds_info(info, info + 4 * n);\n        int final_seeds_num = n;\n"
     "        int one_third = int(block_size / 3);\n        int two_third = block_size - one_third;\n"
     "@SNIPPET@\n        }\n"
     "        for (int i = 0; i < (int)kept_seeds.size(); i++) out[i] = kept_seeds[i];\n"
     "        return kept_seeds_num;\n    }\n};\n"
     "extern \"C\" int ref_stream_keep(const float *info, int n, int bs, float *out)"
     " { KeepShim s; return s.run(info, n, bs, out); }\n"),
]


def _snippet(text, fn_start, start, stop):
    fn = _cut_function(text, fn_start)
    i = fn.index(start)
    j = fn.index(stop, i) + len(stop)
    return fn[i:j]


def _strip_comments(src):
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def _cut_function(src, start):
    i = src.index(start)
    j = src.index("{", i)
    depth = 0
    for k in range(j, len(src)):
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[i:k + 1]
    raise ValueError("unbalanced braces after " + start)


def build_host(force=False):
    """Compiles the reference's host functions listed above; returns the
    library path, or None when the reference tree is not present."""
    srcs = [os.path.join(REF, f) for f, _, _, _, _ in HOST_FUNCS]
    if not all(os.path.exists(f) for f in srcs):
        return None
    if not force and os.path.exists(HOST_LIB) and os.path.getmtime(HOST_LIB) >= max(
            [os.path.getmtime(f) for f in srcs] + [os.path.getmtime(__file__)]):
        return HOST_LIB
    os.makedirs(OUT, exist_ok=True)
    parts = [HOST_PRELUDE]
    for path, start, shim, members, stop in HOST_FUNCS:
        text = _strip_comments(open(os.path.join(REF, path), encoding="latin-1").read())
        if "@" in members:                         # more member functions of the same shim
            members, *more = members.split("@")
            fns = [_cut_function(text, f) for f in [start] + more]
            fns = [re.sub(r"\b\w+::(\w+\s*\()", r"\1", f, count=1) for f in fns]
            parts.append(f"struct {shim} {{\n    {members}\n" + "\n".join(fns) + "\n};\n")
            continue
        if stop is None:
            fn = _cut_function(text, start)
        elif isinstance(stop, tuple):              # host code, glue, host code to the end
            whole = _cut_function(text, start)
            fn = whole[:whole.index(stop[0])] + INIT_GLUE + whole[whole.index(stop[1]):]
        else:                                      # the host part, closed at the marker
            i = text.index(start)
            fn = text[i:text.index(stop, i)] + "}"
        fn = re.sub(r"\b\w+::(\w+\s*\()", r"\1", fn, count=1)
        parts.append(f"struct {shim} {{\n    {members}\n{fn}\n}};\n")
    for path, fn_start, start, stop, wrapper in SNIPPETS:
        text = _strip_comments(open(os.path.join(REF, path), encoding="latin-1").read())
        parts.append(wrapper.replace("@SNIPPET@", _snippet(text, fn_start, start, stop)))
    parts.append(HOST_WRAPPERS)
    cpp = os.path.join(OUT, "ref_host.cpp")
    with open(cpp, "w", encoding="latin-1") as fh:
        fh.write("\n".join(parts))
    tmp = HOST_LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-w", "-o", tmp, cpp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("reference host build failed:\n" + p.stderr[-6000:])
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


if __name__ == "__main__":
    print(build(force=True))
    print(build_host(force=True))
