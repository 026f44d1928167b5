// asv_synth.cpp -- seeded synthetic clips and the host I/O of the pipeline
// (declared in include/asv_host.h).
#include "asv_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

inline uint64_t mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// counter-based uniform in [0, 1)
inline double uni(uint64_t seed, uint64_t stream, uint64_t ctr)
{
    uint64_t h = mix64(seed ^ mix64(stream * 0x632be59bd9b4e019ull + ctr));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

struct Ellipse {
    double cx, cy, a, b, phi, vx, vy;
    double rgb[3];
};

// CIELAB (D65) -> sRGB8, clipped
void lab_to_rgb8(double L, double A, double B, double out[3])
{
    double fy = (L + 16.0) / 116.0, fx = fy + A / 500.0, fz = fy - B / 200.0;
    auto finv = [](double f) { double f3 = f * f * f; return f3 > 0.008856 ? f3 : (116.0 * f - 16.0) / 903.3; };
    double X = 0.950456 * finv(fx), Y = finv(fy), Z = 1.088754 * finv(fz);
    double r = 3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z;
    double g = -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z;
    double b = 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z;
    double lin[3] = { r, g, b };
    for (int k = 0; k < 3; k++) {
        double v = std::min(std::max(lin[k], 0.0), 1.0);
        v = v <= 0.0031308 ? 12.92 * v : 1.055 * std::pow(v, 1.0 / 2.4) - 0.055;
        out[k] = std::min(std::max(v * 255.0, 0.0), 255.0);
    }
}

struct Scene {
    const asv_synth_params *p;
    std::vector<Ellipse> e;
    double c0[3], c1[3], dir_x, dir_y;
};

void build_scene(const asv_synth_params *p, Scene *s)
{
    s->p = p;
    const uint64_t sd = p->seed;
    double m = std::min(p->W, p->H);
    for (int k = 0; k < 3; k++) {
        s->c0[k] = 40.0 + 170.0 * uni(sd, 1, k);
        s->c1[k] = 40.0 + 170.0 * uni(sd, 2, k);
    }
    double th = 2.0 * M_PI * uni(sd, 3, 0);
    s->dir_x = std::cos(th);
    s->dir_y = std::sin(th);
    s->e.resize(p->n_ellipses);
    for (int i = 0; i < p->n_ellipses; i++) {
        Ellipse &E = s->e[i];
        uint64_t st = 100 + (uint64_t)i;
        E.cx = p->W * uni(sd, st, 0);
        E.cy = p->H * uni(sd, st, 1);
        E.a = m / 24.0 + (m / 6.0 - m / 24.0) * uni(sd, st, 2);
        E.b = E.a * (0.4 + 0.6 * uni(sd, st, 3));
        E.phi = M_PI * uni(sd, st, 4);
        double sp = p->vmax * uni(sd, st, 5), dth = 2.0 * M_PI * uni(sd, st, 6);
        E.vx = sp * std::cos(dth);
        E.vy = sp * std::sin(dth);
        double L = 25.0 + 65.0 * uni(sd, st, 7), A = -60.0 + 120.0 * uni(sd, st, 8),
               B = -60.0 + 120.0 * uni(sd, st, 9);
        lab_to_rgb8(L, A, B, E.rgb);
    }
}

// velocity of ellipse i between frame f and f+1
inline void vel(const Scene &s, int i, long f, double *vx, double *vy)
{
    const Ellipse &E = s.e[i];
    double j = s.p->jitter;
    *vx = E.vx + (j > 0 ? j * (2.0 * uni(s.p->seed, 1000 + (uint64_t)i, 2 * (uint64_t)f) - 1.0) : 0.0);
    *vy = E.vy + (j > 0 ? j * (2.0 * uni(s.p->seed, 1000 + (uint64_t)i, 2 * (uint64_t)f + 1) - 1.0) : 0.0);
}

inline void drift(const Scene &s, long f, double *ox, double *oy)
{
    if (s.p->drift_amp <= 0.f || s.p->drift_period <= 0.f) { *ox = *oy = 0.0; return; }
    double w = 2.0 * M_PI * (double)f / s.p->drift_period;
    *ox = s.p->drift_amp * std::sin(w);
    *oy = 0.5 * s.p->drift_amp * std::sin(0.5 * w);
}

void render_frame(const Scene &s, long f, uint8_t *rgb, float *fwd, float *bwd, int32_t *ids = nullptr)
{
    const asv_synth_params *p = s.p;
    const int W = p->W, H = p->H, n = (int)s.e.size();
    std::vector<double> cx(n), cy(n), vfx(n), vfy(n), vbx(n), vby(n);
    for (int i = 0; i < n; i++) {
        double x = s.e[i].cx, y = s.e[i].cy, vx, vy;
        for (long k = 0; k < f; k++) { vel(s, i, k, &vx, &vy); x += vx; y += vy; }
        cx[i] = x; cy[i] = y;
        vel(s, i, f, &vfx[i], &vfy[i]);
        if (f > 0) { vel(s, i, f - 1, &vx, &vy); vbx[i] = -vx; vby[i] = -vy; }
        else { vbx[i] = vby[i] = 0.0; }
    }
    double ox, oy, ox1, oy1, ox0, oy0;
    drift(s, f, &ox, &oy);
    drift(s, f + 1, &ox1, &oy1);
    drift(s, f - 1, &ox0, &oy0);
    std::vector<int> top((size_t)W * H, -1);
    for (int i = 0; i < n; i++) {
        const Ellipse &E = s.e[i];
        double r = std::max(E.a, E.b) + 1.0;
        int x0 = std::max(0, (int)std::floor(cx[i] - r)), x1 = std::min(W - 1, (int)std::ceil(cx[i] + r));
        int y0 = std::max(0, (int)std::floor(cy[i] - r)), y1 = std::min(H - 1, (int)std::ceil(cy[i] + r));
        double c = std::cos(E.phi), sn = std::sin(E.phi);
        for (int y = y0; y <= y1; y++)
            for (int x = x0; x <= x1; x++) {
                double dx = x + 0.5 - cx[i], dy = y + 0.5 - cy[i];
                double u = (dx * c + dy * sn) / E.a, v = (-dx * sn + dy * c) / E.b;
                if (u * u + v * v <= 1.0) top[(size_t)y * W + x] = i;
            }
    }
    const double L = (double)W + (double)H;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            size_t q = (size_t)y * W + x;
            int t = top[q];
            if (ids) ids[q] = t >= 0 ? t : n;   // ground truth: the ellipse on top, n = background
            double col[3];
            if (t >= 0) {
                for (int k = 0; k < 3; k++) col[k] = s.e[t].rgb[k];
                if (fwd) { fwd[2 * q] = (float)vfx[t]; fwd[2 * q + 1] = (float)vfy[t]; }
                if (bwd) { bwd[2 * q] = (float)vbx[t]; bwd[2 * q + 1] = (float)vby[t]; }
            } else {
                double tt = 0.5 + ((x + 0.5 - 0.5 * W - ox) * s.dir_x + (y + 0.5 - 0.5 * H - oy) * s.dir_y) / L;
                tt = std::min(std::max(tt, 0.0), 1.0);
                for (int k = 0; k < 3; k++) col[k] = s.c0[k] + (s.c1[k] - s.c0[k]) * tt;
                if (fwd) { fwd[2 * q] = (float)(ox1 - ox); fwd[2 * q + 1] = (float)(oy1 - oy); }
                if (bwd) {
                    bwd[2 * q] = f > 0 ? (float)(ox0 - ox) : 0.f;
                    bwd[2 * q + 1] = f > 0 ? (float)(oy0 - oy) : 0.f;
                }
            }
            for (int k = 0; k < 3; k++) {
                double nz = 0.0;
                if (p->noise_sigma > 0.f) {
                    uint64_t ctr = ((uint64_t)f * H * W + q) * 3 + k;
                    double u1 = uni(p->seed, 7, 2 * ctr), u2 = uni(p->seed, 7, 2 * ctr + 1);
                    if (u1 < 1e-300) u1 = 1e-300;
                    nz = p->noise_sigma * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
                }
                double v = std::floor(col[k] + nz + 0.5);
                rgb[3 * q + k] = (uint8_t)std::min(std::max(v, 0.0), 255.0);
            }
        }
}

} // namespace

extern "C" int asv_synth_clip(const asv_synth_params *p, uint8_t *rgb, float *fwd, float *bwd)
{
    if (!p || !rgb || p->W < 1 || p->H < 1 || p->nframes < 1 || p->n_ellipses < 0 || p->frame0 < 0)
        return -1;
    Scene s;
    build_scene(p, &s);
    const size_t fr = (size_t)p->W * p->H;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < p->nframes; i++)
        render_frame(s, (long)p->frame0 + i, rgb + 3 * fr * i, fwd ? fwd + 2 * fr * i : nullptr,
                     bwd ? bwd + 2 * fr * i : nullptr);
    return 0;
}

extern "C" int asv_synth_truth(const asv_synth_params *p, int32_t *ids)
{
    if (!p || !ids || p->W < 1 || p->H < 1 || p->nframes < 1 || p->n_ellipses < 0 || p->frame0 < 0)
        return -1;
    Scene s;
    build_scene(p, &s);
    const size_t fr = (size_t)p->W * p->H;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < p->nframes; i++) {
        std::vector<uint8_t> rgb(3 * fr);
        render_frame(s, (long)p->frame0 + i, rgb.data(), nullptr, nullptr, ids + fr * i);
    }
    return 0;
}

extern "C" int asv_preprocess_frame(const uint8_t *bgr, int W, int H, uint8_t *rgb_tex)
{
    if (!bgr || !rgb_tex || W < 1 || H < 1) return -1;
    auto refl = [](int i, int n) {
        if (n == 1) return 0;
        while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
        return i;
    };
    static const int w[3] = { 1, 2, 1 };
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int c = 0; c < 3; c++) {
                int acc = 0;
                for (int j = -1; j <= 1; j++)
                    for (int i = -1; i <= 1; i++)
                        acc += w[j + 1] * w[i + 1] * bgr[3 * ((size_t)refl(y + j, H) * W + refl(x + i, W)) + c];
                int v = (acc + 8) >> 4;
                // BGR -> RGB and flip: output row H-1-y, channel 2-c
                rgb_tex[3 * ((size_t)(H - 1 - y) * W + x) + (2 - c)] = (uint8_t)v;
            }
    return 0;
}

extern "C" int asv_write_labels_txt(const char *path, const int32_t *labels, int W, int H, int D)
{
    if (!path || !labels) return -1;
    FILE *f = std::fopen(path, "w");
    if (!f) return -2;
    char buf[32];
    for (int t = 0; t < D; t++) {
        for (int i = H - 1; i >= 0; i--) {
            const int32_t *row = labels + ((size_t)t * H + i) * W;
            for (int j = 0; j < W; j++) {
                int n = std::snprintf(buf, sizeof(buf), "%d", row[j]);
                std::fputs(buf, f);
                for (int k = n; k < 4; k++) std::fputc(' ', f);
                std::fputc(' ', f);
            }
            std::fputc('\n', f);
        }
        std::fputs("\n\n", f);
    }
    return std::fclose(f) == 0 ? 0 : -3;
}

// the render writer needs the palette of asv_png.cpp; a build of the
// generator alone (ASV_SYNTH_ONLY) leaves it out
#ifndef ASV_SYNTH_ONLY
extern "C" int asv_write_render_ppm(const char *prefix, const int32_t *labels, int W, int H, int D,
                                    int n_labels)
{
    if (!prefix || !labels || n_labels < 0 || W <= 0 || H <= 0 || D < 0) return -1;
    std::vector<uint8_t> rgb((size_t)W * H * 3 * D);
    if (asv_render_rgb(labels, W, H, D, n_labels, rgb.data()) != 0) return -1;   // the same palette
    const size_t frame = (size_t)W * H * 3;
    for (int t = 0; t < D; t++) {
        char name[4096];
        std::snprintf(name, sizeof(name), "%s%05d.ppm", prefix, t);
        FILE *f = std::fopen(name, "wb");
        if (!f) return -2;
        std::fprintf(f, "P6\n%d %d\n255\n", W, H);
        std::fwrite(rgb.data() + frame * t, 1, frame, f);
        if (std::fclose(f) != 0) return -3;
    }
    return 0;
}
#endif
