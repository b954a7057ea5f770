/*
 * sr_oracle.cpp — CPU restatement of softrender's rendering path.
 * TEST INFRASTRUCTURE ONLY (parity oracle and timed CPU baseline); the product
 * library never links or calls it.  Compile with -O2 -ffp-contract=off and no
 * fast-math so every FP32 operation is an IEEE-754 operation in source order.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the rust-softrender repository).  Shader, blend and sampling arithmetic
 * (user code in the reference's examples) comes from include/sr_shaders.h.
 */
#include "sr_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int MAXK = 16;

/* ClipVertex / ScreenVertex {position: Vector4, uniforms: K}
 * (src/geometry/clipvertex.rs:6-14, screenvertex.rs:8-15) */
struct CV {
    float p[4];
    float k[MAXK];
};

enum { VS_MVP_POS_NRM, VS_MVP_POS_NRM_UV, VS_CLIP_COLOR, VS_CLIP_RGBA8 };
enum { FS_BLINN_PHONG_DIR, FS_TEXTURED_BLINN_PHONG, FS_VERTEX_COLOR, FS_ACES_LIGHTS, FS_CONSTANT_COLOR };
enum { BLEND_REPLACE, BLEND_OVER };
enum { GS_CLIP, GS_VERTEX_NORMALS, GS_FACE_NORMALS };

struct Ctx {
    const or_draw* d;
    const sr_uniforms* U;
    or_fb* fb;
    int vs, fs, blend, gs;
    int nk;
    uint32_t W, H;
    uint8_t sref;
    bool has_stencil;
    std::atomic<uint64_t> fragments{0};
    std::atomic<uint32_t> nan_bbox{0};
};

/* ------------------------------------------------------------ threading */
/* Pool::scoped with `thread_count` workers (src/pipeline/mod.rs:115). */
template <class F>
void run_threads(int n, F f) {
    if (n <= 1) { f(); return; }
    std::vector<std::thread> ts;
    ts.reserve(n);
    for (int i = 0; i < n; ++i) ts.emplace_back(f);
    for (auto& t : ts) t.join();
}

/* n workers, worker k receiving k (the deterministic mode's fixed split). */
template <class F>
void run_threads_indexed(int n, F f) {
    if (n <= 1) { f(0); return; }
    std::vector<std::thread> ts;
    ts.reserve(n);
    for (int i = 0; i < n; ++i) ts.emplace_back(f, i);
    for (auto& t : ts) t.join();
}

/* Mapper::map / map_move (src/parallel.rs:57-111): chunks of
 * CACHE_LINE_SIZE * size_of::<U>() elements claimed by an atomic counter. */
template <class F>
void mapper(size_t len, size_t fetch, int nthreads, F f) {
    std::atomic<size_t> index{0};
    run_threads(nthreads, [&]() {
        for (;;) {
            size_t i = index.fetch_add(fetch, std::memory_order_relaxed);
            if (i >= len) break;
            size_t mx = std::min(i + fetch, len);
            for (; i < mx; ++i) f(i);
        }
    });
}

/* ----------------------------------------------------------- shaders */
int vs_id(const char* n) {
    std::string s = n ? n : "";
    if (s == "mvp_pos_nrm") return VS_MVP_POS_NRM;
    if (s == "mvp_pos_nrm_uv") return VS_MVP_POS_NRM_UV;
    if (s == "clip_color") return VS_CLIP_COLOR;
    if (s == "clip_rgba8") return VS_CLIP_RGBA8;
    return -1;
}
int vs_planes(int vs) { return vs == VS_MVP_POS_NRM ? 6 : vs == VS_CLIP_RGBA8 ? 4 : 8; }
int vs_nk(int vs) { return vs == VS_MVP_POS_NRM ? 8 : vs == VS_MVP_POS_NRM_UV ? 10 : 4; }
int fs_id(const char* n) {
    std::string s = n ? n : "";
    if (s == "blinn_phong_dir") return FS_BLINN_PHONG_DIR;
    if (s == "textured_blinn_phong") return FS_TEXTURED_BLINN_PHONG;
    if (s == "vertex_color") return FS_VERTEX_COLOR;
    if (s == "aces_lights") return FS_ACES_LIGHTS;
    if (s == "constant_color") return FS_CONSTANT_COLOR;
    return -1;
}
int blend_id(const char* n) {
    std::string s = n ? n : "replace";
    if (s == "replace") return BLEND_REPLACE;
    if (s == "over") return BLEND_OVER;
    return -1;
}
int gs_id(const char* n) {
    std::string s = n ? n : "clip";
    if (s == "clip") return GS_CLIP;
    if (s == "vertex_normals") return GS_VERTEX_NORMALS;
    if (s == "face_normals") return GS_FACE_NORMALS;
    return -1;
}

CV run_vs(const Ctx& c, uint32_t i) {
    float a[8];
    int np = vs_planes(c.vs);
    for (int j = 0; j < np; ++j) a[j] = c.d->planes[j][i];
    CV out;
    std::memset(&out, 0, sizeof(out));
    sr_v4 clip;
    if (c.vs == VS_MVP_POS_NRM) clip = sr_vs_mvp_pos_nrm(c.U, a, out.k);
    else if (c.vs == VS_MVP_POS_NRM_UV) clip = sr_vs_mvp_pos_nrm_uv(c.U, a, out.k);
    else if (c.vs == VS_CLIP_COLOR) clip = sr_vs_clip_color(c.U, a, out.k);
    else clip = sr_vs_clip_rgba8(c.U, a, out.k);
    out.p[0] = clip.x; out.p[1] = clip.y; out.p[2] = clip.z; out.p[3] = clip.w;
    return out;
}

sr_v4 v4(const float* f) { return sr_make_v4(f[0], f[1], f[2], f[3]); }

/* The fragment closure: returns the RGBA f32 colour (none of these discard). */
sr_v4 run_fs(const Ctx& c, const CV& sv) {
    const sr_uniforms* U = c.U;
    switch (c.fs) {
    case FS_BLINN_PHONG_DIR:
        return sr_blinn_phong(U, v4(sv.k), v4(sv.k + 4), v4(U->color));
    case FS_TEXTURED_BLINN_PHONG: {
        sr_v4 t = sr_sample(c.d->texture, c.d->tex_f32, c.d->tex_w, c.d->tex_h, sv.k[8], sv.k[9],
                            (int)c.d->tex_filter, (int)c.d->tex_edge);
        t = sr_decode_gamma(t, U->gamma);
        return sr_blinn_phong(U, v4(sv.k), v4(sv.k + 4), t);
    }
    case FS_VERTEX_COLOR:
        return v4(sv.k);
    case FS_ACES_LIGHTS:
        return sr_aces_lights(U, v4(sv.k), v4(sv.k + 4));
    default:
        return v4(U->color);
    }
}

/* ----------------------------------------------------------- geometry */

/* ClipVertex::normalize (src/geometry/clipvertex.rs:89-127) */
void normalize_pos(const float* in, const float* vp, float* out) {
    float x = in[0], y = in[1], z = in[2], w = in[3];
    float left = vp[0], bottom = vp[1], width = vp[2], height = vp[3], near_ = vp[4], far_ = vp[5];
    float right = left + width;
    float top = bottom + height;
    float m[16] = {(right - left) / 2.0f, 0.0f, 0.0f, (right + left) / 2.0f,
                   0.0f, (top - bottom) / -2.0f, 0.0f, (top + bottom) / 2.0f,
                   0.0f, 0.0f, (far_ - near_) / -2.0f, (far_ + near_) / -2.0f,
                   0.0f, 0.0f, 0.0f, 1.0f};
    sr_v4 s = sr_m4_mul_v4(m, sr_make_v4(x / w, y / w, z / w, 1.0f));
    s.w = 1.0f / w;
    out[0] = s.x; out[1] = s.y; out[2] = s.z; out[3] = s.w;
}
CV normalize(const CV& v, const float* vp, int nk) {
    CV o;
    normalize_pos(v.p, vp, o.p);
    for (int i = 0; i < nk; ++i) o.k[i] = v.k[i];
    return o;
}

/* ClippingPlane::has_inside (src/geometry/clip.rs:33-44); plane order
 * Left, Right, Top, Bottom, Near, Far (ALL_CLIPPING_PLANES, clip.rs:22-29). */
bool has_inside(int plane, const CV& v) {
    float x = v.p[0], y = v.p[1], z = v.p[2], w = v.p[3];
    switch (plane) {
    case 0: return x >= -w;
    case 1: return x <= w;
    case 2: return y >= -w;
    case 3: return y <= w;
    case 4: return z >= 0.0f;
    default: return z <= w;
    }
}
/* Interpolate::linear_interpolate for f32 components (src/numeric/interpolate.rs:55-57) */
inline float lerp(float t, float x1, float x2) { return (1.0f - t) * x1 + t * x2; }
/* ClippingPlane::intersect (src/geometry/clip.rs:46-63) */
CV intersect(int plane, const CV& v1, const CV& v2, int nk) {
    float x1 = v1.p[0], y1 = v1.p[1], z1 = v1.p[2], w1 = v1.p[3];
    float x2 = v2.p[0], y2 = v2.p[1], z2 = v2.p[2], w2 = v2.p[3];
    float a, b;
    switch (plane) {
    case 0: a = w1 + x1; b = w2 + x2; break;
    case 1: a = w1 - x1; b = w2 - x2; break;
    case 2: a = w1 + y1; b = w2 + y2; break;
    case 3: a = w1 - y1; b = w2 - y2; break;
    case 4: a = z1; b = z2; break;
    default: a = w1 - z1; b = w2 - z2; break;
    }
    float t = a / (a - b);
    CV o;
    for (int i = 0; i < 4; ++i) o.p[i] = lerp(t, v1.p[i], v2.p[i]);
    for (int i = 0; i < nk; ++i) o.k[i] = lerp(t, v1.k[i], v2.k[i]);
    return o;
}

/* clip_primitives, triangle arm (src/pipeline/stages/geometry.rs:264-299).
 * Appends the emitted vertices (3 per triangle) to out. */
void clip_triangle(const CV& a, const CV& b, const CV& c, int nk, std::vector<CV>& out) {
    CV poly[36];
    int n = 0;
    const CV* pairs[3][2] = {{&a, &b}, {&b, &c}, {&c, &a}};
    for (int e = 0; e < 3; ++e) {
        const CV& s = *pairs[e][0];
        const CV& p = *pairs[e][1];
        for (int plane = 0; plane < 6; ++plane) {
            bool s_in = has_inside(plane, s);
            bool p_in = has_inside(plane, p);
            if (s_in != p_in) poly[n++] = intersect(plane, s, p, nk);
            if (p_in) poly[n++] = p;
        }
    }
    if (n == 3) {
        out.push_back(poly[0]); out.push_back(poly[1]); out.push_back(poly[2]);
    } else if (n > 3) {
        const CV last = poly[n - 1];
        for (int i = 0; i < n - 2; ++i) {
            out.push_back(last); out.push_back(poly[i]); out.push_back(poly[i + 1]);
        }
    }
}

/* clip_primitives, line arm (geometry.rs:300-328) */
void clip_line(const CV& s0, const CV& e0, int nk, std::vector<CV>& out) {
    CV start = s0, end = e0;
    int intersections = 0;
    for (int plane = 0; plane < 6; ++plane) {
        bool s_in = has_inside(plane, start);
        bool p_in = has_inside(plane, end);
        if (s_in != p_in) {
            CV inter = intersect(plane, start, end, nk);
            if (s_in) end = inter;
            else if (p_in) start = inter;
            intersections += 1;
        } else if (!s_in) {
            return;
        }
        if (intersections > 2) break;
    }
    out.push_back(start); out.push_back(end);
}

/* clip_primitives, point arm (geometry.rs:329-333) */
void clip_point(const CV& p, std::vector<CV>& out) {
    for (int plane = 0; plane < 6; ++plane)
        if (!has_inside(plane, p)) return;
    out.push_back(p);
}

/* Normal-visualisation geometry shaders (full_example/src/shaders.rs:35-89):
 * triangles emit lines, other primitives are re-emitted. */
void gs_normals(int which, const CV* v, int prim_n, const sr_uniforms* U, int nk,
                std::vector<CV>& lines, std::vector<CV>& same) {
    const float NORMAL_LENGTH = 0.05f;
    if (prim_n != 3) {
        for (int i = 0; i < prim_n; ++i) same.push_back(v[i]);
        return;
    }
    if (which == GS_VERTEX_NORMALS) {
        for (int i = 0; i < 3; ++i) {
            sr_v4 pos = v4(v[i].k), nrm = v4(v[i].k + 4);
            sr_v4 st = sr_m4_mul_v4(U->pv, pos);
            sr_v4 en = sr_m4_mul_v4(U->pv, sr_add4(pos, sr_scale4(nrm, NORMAL_LENGTH)));
            CV a = v[i], b = v[i];
            a.p[0] = st.x; a.p[1] = st.y; a.p[2] = st.z; a.p[3] = st.w;
            b.p[0] = en.x; b.p[1] = en.y; b.p[2] = en.z; b.p[3] = en.w;
            lines.push_back(a); lines.push_back(b);
        }
    } else {
        const float ONE_THIRD = 1.0f / 3.0f;
        CV center;
        std::memset(&center, 0, sizeof(center));
        for (int i = 0; i < nk; ++i)
            center.k[i] = (v[0].k[i] * ONE_THIRD + v[1].k[i] * ONE_THIRD) + v[2].k[i] * ONE_THIRD;
        sr_v4 pos = v4(center.k), nrm = v4(center.k + 4);
        sr_v4 st = sr_m4_mul_v4(U->pv, pos);
        sr_v4 en = sr_m4_mul_v4(U->pv, sr_add4(pos, sr_scale4(sr_normalize4(nrm), NORMAL_LENGTH)));
        CV a = center, b = center;
        a.p[0] = st.x; a.p[1] = st.y; a.p[2] = st.z; a.p[3] = st.w;
        b.p[0] = en.x; b.p[1] = en.y; b.p[2] = en.z; b.p[3] = en.w;
        lines.push_back(a); lines.push_back(b);
    }
}

/* ----------------------------------------------------------- stencil */
/* StencilTest::test(value, mask) (src/stencil.rs:114-129) */
bool stencil_test(uint32_t test, uint8_t value, uint8_t mask) {
    switch (test) {
    case 0: return true;
    case 1: return false;
    case 2: return mask < value;
    case 3: return mask > value;
    case 4: return mask <= value;
    case 5: return mask >= value;
    case 6: return mask == value;
    default: return mask != value;
    }
}
/* StencilOp::op(value, mask) (src/stencil.rs:149-164) for u8 */
uint8_t stencil_op(uint32_t op, uint32_t wrap, uint8_t value, uint8_t mask) {
    switch (op) {
    case 0: return value;
    case 1: return (uint8_t)~value;
    case 2: return 0;
    case 3: return mask;
    case 4: return wrap ? (uint8_t)(value + 1) : (uint8_t)(value == 255 ? 255 : value + 1);
    default: return wrap ? (uint8_t)(value - 1) : (uint8_t)(value == 0 ? 0 : value - 1);
    }
}

/* ----------------------------------------------------------- raster */
struct Tile {
    uint32_t x0, y0, x1, y1;  /* inclusive corners */
};

/* Tile generation (src/pipeline/stages/fragment.rs:188-216) */
std::vector<Tile> make_tiles(uint32_t W, uint32_t H, uint32_t tw, uint32_t th) {
    std::vector<Tile> tiles;
    uint32_t xmax = W - 1, ymax = H - 1;
    uint32_t y = 0;
    while (y < ymax) {
        uint32_t x = 0;
        uint32_t ny = std::min(y + th, ymax);
        while (x < xmax) {
            uint32_t nx = std::min(x + tw, xmax);
            tiles.push_back(Tile{x, y, nx, ny});
            x = nx;
        }
        y = ny;
    }
    return tiles;
}

/* the pixel's events are counted once, in the tile that owns it under
 * half-open ownership (the last column / row belong to the last tile) */
inline bool owner(const Ctx& c, const Tile& t, uint32_t px, uint32_t py) {
    return (px < t.x1 || t.x1 == c.W - 1) && (py < t.y1 || t.y1 == c.H - 1);
}

/* Depth test, shading, blend and writes shared by the three rasterisers:
 * triangle.rs:117-147, line.rs:79-106, point.rs:300-323.  `alpha_mul` < 0
 * means no mul_alpha (triangles, points). */
void shade_and_write(Ctx& c, size_t idx, const CV& sv, double alpha_mul) {
    float z = sv.p[2];
    if (!(z < 0.0f)) return;
    or_fb* fb = c.fb;
    if (fb->depth) {
        float dt = fb->depth[idx];
        if (!(z >= dt)) return;
    }
    sr_v4 col = run_fs(c, sv);
    if (fb->color_format == 1) {
        float* px = (float*)fb->color + idx * 4;
        if (alpha_mul >= 0.0) col.w = col.w * (float)alpha_mul;  /* AlphaMultiply for f32 */
        sr_v4 dst = sr_make_v4(px[0], px[1], px[2], px[3]);
        sr_v4 out = c.blend == BLEND_OVER ? sr_blend_over_f32(col, dst) : col;
        px[0] = out.x; px[1] = out.y; px[2] = out.z; px[3] = out.w;
    } else if (fb->color_format == 2) {
        uint32_t* px = (uint32_t*)fb->color + idx;
        uint32_t src = sr_to_rgba8(col);
        if (alpha_mul >= 0.0) {
            /* AlphaMultiply for u8 (src/color/helper.rs:31-40) with the alpha
             * scalar converted by ColorAlpha::from_scalar (NumCast f64 -> u8) */
            double am = alpha_mul;
            uint8_t a8 = am >= 0.0 && am < 256.0 ? (uint8_t)am : 0;
            uint8_t ch = (uint8_t)(src >> 24);
            uint8_t na = sr_f32_to_u8((float)ch * ((float)a8 / 255.0f));
            src = (src & 0x00ffffffu) | ((uint32_t)na << 24);
        }
        *px = c.blend == BLEND_OVER ? sr_blend_over_rgba8(src, *px) : src;
    }
    if (fb->depth) fb->depth[idx] = z;
}

/* rasterize_triangle (src/pipeline/stages/rasterization/triangle.rs:23-156) */
void rasterize_triangle(Ctx& c, const Tile& tile, const CV& a, const CV& b, const CV& cc) {
    const or_draw* d = c.d;
    float x1 = a.p[0], y1 = a.p[1];
    float x2 = b.p[0], y2 = b.p[1];
    float x3 = cc.p[0], y3 = cc.p[1];
    if (d->cull != 0) {
        /* Shoelace, left to right (triangle.rs:53-61) */
        float ar = x1 * y2 + x2 * y3 + x3 * y1 - x2 * y1 - x3 * y2 - x1 * y3;
        bool neg = std::isnan(ar) ? false : std::signbit(ar);
        uint32_t winding = neg ? 1u : 2u;  /* Clockwise : CounterClockwise */
        if (d->cull == winding) return;
    }
    float det = (y2 - y3) * (x1 - x3) + (x3 - x2) * (y1 - y3);
    float mnx = sr_min(sr_min(x1, x2), x3), mny = sr_min(sr_min(y1, y2), y3);
    float mxx = sr_max(sr_max(x1, x2), x3), mxy = sr_max(sr_max(y1, y2), y3);
    if (std::isnan(mnx) || std::isnan(mny)) {
        /* clamp_as_int's cast(value).unwrap() panics on NaN (triangle.rs:70) */
        c.nan_bbox.fetch_add(1, std::memory_order_relaxed);
        return;
    }
    auto clamp_as_int = [](float v, uint32_t lo, uint32_t hi) -> uint32_t {
        if (v < (float)lo) return lo;
        if (v > (float)hi) return hi;
        return (uint32_t)v;
    };
    uint32_t minx = clamp_as_int(mnx, tile.x0, tile.x1);
    uint32_t miny = clamp_as_int(mny, tile.y0, tile.y1);
    uint32_t maxx = clamp_as_int(mxx, tile.x0, tile.x1);
    uint32_t maxy = clamp_as_int(mxy, tile.y0, tile.y1);
    or_fb* fb = c.fb;
    for (uint32_t py = miny; py <= maxy; ++py) {
        for (uint32_t px = minx; px <= maxx; ++px) {
            size_t idx = (size_t)px + (size_t)py * c.W;
            uint8_t s = c.has_stencil ? fb->stencil[idx] : 0;
            if (!stencil_test(d->stencil_test, s, c.sref)) continue;
            if (c.has_stencil) fb->stencil[idx] = stencil_op(d->stencil_op, d->stencil_wrap, s, c.sref);
            float x = (float)px + 0.5f;
            float y = (float)py + 0.5f;
            float u = ((y2 - y3) * (x - x3) + (x3 - x2) * (y - y3)) / det;
            float v = ((y3 - y1) * (x - x3) + (x1 - x3) * (y - y3)) / det;
            float w = 1.0f - u - v;
            if (!(u < 0.0f || v < 0.0f || w < 0.0f)) {
                CV sv;
                for (int i = 0; i < 4; ++i) sv.p[i] = (a.p[i] * u + b.p[i] * v) + cc.p[i] * w;
                if (sv.p[2] < 0.0f && owner(c, tile, px, py))
                    c.fragments.fetch_add(1, std::memory_order_relaxed);
                if (sv.p[2] < 0.0f) {
                    for (int i = 0; i < c.nk; ++i) sv.k[i] = (a.k[i] * u + b.k[i] * v) + cc.k[i] * w;
                    shade_and_write(c, idx, sv, -1.0);
                }
            }
        }
    }
}

/* hypot: (float)sqrt((double)x*x + (double)y*y) (f32::hypot, unpinned libm) */
inline float hypotf_(float x, float y) {
    double dx = x, dy = y;
    return (float)std::sqrt(dx * dx + dy * dy);
}

/* liang_barsky_iterative (src/geometry/line.rs:6-54) */
bool liang_barsky(float x1, float y1, float x2, float y2, float xmin, float ymin, float xmax,
                  float ymax, float* o) {
    float t0 = 0.0f, t1 = 1.0f;
    float dx = x2 - x1, dy = y2 - y1;
    for (int edge = 0; edge < 4; ++edge) {
        float p, q;
        switch (edge) {
        case 0: p = -dx; q = x1 - xmin; break;
        case 1: p = dx; q = xmax - x1; break;
        case 2: p = -dy; q = y1 - ymin; break;
        default: p = dy; q = ymax - y1; break;
        }
        if (p == 0.0f && q < 0.0f) return false;
        float r = q / p;
        if (p < 0.0f) {
            if (r > t1) return false;
            else if (r > t0) t0 = r;
        } else if (p > 0.0f) {
            if (r < t0) return false;
            else if (r < t1) t1 = r;
        }
    }
    o[0] = x1 + t0 * dx; o[1] = y1 + t0 * dy;
    o[2] = x1 + t1 * dx; o[3] = y1 + t1 * dy;
    return true;
}

/* rasterize_line's per-pixel closure (rasterization/line.rs:54-109); pixels
 * outside the framebuffer are skipped (the reference indexes unchecked). */
void line_fragment(Ctx& c, const Tile& tile, const CV& st, const CV& en, float cx1, float cy1,
                   float dlen, int64_t x, int64_t y, double alpha) {
    if (!(x >= 0 && y >= 0)) return;
    if ((uint64_t)x >= c.W || (uint64_t)y >= c.H) return;
    or_fb* fb = c.fb;
    size_t idx = (size_t)x + (size_t)y * c.W;
    uint8_t s = c.has_stencil ? fb->stencil[idx] : 0;
    if (!stencil_test(c.d->stencil_test, s, c.sref)) return;
    if (c.has_stencil) fb->stencil[idx] = stencil_op(c.d->stencil_op, c.d->stencil_wrap, s, c.sref);
    float xf = (float)x + 0.5f, yf = (float)y + 0.5f;
    float t = hypotf_(cx1 - xf, cy1 - yf) / dlen;
    CV sv;
    for (int i = 0; i < 4; ++i) sv.p[i] = lerp(t, st.p[i], en.p[i]);
    if (sv.p[2] < 0.0f && owner(c, tile, (uint32_t)x, (uint32_t)y))
        c.fragments.fetch_add(1, std::memory_order_relaxed);
    for (int i = 0; i < c.nk; ++i) sv.k[i] = lerp(t, st.k[i], en.k[i]);
    shade_and_write(c, idx, sv, alpha);
}

/* f32 -> i64 NumCast (truncation; out-of-range panics in the reference) */
inline int64_t f2i64(float v) { return (int64_t)v; }
inline int64_t d2i64(double v) { return std::isnan(v) ? 0 : (int64_t)v; }

/* rasterize_line (rasterization/line.rs:22-119) with Bresenham (:125-151)
 * or Xiaolin Wu (:159-239). */
void rasterize_line(Ctx& c, const Tile& tile, const CV& st, const CV& en) {
    float o[4];
    if (!liang_barsky(st.p[0], st.p[1], en.p[0], en.p[1], (float)tile.x0, (float)tile.y0,
                      (float)tile.x1, (float)tile.y1, o))
        return;
    float x1 = o[0], y1 = o[1], x2 = o[2], y2 = o[3];
    /* a NaN clipped end point (a NaN or infinite vertex): cast(x1).unwrap()
     * to i64 panics for Bresenham (line.rs:111-116), and Xiaolin Wu's
     * `as i64` of NaN (line.rs:163) was undefined when the reference was
     * written; the line is skipped and the draw reports status 7 */
    if (std::isnan(x1) || std::isnan(y1) || std::isnan(x2) || std::isnan(y2)) {
        c.nan_bbox.fetch_add(1, std::memory_order_relaxed);
        return;
    }
    float dlen = hypotf_(x1 - x2, y1 - y2);
    auto plot = [&](int64_t x, int64_t y, double a) { line_fragment(c, tile, st, en, x1, y1, dlen, x, y, a); };
    if (c.d->aa_lines) {
        double X0 = x1, Y0 = y1, X1 = x2, Y1 = y2;
        auto plotf = [&](double x, double y, double op) { plot(d2i64(x), d2i64(y), op); };
        bool steep = std::fabs(Y1 - Y0) > std::fabs(X1 - X0);
        if (steep) { std::swap(X0, Y0); std::swap(X1, Y1); }
        if (X0 > X1) { std::swap(X0, X1); std::swap(Y0, Y1); }
        double dx = X1 - X0, dy = Y1 - Y0;
        double gradient = dx < 0.0001 ? 1.0 : dy / dx;
        auto fract = [](double v) { return v - std::trunc(v); };
        double xend = std::round(X0);
        double yend = Y0 + gradient * (xend - X0);
        double xgap = 1.0 - fract(X0 + 0.5);
        double xpxl1 = xend, ypxl1 = std::trunc(yend);
        if (steep) {
            plotf(ypxl1, xpxl1, (1.0 - fract(yend)) * xgap);
            plotf(ypxl1 + 1.0, xpxl1, fract(yend) * xgap);
        } else {
            plotf(xpxl1, ypxl1, (1.0 - fract(yend)) * xgap);
            plotf(xpxl1, ypxl1 + 1.0, fract(yend) * xgap);
        }
        double intery = yend + gradient;
        xend = std::round(X1);
        yend = Y1 + gradient * (xend - X1);
        xgap = fract(X1 + 0.5);
        double xpxl2 = xend, ypxl2 = std::trunc(yend);
        if (steep) {
            plotf(ypxl2, xpxl2, (1.0 - fract(yend)) * xgap);
            plotf(ypxl2 + 1.0, xpxl2, fract(yend) * xgap);
        } else {
            plotf(xpxl2, ypxl2, (1.0 - fract(yend)) * xgap);
            plotf(xpxl2, ypxl2 + 1.0, fract(yend) * xgap);
        }
        double x = xpxl1 + 1.0;
        while (x <= (xpxl2 - 1.0)) {
            double y = std::trunc(intery);
            if (steep) {
                plotf(y, x, 1.0 - fract(intery));
                plotf(y + 1.0, x, fract(intery));
            } else {
                plotf(x, y, 1.0 - fract(intery));
                plotf(x, y + 1.0, fract(intery));
            }
            intery += gradient;
            x += 1.0;
        }
    } else {
        int64_t X0 = f2i64(x1), Y0 = f2i64(y1), X1 = f2i64(x2), Y1 = f2i64(y2);
        int64_t dx = X1 > X0 ? X1 - X0 : X0 - X1;
        int64_t dy = -(Y1 > Y0 ? Y1 - Y0 : Y0 - Y1);
        int64_t sx = X0 < X1 ? 1 : -1;
        int64_t sy = Y0 < Y1 ? 1 : -1;
        int64_t err = dx + dy;
        for (;;) {
            plot(X0, Y0, 1.0);
            if (X0 == X1 && Y0 == Y1) break;
            int64_t e2 = 2 * err;
            if (e2 >= dy) { err += dy; X0 += sx; }
            if (e2 <= dx) { err += dx; Y0 += sy; }
        }
    }
}

/* rasterize_point (rasterization/point.rs:21-87) */
void rasterize_point(Ctx& c, const Tile& tile, const CV& p) {
    float x = p.p[0], y = p.p[1];
    if (!((float)tile.x0 <= x && x < (float)tile.x1 && (float)tile.y0 <= y && y < (float)tile.y1)) return;
    uint32_t px = (uint32_t)x, py = (uint32_t)y;
    or_fb* fb = c.fb;
    size_t idx = (size_t)px + (size_t)py * c.W;
    uint8_t s = c.has_stencil ? fb->stencil[idx] : 0;
    if (!stencil_test(c.d->stencil_test, s, c.sref)) return;
    if (c.has_stencil) fb->stencil[idx] = stencil_op(c.d->stencil_op, c.d->stencil_wrap, s, c.sref);
    if (p.p[2] < 0.0f && owner(c, tile, px, py)) c.fragments.fetch_add(1, std::memory_order_relaxed);
    shade_and_write(c, idx, p, -1.0);
}

}  // namespace

extern "C" {

void or_derive_uniforms(sr_uniforms* u) { sr_uniforms_derive(u); }

void or_clear(or_fb* fb, const void* color) {
    size_t n = (size_t)fb->width * fb->height;
    for (size_t i = 0; i < n; ++i) {
        if (fb->color_format == 1) std::memcpy((float*)fb->color + 4 * i, color, 16);
        else if (fb->color_format == 2) std::memcpy((uint32_t*)fb->color + i, color, 4);
        if (fb->depth) fb->depth[i] = -3.40282347e+38f;  /* f32::MIN (depth.rs:31) */
        if (fb->stencil) fb->stencil[i] = 0;
    }
}

void or_tiles(uint32_t width, uint32_t height, uint32_t tw, uint32_t th, uint32_t* out, uint32_t cap,
              uint32_t* n_out) {
    std::vector<Tile> t = make_tiles(width, height, tw, th);
    *n_out = (uint32_t)t.size();
    for (uint32_t i = 0; i < t.size() && i < cap; ++i) {
        out[4 * i] = t[i].x0; out[4 * i + 1] = t[i].y0; out[4 * i + 2] = t[i].x1; out[4 * i + 3] = t[i].y1;
    }
}

void or_normalize(const float clip[4], const float viewport[6], float out[4]) {
    normalize_pos(clip, viewport, out);
}

uint32_t or_clip_triangle(const float* a, const float* b, const float* c, uint32_t nk, float* out,
                          uint32_t cap) {
    CV va, vb, vc;
    std::memset(&va, 0, sizeof va); std::memset(&vb, 0, sizeof vb); std::memset(&vc, 0, sizeof vc);
    std::memcpy(va.p, a, 16); std::memcpy(vb.p, b, 16); std::memcpy(vc.p, c, 16);
    std::memcpy(va.k, a + 4, nk * 4); std::memcpy(vb.k, b + 4, nk * 4); std::memcpy(vc.k, c + 4, nk * 4);
    std::vector<CV> o;
    clip_triangle(va, vb, vc, (int)nk, o);
    uint32_t stride = 4 + nk;
    for (uint32_t i = 0; i < o.size() && i < cap; ++i) {
        std::memcpy(out + i * stride, o[i].p, 16);
        std::memcpy(out + i * stride + 4, o[i].k, nk * 4);
    }
    return (uint32_t)o.size();
}

float or_powf(float x, float y) { return sr_powf(x, y); }
float or_u8_unit(uint32_t c) { return sr_u8_unit(c); }

/* Coordinate::into_index / from_index (src/geometry/coordinate.rs:44-61) */
uint64_t or_coordinate_into_index(uint32_t x, uint32_t y, uint32_t width) {
    return (uint64_t)x + (uint64_t)y * width;
}
void or_coordinate_from_index(uint64_t index, uint32_t width, uint32_t* x, uint32_t* y) {
    uint64_t xx = index % width;
    *x = (uint32_t)xx;
    *y = (uint32_t)((index - xx) / width);
}

int or_render_impl(const or_draw* d, or_fb* fb, int n_threads, uint32_t tile_begin, uint32_t tile_end,
                   uint32_t tile_step, or_stats* stats, float* tris_out, uint64_t tris_cap, uint64_t* n_tris_out);

int or_render(const or_draw* d, or_fb* fb, int n_threads, uint32_t tile_begin, uint32_t tile_end,
              or_stats* stats) {
    return or_render_impl(d, fb, n_threads, tile_begin, tile_end, 1, stats, nullptr, 0, nullptr);
}

int or_render_strided(const or_draw* d, or_fb* fb, int n_threads, uint32_t tile_first, uint32_t tile_step,
                      uint32_t n, or_stats* stats) {
    if (tile_step == 0) return 1;
    const uint64_t end = (uint64_t)tile_first + (uint64_t)tile_step * n;
    return or_render_impl(d, fb, n_threads, tile_first, (uint32_t)std::min<uint64_t>(end, 0xffffffffu), tile_step,
                          stats, nullptr, 0, nullptr);
}

int or_raster_tris(const or_draw* d, uint32_t width, uint32_t height, float* out, uint64_t cap, uint64_t* n) {
    or_fb fb;
    std::memset(&fb, 0, sizeof(fb));
    fb.width = width;
    fb.height = height;
    return or_render_impl(d, &fb, 1, 0, 0, 1, nullptr, out, cap, n);
}

int or_render_impl(const or_draw* d, or_fb* fb, int n_threads, uint32_t tile_begin, uint32_t tile_end,
                   uint32_t tile_step, or_stats* stats, float* tris_out, uint64_t tris_cap, uint64_t* n_tris_out) {
    Ctx c;
    c.d = d;
    c.U = d->uniforms;
    c.fb = fb;
    c.vs = vs_id(d->vs);
    c.fs = fs_id(d->fs);
    c.blend = blend_id(d->blend);
    c.gs = d->gs_mode == 2 ? gs_id(d->gs) : GS_CLIP;
    if (c.vs < 0 || c.fs < 0 || c.blend < 0 || c.gs < 0) return 8;
    if (fb->width == 0 || fb->height == 0) return 1;      /* mod.rs:129-130 */
    if (d->tile_w == 0 || d->tile_h == 0) return 1;
    if (d->n_planes < (uint32_t)vs_planes(c.vs)) return 1;
    uint32_t pn = d->prim;
    if (pn != 1 && pn != 2 && pn != 3) return 1;
    if (d->n_indices % pn != 0) return 1;                 /* mod.rs:148 */
    for (uint64_t i = 0; i < d->n_indices; ++i)
        if (d->indices[i] >= d->n_verts) return 1;
    if (c.fs == FS_TEXTURED_BLINN_PHONG && (!d->texture || d->tex_w == 0 || d->tex_h == 0)) return 1;
    c.nk = vs_nk(c.vs);
    c.W = fb->width;
    c.H = fb->height;
    c.has_stencil = fb->stencil != nullptr;
    c.sref = c.has_stencil ? (uint8_t)d->stencil_ref : 0;
    /* n_threads < 0: |n_threads| workers in the deterministic mode, whose
     * result equals the 1-thread order (the geometry stage's outputs are
     * concatenated in input order, and the fragment stage runs the tiles in
     * phases: tile (r, c) in phase c + 2 r (c + K r for Xiaolin Wu lines on
     * tiles narrower than 3 pixels, which plot one pixel past their tile),
     * so tiles sharing a pixel fall in distinct phases taken in row-major
     * order, and the tiles of one phase, which share none, run concurrently). */
    const bool phased = n_threads < 0;
    int nt = phased ? -n_threads : (n_threads < 1 ? 1 : n_threads);
    const size_t vfetch = 64 * (size_t)(vs_planes(c.vs) * 4);

    using clk = std::chrono::steady_clock;
    const clk::time_point t_start = clk::now();

    /* vertex stage (vertex.rs:87-160) */
    std::vector<CV> verts(d->n_verts);
    if (d->gs_mode == 0) {
        mapper(d->n_verts, vfetch, nt, [&](size_t i) { verts[i] = normalize(run_vs(c, (uint32_t)i), d->viewport, c.nk); });
    } else {
        mapper(d->n_verts, vfetch, nt, [&](size_t i) { verts[i] = run_vs(c, (uint32_t)i); });
    }

    const clk::time_point t_vertex = clk::now();

    /* geometry stage (geometry.rs:132-258): each worker claims one primitive
     * per fetch_add and appends to its own storage; storages are merged in
     * the order the workers finish (lock order). */
    std::vector<CV> gen_tris, gen_lines, gen_points;
    bool indexed = d->gs_mode == 0;
    auto geometry_of = [&](uint64_t i, std::vector<CV>& tris, std::vector<CV>& lines, std::vector<CV>& points) {
        CV v[3];
        for (uint32_t j = 0; j < pn; ++j) v[j] = verts[d->indices[i + j]];
        if (c.gs == GS_CLIP) {
            if (pn == 3) clip_triangle(v[0], v[1], v[2], c.nk, tris);
            else if (pn == 2) clip_line(v[0], v[1], c.nk, lines);
            else clip_point(v[0], points);
        } else {
            std::vector<CV>& same = pn == 3 ? tris : pn == 2 ? lines : points;
            gs_normals(c.gs, v, (int)pn, c.U, c.nk, lines, same);
        }
    };
    if (!indexed && phased) {
        /* contiguous primitive ranges per worker, concatenated in range order */
        const uint64_t nprim = d->n_indices / pn;
        const uint64_t chunk = (nprim + (uint64_t)nt - 1) / (uint64_t)nt;
        std::vector<std::vector<CV>> tp(nt), lp(nt), pp(nt);
        run_threads_indexed(nt, [&](int k) {
            const uint64_t b = (uint64_t)k * chunk, e = std::min<uint64_t>(b + chunk, nprim);
            for (uint64_t q = b; q < e; ++q) geometry_of(q * pn, tp[k], lp[k], pp[k]);
        });
        for (int k = 0; k < nt; ++k) {
            gen_tris.insert(gen_tris.end(), tp[k].begin(), tp[k].end());
            gen_lines.insert(gen_lines.end(), lp[k].begin(), lp[k].end());
            gen_points.insert(gen_points.end(), pp[k].begin(), pp[k].end());
        }
    } else if (!indexed) {
        std::atomic<uint64_t> next{0};
        std::mutex mu;
        std::vector<std::vector<CV>> tri_parts, line_parts, point_parts;
        run_threads(nt, [&]() {
            std::vector<CV> tris, lines, points;
            for (;;) {
                uint64_t i = next.fetch_add(pn, std::memory_order_relaxed);
                if (i >= d->n_indices) break;
                geometry_of(i, tris, lines, points);
            }
            std::lock_guard<std::mutex> g(mu);
            tri_parts.push_back(std::move(tris));
            line_parts.push_back(std::move(lines));
            point_parts.push_back(std::move(points));
        });
        for (auto& p : tri_parts) gen_tris.insert(gen_tris.end(), p.begin(), p.end());
        for (auto& p : line_parts) gen_lines.insert(gen_lines.end(), p.begin(), p.end());
        for (auto& p : point_parts) gen_points.insert(gen_points.end(), p.begin(), p.end());
    }
    if (!indexed) {
        /* finish (geometry.rs:60-129): normalise every generated vertex */
        auto norm_all = [&](std::vector<CV>& vv) {
            std::vector<CV> out(vv.size());
            mapper(vv.size(), 64 * sizeof(CV), nt, [&](size_t i) { out[i] = normalize(vv[i], d->viewport, c.nk); });
            vv.swap(out);
        };
        norm_all(gen_tris);
        norm_all(gen_lines);
        norm_all(gen_points);
    }

    const clk::time_point t_geometry = clk::now();

    if (tris_out || n_tris_out) {
        /* screen positions of the triangles the fragment stage rasterises */
        uint64_t k = 0;
        auto put = [&](const CV& a, const CV& b, const CV& c2) {
            if (k < tris_cap) {
                const CV* v[3] = {&a, &b, &c2};
                for (int j = 0; j < 3; ++j)
                    for (int q = 0; q < 4; ++q) tris_out[k * 12 + j * 4 + q] = v[j]->p[q];
            }
            ++k;
        };
        if (pn == 3 && indexed)
            for (uint64_t i = 0; i < d->n_indices; i += 3)
                put(verts[d->indices[i]], verts[d->indices[i + 1]], verts[d->indices[i + 2]]);
        for (size_t i = 0; i + 2 < gen_tris.size(); i += 3) put(gen_tris[i], gen_tris[i + 1], gen_tris[i + 2]);
        if (n_tris_out) *n_tris_out = k;
        return 0;
    }

    /* fragment stage (fragment.rs:168-319) */
    std::vector<Tile> tiles = make_tiles(c.W, c.H, d->tile_w, d->tile_h);
    // the tiles to rasterise, in row-major order: all of [tile_begin, tile_end)
    // for or_render, every tile_step-th of them for timing samples
    uint32_t tb = std::min<uint32_t>(tile_begin, (uint32_t)tiles.size());
    uint32_t te = std::min<uint32_t>(tile_end, (uint32_t)tiles.size());
    std::vector<uint32_t> sel;
    for (uint64_t t = tb; t < te; t += std::max(1u, tile_step)) sel.push_back((uint32_t)t);
    auto raster_tile = [&](const Tile& tile) {
        if (pn == 3 && indexed)
            for (uint64_t i = 0; i < d->n_indices; i += 3)
                rasterize_triangle(c, tile, verts[d->indices[i]], verts[d->indices[i + 1]], verts[d->indices[i + 2]]);
        for (size_t i = 0; i + 2 < gen_tris.size(); i += 3)
            rasterize_triangle(c, tile, gen_tris[i], gen_tris[i + 1], gen_tris[i + 2]);
        if (pn == 2 && indexed)
            for (uint64_t i = 0; i < d->n_indices; i += 2)
                rasterize_line(c, tile, verts[d->indices[i]], verts[d->indices[i + 1]]);
        for (size_t i = 0; i + 1 < gen_lines.size(); i += 2)
            rasterize_line(c, tile, gen_lines[i], gen_lines[i + 1]);
        if (pn == 1 && indexed)
            for (uint64_t i = 0; i < d->n_indices; ++i)
                rasterize_point(c, tile, verts[d->indices[i]]);
        for (size_t i = 0; i < gen_points.size(); ++i)
            rasterize_point(c, tile, gen_points[i]);
    };
    if (phased) {
        uint32_t ncols = 0;
        while (ncols < tiles.size() && tiles[ncols].y0 == tiles[0].y0) ++ncols;
        const bool wu_narrow = d->aa_lines && (pn == 2 || !gen_lines.empty()) && d->tile_w < 3;
        const uint32_t K = wu_narrow ? (d->tile_w == 2 ? 3u : 4u) : 2u;
        std::vector<std::vector<uint32_t>> phases;
        for (uint32_t t : sel) {
            const uint32_t ph = (t % ncols) + K * (t / ncols);
            if (ph >= phases.size()) phases.resize(ph + 1);
            phases[ph].push_back(t);
        }
        for (const auto& ph : phases) {
            std::atomic<size_t> next{0};
            run_threads(std::min<int>(nt, (int)ph.size()), [&]() {
                for (;;) {
                    const size_t k = next.fetch_add(1, std::memory_order_relaxed);
                    if (k >= ph.size()) break;
                    raster_tile(tiles[ph[k]]);
                }
            });
        }
    } else {
        std::atomic<size_t> tile_counter{0};
        run_threads(nt, [&]() {
            for (;;) {
                const size_t k = tile_counter.fetch_add(1, std::memory_order_relaxed);
                if (k >= sel.size()) break;
                raster_tile(tiles[sel[k]]);
            }
        });
    }

    const clk::time_point t_raster = clk::now();

    if (stats) {
        stats->vertex_s = std::chrono::duration<double>(t_vertex - t_start).count();
        stats->geometry_s = std::chrono::duration<double>(t_geometry - t_vertex).count();
        stats->raster_s = std::chrono::duration<double>(t_raster - t_geometry).count();
        stats->triangles_generated = gen_tris.size() / 3 + gen_lines.size() / 2 + gen_points.size();
        stats->fragments = c.fragments.load();
        stats->tiles = tiles.size();
        stats->nan_bbox = c.nan_bbox.load();
        stats->status = c.nan_bbox.load() ? 7 : 0;
    }
    return c.nan_bbox.load() ? 7 : 0;
}

}  // extern "C"
