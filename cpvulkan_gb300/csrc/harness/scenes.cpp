// scenes.cpp — seeded generators of the benchmark and test scenes
// (cpv/scene.h). Every byte a scene holds is produced here, once, and given
// unchanged to both the GPU path (through Vulkan) and the CPU oracle.
//
// Workloads (sizes and distributions as the benchmark configurations state):
//   cube        36-vertex unit cube, per-face colour, MVP of the draw_cube
//               sample (fov 45°, lookAt (-5,3,-10) → 0, up (0,-1,0), Vulkan
//               clip matrix) times a rotation about Y by 2π·frame/360;
//               500×500 B8G8R8A8_UNORM + D16, cull back, front CW, LESS.
//   heightfield N×N grid (N = 1024 → 2,093,058 triangles, uint32 indices),
//               value-noise heights, pos3+uv2+normal3, 1024² RGBA8 random
//               texture with a full box-filtered mip chain, trilinear
//               sampler, Lambert light; 1920×1080 RGBA8 + D32, LESS.
//   blend       200,000 screen-space quads, centres uniform, sides
//               log-uniform in [4, 256] px, flat RGBA colour with α in
//               [0.1, 0.9], src-over blending in API order, no depth.
//   batch       4096 indexed draws of displaced icospheres, triangles
//               log-uniform in [12, 200k], 25% instanced 1-64×, MVP+colour
//               in push constants, 70% opaque / 30% blended, 2560×1440.
//   serve       one offscreen request of the serving workload: a textured
//               icosphere into a square RGBA8 + D32 target.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../../include/cpv/vk_subset.h"
#include "../../../include/cpv_harness.h"

namespace {

// splitmix64: deterministic on every host.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * uniform(); }
    double log_uniform(double a, double b) { return std::exp(range(std::log(a), std::log(b))); }
    uint32_t below(uint32_t n) { return static_cast<uint32_t>(next() % n); }
};

struct Mat4 {
    double m[16];  // column-major
    static Mat4 identity() {
        Mat4 r{};
        r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0;
        return r;
    }
    double& at(int col, int row) { return m[col * 4 + row]; }
    double at(int col, int row) const { return m[col * 4 + row]; }
};

Mat4 mul(const Mat4& a, const Mat4& b) {
    Mat4 r{};
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a.at(k, row) * b.at(c, k);
            r.at(c, row) = s;
        }
    return r;
}

struct V3 {
    double x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 norm(V3 a) {
    const double l = std::sqrt(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}

// Right-handed perspective with OpenGL depth range, and lookAt.
Mat4 perspective(double fovy, double aspect, double n, double f) {
    Mat4 r{};
    const double t = std::tan(fovy / 2);
    r.at(0, 0) = 1.0 / (aspect * t);
    r.at(1, 1) = 1.0 / t;
    r.at(2, 2) = -(f + n) / (f - n);
    r.at(2, 3) = -1.0;
    r.at(3, 2) = -(2.0 * f * n) / (f - n);
    return r;
}

Mat4 look_at(V3 eye, V3 centre, V3 up) {
    const V3 f = norm(sub(centre, eye));
    const V3 s = norm(cross(f, up));
    const V3 u = cross(s, f);
    Mat4 r = Mat4::identity();
    r.at(0, 0) = s.x; r.at(1, 0) = s.y; r.at(2, 0) = s.z;
    r.at(0, 1) = u.x; r.at(1, 1) = u.y; r.at(2, 1) = u.z;
    r.at(0, 2) = -f.x; r.at(1, 2) = -f.y; r.at(2, 2) = -f.z;
    r.at(3, 0) = -dot(s, eye);
    r.at(3, 1) = -dot(u, eye);
    r.at(3, 2) = dot(f, eye);
    return r;
}

// Vulkan clip correction used by the LunarG samples: y flipped, z halved.
Mat4 clip_matrix() {
    Mat4 r = Mat4::identity();
    r.at(1, 1) = -1.0;
    r.at(2, 2) = 0.5;
    r.at(3, 2) = 0.5;
    return r;
}

Mat4 translate_scale(V3 t, double s) {
    Mat4 r = Mat4::identity();
    r.at(0, 0) = r.at(1, 1) = r.at(2, 2) = s;
    r.at(3, 0) = t.x;
    r.at(3, 1) = t.y;
    r.at(3, 2) = t.z;
    return r;
}

void store_mat(const Mat4& m, float* out) {
    for (int i = 0; i < 16; i++) out[i] = static_cast<float>(m.m[i]);
}

struct Store {
    cpv_scene scene{};
    uint32_t config = 0;
    std::vector<uint8_t> vertex, index, uniform, texture;
    std::vector<cpv_scene_pipeline> pipelines;
    std::vector<cpv_scene_draw> draws;

    void finish() {
        scene.vertex_data = vertex.empty() ? nullptr : vertex.data();
        scene.vertex_bytes = vertex.size();
        scene.index_data = index.empty() ? nullptr : index.data();
        scene.index_bytes = index.size();
        scene.uniform_data = uniform.empty() ? nullptr : uniform.data();
        scene.uniform_bytes = static_cast<uint32_t>(uniform.size());
        scene.texture_data = texture.empty() ? nullptr : texture.data();
        scene.texture_bytes = texture.size();
        scene.pipelines = pipelines.data();
        scene.num_pipelines = static_cast<uint32_t>(pipelines.size());
        scene.draws = draws.data();
        scene.num_draws = static_cast<uint32_t>(draws.size());
    }
};

template <typename T>
void append(std::vector<uint8_t>& v, const T& x) {
    const uint8_t* p = reinterpret_cast<const uint8_t*>(&x);
    v.insert(v.end(), p, p + sizeof(T));
}
void append_f(std::vector<uint8_t>& v, float x) { append(v, x); }

cpv_scene_pipeline base_pipeline(uint32_t program) {
    cpv_scene_pipeline p{};
    p.program = program;
    p.topology = VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST;
    p.cull_mode = VK_CULL_MODE_NONE;
    p.front_face = VK_FRONT_FACE_COUNTER_CLOCKWISE;
    p.depth_compare = VK_COMPARE_OP_LESS;
    p.stencil_front.compare_op = p.stencil_back.compare_op = VK_COMPARE_OP_ALWAYS;
    p.stencil_front.compare_mask = p.stencil_back.compare_mask = 0xFF;
    p.stencil_front.write_mask = p.stencil_back.write_mask = 0xFF;
    p.src_color = p.src_alpha = VK_BLEND_FACTOR_ONE;
    p.dst_color = p.dst_alpha = VK_BLEND_FACTOR_ZERO;
    for (auto& b : p.extra_blend) {
        b.src_color = b.src_alpha = VK_BLEND_FACTOR_ONE;
        b.dst_color = b.dst_alpha = VK_BLEND_FACTOR_ZERO;
        b.color_write_mask = 0xF;
    }
    p.line_width = 1.0f;
    p.color_write_mask = 0xF;
    return p;
}

void set_src_over(cpv_scene_pipeline& p) {
    p.blend_enable = 1;
    p.src_color = p.src_alpha = VK_BLEND_FACTOR_SRC_ALPHA;
    p.dst_color = p.dst_alpha = VK_BLEND_FACTOR_ONE_MINUS_SRC_ALPHA;
    p.color_op = p.alpha_op = VK_BLEND_OP_ADD;
}

void viewport_full(cpv_scene& s) {
    s.viewport[0] = 0;
    s.viewport[1] = 0;
    s.viewport[2] = static_cast<float>(s.width);
    s.viewport[3] = static_cast<float>(s.height);
    s.viewport[4] = 0;
    s.viewport[5] = 1;
}

// ---------------------------------------------------------------- cube --

Mat4 cube_mvp(uint32_t frame, uint32_t width, uint32_t height) {
    double fov = 45.0 * M_PI / 180.0;
    if (width > height) fov *= static_cast<double>(height) / width;
    const Mat4 proj = perspective(fov, static_cast<double>(width) / height, 0.1, 100.0);
    const Mat4 view = look_at({-5, 3, -10}, {0, 0, 0}, {0, -1, 0});
    const double th = 2.0 * M_PI * frame / 360.0;
    Mat4 model = Mat4::identity();
    model.at(0, 0) = std::cos(th);
    model.at(2, 0) = std::sin(th);
    model.at(0, 2) = -std::sin(th);
    model.at(2, 2) = std::cos(th);
    return mul(clip_matrix(), mul(proj, mul(view, model)));
}

void build_cube(Store& st, uint32_t frame) {
    cpv_scene& s = st.scene;
    s.width = 500;
    s.height = 500;
    s.color_format = VK_FORMAT_B8G8R8A8_UNORM;
    s.depth_format = VK_FORMAT_D16_UNORM;
    for (int i = 0; i < 4; i++) s.clear_color[i] = 0.2f;
    s.clear_depth = 1.0f;
    viewport_full(s);
    // Six faces; each triangle's (v1 - v0) × (v2 - v0) points into the cube,
    // the winding of the sample's cube data, so cull-back + front-CW keeps
    // the faces turned to the camera.
    struct Face { V3 n, a, b; float rgb[3]; };
    const Face faces[6] = {
        {{0, 0, 1}, {1, 0, 0}, {0, 1, 0}, {1, 0, 0}}, {{0, 0, -1}, {0, 1, 0}, {1, 0, 0}, {0, 1, 0}},
        {{-1, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 0, 1}}, {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}},
        {{0, 1, 0}, {0, 0, 1}, {1, 0, 0}, {1, 0, 1}}, {{0, -1, 0}, {1, 0, 0}, {0, 0, 1}, {0, 1, 1}},
    };
    for (const Face& f : faces) {
        auto corner = [&](double sa, double sb) { return V3{f.n.x + sa * f.a.x + sb * f.b.x, f.n.y + sa * f.a.y + sb * f.b.y, f.n.z + sa * f.a.z + sb * f.b.z}; };
        const V3 v[6] = {corner(-1, -1), corner(-1, 1), corner(1, -1), corner(1, -1), corner(-1, 1), corner(1, 1)};
        for (const V3& p : v) {
            append_f(st.vertex, static_cast<float>(p.x));
            append_f(st.vertex, static_cast<float>(p.y));
            append_f(st.vertex, static_cast<float>(p.z));
            append_f(st.vertex, 1.0f);
            append_f(st.vertex, f.rgb[0]);
            append_f(st.vertex, f.rgb[1]);
            append_f(st.vertex, f.rgb[2]);
            append_f(st.vertex, 1.0f);
        }
    }
    st.uniform.resize(64);
    store_mat(cube_mvp(frame, s.width, s.height), reinterpret_cast<float*>(st.uniform.data()));
    cpv_scene_pipeline p = base_pipeline(CPV_PROGRAM_CUBE);
    p.cull_mode = VK_CULL_MODE_BACK_BIT;
    p.front_face = VK_FRONT_FACE_CLOCKWISE;
    p.depth_test = 1;
    p.depth_write = 1;
    p.depth_compare = VK_COMPARE_OP_LESS;
    p.num_bindings = 1;
    p.bindings[0] = {0, 32, VK_VERTEX_INPUT_RATE_VERTEX};
    p.num_attributes = 2;
    p.attributes[0] = {0, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 0};
    p.attributes[1] = {1, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 16};
    st.pipelines.push_back(p);
    cpv_scene_draw d{};
    d.pipeline = 0;
    d.count = 36;
    d.instance_count = 1;
    st.draws.push_back(d);
}

// ---------------------------------------------------------- heightfield --

void make_texture(Store& st, uint32_t side, uint64_t seed) {
    cpv_scene& s = st.scene;
    Rng rng(seed);
    uint32_t levels = 1;
    while ((side >> (levels - 1)) > 1) levels++;
    std::vector<std::vector<uint8_t>> lv(levels);
    lv[0].resize(static_cast<size_t>(side) * side * 4);
    for (auto& b : lv[0]) b = static_cast<uint8_t>(rng.next() & 0xFF);
    uint32_t w = side;
    for (uint32_t l = 1; l < levels; l++) {
        const uint32_t nw = std::max(w / 2, 1u);
        lv[l].resize(static_cast<size_t>(nw) * nw * 4);
        for (uint32_t y = 0; y < nw; y++)
            for (uint32_t x = 0; x < nw; x++)
                for (int c = 0; c < 4; c++) {
                    auto at = [&](uint32_t xx, uint32_t yy) { return lv[l - 1][(static_cast<size_t>(std::min(yy, w - 1)) * w + std::min(xx, w - 1)) * 4 + c]; };
                    const uint32_t sum = at(2 * x, 2 * y) + at(2 * x + 1, 2 * y) + at(2 * x, 2 * y + 1) + at(2 * x + 1, 2 * y + 1);
                    lv[l][(static_cast<size_t>(y) * nw + x) * 4 + c] = static_cast<uint8_t>((sum + 2) / 4);
                }
        w = nw;
    }
    for (auto& l : lv) st.texture.insert(st.texture.end(), l.begin(), l.end());
    s.texture_width = side;
    s.texture_height = side;
    s.texture_levels = levels;
    s.texture_format = VK_FORMAT_R8G8B8A8_UNORM;
    s.sampler.mag_filter = VK_FILTER_LINEAR;
    s.sampler.min_filter = VK_FILTER_LINEAR;
    s.sampler.mipmap_mode = VK_SAMPLER_MIPMAP_MODE_LINEAR;
    s.sampler.address_u = s.sampler.address_v = s.sampler.address_w = VK_SAMPLER_ADDRESS_MODE_REPEAT;
    s.sampler.mip_lod_bias = 0.0f;
    s.sampler.min_lod = 0.0f;
    s.sampler.max_lod = static_cast<float>(levels);
    s.sampler.border_color = VK_BORDER_COLOR_FLOAT_OPAQUE_BLACK;
}

cpv_scene_pipeline texlit_pipeline() {
    cpv_scene_pipeline p = base_pipeline(CPV_PROGRAM_TEXLIT);
    p.depth_test = 1;
    p.depth_write = 1;
    p.num_bindings = 1;
    p.bindings[0] = {0, 32, VK_VERTEX_INPUT_RATE_VERTEX};
    p.num_attributes = 3;
    p.attributes[0] = {0, 0, VK_FORMAT_R32G32B32_SFLOAT, 0};
    p.attributes[1] = {1, 0, VK_FORMAT_R32G32_SFLOAT, 12};
    p.attributes[2] = {2, 0, VK_FORMAT_R32G32B32_SFLOAT, 20};
    return p;
}

void build_heightfield(Store& st, uint64_t seed, uint32_t n, uint32_t width, uint32_t height) {
    cpv_scene& s = st.scene;
    s.width = width;
    s.height = height;
    s.color_format = VK_FORMAT_R8G8B8A8_UNORM;
    s.depth_format = VK_FORMAT_D32_SFLOAT;
    s.clear_color[0] = 0.1f; s.clear_color[1] = 0.1f; s.clear_color[2] = 0.15f; s.clear_color[3] = 1.0f;
    s.clear_depth = 1.0f;
    viewport_full(s);
    // Value noise: 17×17 lattice (16×16 cells) of seeded values, smoothstep.
    Rng rng(seed);
    const int L = 16;
    std::vector<double> lattice((L + 1) * (L + 1));
    for (auto& v : lattice) v = rng.uniform();
    auto height_at = [&](double u, double v) {
        const double x = u * L, y = v * L;
        int ix = std::min(static_cast<int>(x), L - 1), iy = std::min(static_cast<int>(y), L - 1);
        double fx = x - ix, fy = y - iy;
        fx = fx * fx * (3 - 2 * fx);
        fy = fy * fy * (3 - 2 * fy);
        auto g = [&](int a, int b) { return lattice[b * (L + 1) + a]; };
        const double a = g(ix, iy) + (g(ix + 1, iy) - g(ix, iy)) * fx;
        const double b = g(ix, iy + 1) + (g(ix + 1, iy + 1) - g(ix, iy + 1)) * fx;
        return a + (b - a) * fy;
    };
    const double amp = 0.35;
    st.vertex.reserve(static_cast<size_t>(n) * n * 32);
    const double step = 2.0 / (n - 1);
    for (uint32_t j = 0; j < n; j++) {
        for (uint32_t i = 0; i < n; i++) {
            const double u = static_cast<double>(i) / (n - 1), v = static_cast<double>(j) / (n - 1);
            const double h = amp * height_at(u, v);
            const double du = 1.0 / (n - 1);
            const double hx = amp * (height_at(std::min(u + du, 1.0), v) - height_at(std::max(u - du, 0.0), v)) / (2 * step);
            const double hz = amp * (height_at(u, std::min(v + du, 1.0)) - height_at(u, std::max(v - du, 0.0))) / (2 * step);
            const V3 nn = norm({-hx, 1.0, -hz});
            append_f(st.vertex, static_cast<float>(-1.0 + 2.0 * u));
            append_f(st.vertex, static_cast<float>(h));
            append_f(st.vertex, static_cast<float>(-1.0 + 2.0 * v));
            append_f(st.vertex, static_cast<float>(u * 4.0));
            append_f(st.vertex, static_cast<float>(v * 4.0));
            append_f(st.vertex, static_cast<float>(nn.x));
            append_f(st.vertex, static_cast<float>(nn.y));
            append_f(st.vertex, static_cast<float>(nn.z));
        }
    }
    st.index.reserve(static_cast<size_t>(n - 1) * (n - 1) * 6 * 4);
    for (uint32_t j = 0; j + 1 < n; j++)
        for (uint32_t i = 0; i + 1 < n; i++) {
            const uint32_t a = j * n + i, b = a + 1, c = a + n, d = c + 1;
            const uint32_t idx[6] = {a, c, b, b, c, d};
            for (uint32_t x : idx) append(st.index, x);
        }
    s.index_type = VK_INDEX_TYPE_UINT32;
    const Mat4 proj = perspective(60.0 * M_PI / 180.0, static_cast<double>(width) / height, 0.1, 10.0);
    const Mat4 view = look_at({0, 0.9, -1.55}, {0, 0.05, 0.25}, {0, 1, 0});
    st.uniform.resize(80);
    store_mat(mul(clip_matrix(), mul(proj, view)), reinterpret_cast<float*>(st.uniform.data()));
    const V3 light = norm({0.4, 0.8, -0.45});
    float* lp = reinterpret_cast<float*>(st.uniform.data() + 64);
    lp[0] = static_cast<float>(light.x);
    lp[1] = static_cast<float>(light.y);
    lp[2] = static_cast<float>(light.z);
    lp[3] = 0.0f;
    make_texture(st, 1024, seed + 1);
    st.pipelines.push_back(texlit_pipeline());
    cpv_scene_draw d{};
    d.pipeline = 0;
    d.indexed = 1;
    d.count = (n - 1) * (n - 1) * 6;
    d.instance_count = 1;
    st.draws.push_back(d);
}

// ---------------------------------------------------------------- blend --

// smooth = 0: flat colour per quad (FLATQUAD program). smooth = 1: the same
// quads drawn with the CUBE program (identity MVP, w = 1) and a colour per
// corner, so the fragment shader's input is interpolated per pixel.
void build_blend(Store& st, uint64_t seed, uint32_t quads, uint32_t width, uint32_t height, uint32_t smooth) {
    cpv_scene& s = st.scene;
    s.width = width;
    s.height = height;
    s.color_format = VK_FORMAT_R8G8B8A8_UNORM;
    s.depth_format = 0;
    s.clear_color[0] = 0.0f; s.clear_color[1] = 0.0f; s.clear_color[2] = 0.0f; s.clear_color[3] = 1.0f;
    viewport_full(s);
    Rng rng(seed);
    st.vertex.reserve(static_cast<size_t>(quads) * 4 * 24);
    st.index.reserve(static_cast<size_t>(quads) * 6 * 4);
    for (uint32_t q = 0; q < quads; q++) {
        const double cx = rng.range(0, width), cy = rng.range(0, height);
        const double w = rng.log_uniform(4, 256), h = rng.log_uniform(4, 256);
        const float col[4] = {static_cast<float>(rng.uniform()), static_cast<float>(rng.uniform()), static_cast<float>(rng.uniform()),
                              static_cast<float>(rng.range(0.1, 0.9))};
        const double xs[2] = {cx - w / 2, cx + w / 2}, ys[2] = {cy - h / 2, cy + h / 2};
        for (int k = 0; k < 4; k++) {
            const double px = xs[k & 1], py = ys[k >> 1];
            append_f(st.vertex, static_cast<float>(px / width * 2.0 - 1.0));
            append_f(st.vertex, static_cast<float>(py / height * 2.0 - 1.0));
            if (smooth) {
                append_f(st.vertex, 0.0f);
                append_f(st.vertex, 1.0f);
                // each corner's colour: the quad's, channels scaled by [0.5, 1)
                for (int c = 0; c < 3; c++) append_f(st.vertex, col[c] * static_cast<float>(rng.range(0.5, 1.0)));
                append_f(st.vertex, col[3]);
            } else {
                for (float c : col) append_f(st.vertex, c);
            }
        }
        const uint32_t b = q * 4;
        const uint32_t idx[6] = {b, b + 1, b + 2, b + 2, b + 1, b + 3};
        for (uint32_t x : idx) append(st.index, x);
    }
    s.index_type = VK_INDEX_TYPE_UINT32;
    cpv_scene_pipeline p = base_pipeline(smooth ? CPV_PROGRAM_CUBE : CPV_PROGRAM_FLATQUAD);
    set_src_over(p);
    p.num_bindings = 1;
    p.num_attributes = 2;
    if (smooth) {
        p.bindings[0] = {0, 32, VK_VERTEX_INPUT_RATE_VERTEX};
        p.attributes[0] = {0, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 0};
        p.attributes[1] = {1, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 16};
        st.uniform.assign(64, 0);
        float* m = reinterpret_cast<float*>(st.uniform.data());
        m[0] = m[5] = m[10] = m[15] = 1.0f;  // identity MVP
    } else {
        p.bindings[0] = {0, 24, VK_VERTEX_INPUT_RATE_VERTEX};
        p.attributes[0] = {0, 0, VK_FORMAT_R32G32_SFLOAT, 0};
        p.attributes[1] = {1, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 8};
    }
    st.pipelines.push_back(p);
    cpv_scene_draw d{};
    d.pipeline = 0;
    d.indexed = 1;
    d.count = quads * 6;
    d.instance_count = 1;
    st.draws.push_back(d);
}

// ----------------------------------------------------------- icospheres --

// Geodesic icosphere of frequency n (20 n² triangles); vertices are not
// shared across the 20 base faces. Each triangle's (v1 - v0) × (v2 - v0)
// points inward (the cube's winding). Displacement r(dir) = 1 + disp·f(dir)
// with a smooth seeded f, so duplicated edge vertices stay crack-free.
void icosphere(uint32_t n, double disp, const double phase[3], bool with_uv, std::vector<uint8_t>& vb, std::vector<uint8_t>& ib, uint32_t& vcount,
               uint32_t& icount) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    const V3 base[12] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    const int faces[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                              {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                              {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    const uint32_t first_vertex = vcount;
    for (const auto& f : faces) {
        const V3 A = base[f[0]], B = base[f[1]], C = base[f[2]];
        const uint32_t face_base = vcount - first_vertex;
        for (uint32_t i = 0; i <= n; i++) {
            for (uint32_t j = 0; j <= n - i; j++) {
                const double a = static_cast<double>(i) / n, b = static_cast<double>(j) / n, c = 1.0 - a - b;
                V3 p = {c * A.x + a * B.x + b * C.x, c * A.y + a * B.y + b * C.y, c * A.z + a * B.z + b * C.z};
                const V3 d = norm(p);
                const double r = 1.0 + disp * std::sin(3.1 * d.x + phase[0]) * std::sin(2.7 * d.y + phase[1]) * std::sin(3.7 * d.z + phase[2]);
                append_f(vb, static_cast<float>(d.x * r));
                append_f(vb, static_cast<float>(d.y * r));
                append_f(vb, static_cast<float>(d.z * r));
                if (with_uv) {
                    append_f(vb, static_cast<float>(0.5 + std::atan2(d.z, d.x) / (2 * M_PI)));
                    append_f(vb, static_cast<float>(0.5 - std::asin(std::max(-1.0, std::min(1.0, d.y))) / M_PI));
                }
                append_f(vb, static_cast<float>(d.x));
                append_f(vb, static_cast<float>(d.y));
                append_f(vb, static_cast<float>(d.z));
                vcount++;
            }
        }
        auto vid = [&](uint32_t i, uint32_t j) {
            // row i holds n - i + 1 vertices
            uint32_t off = 0;
            for (uint32_t k = 0; k < i; k++) off += n - k + 1;
            return face_base + off + j;
        };
        for (uint32_t i = 0; i < n; i++) {
            for (uint32_t j = 0; j < n - i; j++) {
                // outward-CCW triangles of the face, emitted reversed (inward winding)
                uint32_t tri[3] = {vid(i, j), vid(i + 1, j), vid(i, j + 1)};
                std::swap(tri[1], tri[2]);
                for (uint32_t x : tri) append(ib, x);
                icount += 3;
                if (j + 1 < n - i) {
                    uint32_t tri2[3] = {vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)};
                    std::swap(tri2[1], tri2[2]);
                    for (uint32_t x : tri2) append(ib, x);
                    icount += 3;
                }
            }
        }
    }
}

void build_batch(Store& st, uint64_t seed, uint32_t draws, uint32_t max_tris, uint32_t width, uint32_t height) {
    cpv_scene& s = st.scene;
    s.width = width;
    s.height = height;
    s.color_format = VK_FORMAT_R8G8B8A8_UNORM;
    s.depth_format = VK_FORMAT_D32_SFLOAT;
    s.clear_color[0] = 0.05f; s.clear_color[1] = 0.05f; s.clear_color[2] = 0.08f; s.clear_color[3] = 1.0f;
    s.clear_depth = 1.0f;
    viewport_full(s);
    Rng rng(seed);
    const Mat4 proj = perspective(50.0 * M_PI / 180.0, static_cast<double>(width) / height, 0.5, 100.0);
    const Mat4 vp = mul(clip_matrix(), mul(proj, look_at({0, 0, -14}, {0, 0, 10}, {0, -1, 0})));
    // Instance offsets live after the meshes in the same vertex blob
    // (binding 1, instance rate, 16-byte stride).
    std::vector<float> instances;
    std::vector<uint8_t> vb, ib;
    uint32_t vcount = 0, icount = 0;
    for (uint32_t d = 0; d < draws; d++) {
        const double T = rng.log_uniform(12.0, static_cast<double>(std::max(max_tris, 13u)));
        const uint32_t n = std::max<uint32_t>(1, static_cast<uint32_t>(std::lround(std::sqrt(T / 20.0))));
        const double phase[3] = {rng.range(0, 6.283), rng.range(0, 6.283), rng.range(0, 6.283)};
        const uint32_t v0 = vcount, i0 = icount;
        icosphere(n, 0.15, phase, false, vb, ib, vcount, icount);
        uint32_t inst = 1;
        if (rng.uniform() < 0.25) inst = 1 + rng.below(64);
        const uint32_t first_inst = static_cast<uint32_t>(instances.size() / 4);
        for (uint32_t k = 0; k < inst; k++) {
            const bool moved = inst > 1;
            instances.push_back(moved ? static_cast<float>(rng.range(-2.5, 2.5)) : 0.0f);
            instances.push_back(moved ? static_cast<float>(rng.range(-2.5, 2.5)) : 0.0f);
            instances.push_back(moved ? static_cast<float>(rng.range(-2.5, 2.5)) : 0.0f);
            instances.push_back(0.0f);
        }
        const bool blended = rng.uniform() < 0.3;
        const V3 c = {rng.range(-8, 8), rng.range(-4.5, 4.5), rng.range(0, 20)};
        const double scale = 0.4 + 1.2 * rng.uniform();
        cpv_scene_draw dr{};
        dr.pipeline = blended ? 1 : 0;
        dr.indexed = 1;
        dr.count = icount - i0;
        dr.first = i0;
        dr.vertex_offset = static_cast<int32_t>(v0);
        dr.instance_count = inst;
        dr.first_instance = first_inst;
        dr.push_size = 80;
        float push[20];
        store_mat(mul(vp, translate_scale(c, scale)), push);
        push[16] = static_cast<float>(rng.uniform());
        push[17] = static_cast<float>(rng.uniform());
        push[18] = static_cast<float>(rng.uniform());
        push[19] = blended ? static_cast<float>(rng.range(0.3, 0.7)) : 1.0f;
        std::memcpy(dr.push, push, sizeof(push));
        st.draws.push_back(dr);
    }
    st.vertex = std::move(vb);
    const uint64_t inst_off = (st.vertex.size() + 15) & ~15ull;
    st.vertex.resize(inst_off);
    const uint8_t* ip = reinterpret_cast<const uint8_t*>(instances.data());
    st.vertex.insert(st.vertex.end(), ip, ip + instances.size() * 4);
    for (auto& d : st.draws) d.vertex_offsets[1] = inst_off;
    st.index = std::move(ib);
    s.index_type = VK_INDEX_TYPE_UINT32;
    for (int k = 0; k < 2; k++) {
        cpv_scene_pipeline p = base_pipeline(CPV_PROGRAM_MESHPC);
        p.cull_mode = VK_CULL_MODE_BACK_BIT;
        p.front_face = VK_FRONT_FACE_CLOCKWISE;
        p.depth_test = 1;
        p.depth_write = k == 0 ? 1 : 0;
        if (k == 1) set_src_over(p);
        p.num_bindings = 2;
        p.bindings[0] = {0, 24, VK_VERTEX_INPUT_RATE_VERTEX};
        p.bindings[1] = {1, 16, VK_VERTEX_INPUT_RATE_INSTANCE};
        p.num_attributes = 3;
        p.attributes[0] = {0, 0, VK_FORMAT_R32G32B32_SFLOAT, 0};
        p.attributes[1] = {1, 0, VK_FORMAT_R32G32B32_SFLOAT, 12};
        p.attributes[2] = {2, 1, VK_FORMAT_R32G32B32A32_SFLOAT, 0};
        st.pipelines.push_back(p);
    }
}

void build_serve(Store& st, uint64_t seed, uint32_t side, uint32_t tris, uint32_t client) {
    cpv_scene& s = st.scene;
    s.width = side;
    s.height = side;
    s.color_format = VK_FORMAT_R8G8B8A8_UNORM;
    s.depth_format = VK_FORMAT_D32_SFLOAT;
    s.clear_color[0] = 0.0f; s.clear_color[1] = 0.0f; s.clear_color[2] = 0.0f; s.clear_color[3] = 1.0f;
    s.clear_depth = 1.0f;
    viewport_full(s);
    Rng rng(seed ^ (static_cast<uint64_t>(client) << 32));
    const uint32_t n = std::max<uint32_t>(1, static_cast<uint32_t>(std::lround(std::sqrt(tris / 20.0))));
    const double phase[3] = {rng.range(0, 6.283), rng.range(0, 6.283), rng.range(0, 6.283)};
    uint32_t vcount = 0, icount = 0;
    icosphere(n, 0.15, phase, true, st.vertex, st.index, vcount, icount);
    s.index_type = VK_INDEX_TYPE_UINT32;
    const Mat4 proj = perspective(45.0 * M_PI / 180.0, 1.0, 0.5, 20.0);
    const double ang = rng.range(0, 6.283);
    const Mat4 view = look_at({4.0 * std::sin(ang), 1.5, -4.0 * std::cos(ang)}, {0, 0, 0}, {0, -1, 0});
    st.uniform.resize(80);
    store_mat(mul(clip_matrix(), mul(proj, view)), reinterpret_cast<float*>(st.uniform.data()));
    const V3 light = norm({0.5, 0.7, -0.5});
    float* lp = reinterpret_cast<float*>(st.uniform.data() + 64);
    lp[0] = static_cast<float>(light.x); lp[1] = static_cast<float>(light.y); lp[2] = static_cast<float>(light.z); lp[3] = 0;
    make_texture(st, 512, 1000 + client);
    cpv_scene_pipeline p = texlit_pipeline();
    p.cull_mode = VK_CULL_MODE_BACK_BIT;
    p.front_face = VK_FRONT_FACE_CLOCKWISE;
    st.pipelines.push_back(p);
    cpv_scene_draw d{};
    d.indexed = 1;
    d.count = icount;
    d.instance_count = 1;
    st.draws.push_back(d);
}

// ------------------------------------------------------- program tests --
// Small scenes that exercise one shader program and a fixed-function
// variant. variant bits: 0-1 cull mode, 2 front CW, 3-4 depth format
// (0 none, 1 D16, 2 D32, 3 D32S8), 5 blend, 6-7 depth op (LESS, LEQUAL,
// GREATER, ALWAYS), 8 stencil test, 9 BGRA target, 10-11 topology
// (list, strip, fan; with bit 16: points, lines, line strip), 12 uint16
// indices, 13 depth write off, 16 point/line topologies (line width 1 + 2.5
// × bit 17), 18 logic op (op in 20-23), 19 colour write mask (mask in
// 24-27), 28-29 depth bounds, 30 no colour attachment (a depth-only pass;
// D32 when bits 3-4 pick no depth format).
// Bytes per vertex of the colour attribute in `format` (the normalised
// 8/16-bit and 16-bit float formats the translator converts), 0 otherwise.
uint32_t colour_attribute_bytes(uint32_t format) {
    switch (format) {
    case 9: case 10: return 1;                         // R8
    case 16: case 17: case 70: case 71: case 76: return 2;  // R8G8, R16
    case 23: case 24: return 3;                        // R8G8B8
    case 37: case 38: case 44: case 77: case 78: case 83: return 4;
    case 84: case 85: case 90: return 6;               // R16G16B16
    case 91: case 92: case 97: return 8;               // R16G16B16A16
    default: return 0;
    }
}

// colour_format != 0 (CUBE-family programs): the colour attribute comes
// from a second binding in that format, its bytes seeded at random over the
// whole code range (half floats: any sign, exponents 0-15, so subnormals
// and values up to 2). For the FETCH program the same parameter is the
// value of the fragment shader's specialisation constant (0: none).
// attachment_format != 0: the colour attachment's format (R8, R8G8, R16,
// R16G16 UNORM, R8G8B8A8 SNORM, R16G16 or R32 SFLOAT), cleared to a colour
// with channels outside [0, 1].
void build_program(Store& st, uint64_t seed, uint32_t program, uint32_t variant, uint32_t width, uint32_t height, uint32_t tris,
                   uint32_t colour_format, uint32_t attachment_format, uint64_t extra_formats, uint64_t extra_blend) {
    cpv_scene& s = st.scene;
    s.width = width;
    s.height = height;
    s.color_format = (variant & 0x200) ? VK_FORMAT_B8G8R8A8_UNORM : VK_FORMAT_R8G8B8A8_UNORM;
    if (attachment_format) s.color_format = attachment_format;
    const bool depth_only = (variant & 0x40000000u) != 0;
    if (depth_only) s.color_format = 0;
    const uint32_t dsel = depth_only && ((variant >> 3) & 3) == 0 ? 2u : (variant >> 3) & 3;
    const uint32_t dfmts[4] = {0, VK_FORMAT_D16_UNORM, VK_FORMAT_D32_SFLOAT, VK_FORMAT_D32_SFLOAT_S8_UINT};
    s.depth_format = dfmts[dsel];
    s.clear_color[0] = 0.25f; s.clear_color[1] = 0.5f; s.clear_color[2] = 0.75f; s.clear_color[3] = 1.0f;
    if (attachment_format) { s.clear_color[0] = -0.3f; s.clear_color[1] = 0.6f; s.clear_color[2] = 1.7f; s.clear_color[3] = 0.45f; }
    // The textured and mesh programs view their geometry from afar (NDC
    // depth near 1): their depth is cleared to 1 so a LESS test passes.
    const bool textured = program == CPV_PROGRAM_TEXLIT || program == CPV_PROGRAM_FETCH || program == CPV_PROGRAM_STORAGE ||
                          program == CPV_PROGRAM_SEPARATE;
    const bool far_geometry = textured || program == CPV_PROGRAM_MESHPC;
    s.clear_depth = far_geometry ? 1.0f : 0.75f;
    s.clear_stencil = 3;
    viewport_full(s);
    Rng rng(seed);
    cpv_scene_pipeline p = base_pipeline(program);
    p.cull_mode = variant & 3;
    p.front_face = (variant & 4) ? VK_FRONT_FACE_CLOCKWISE : VK_FRONT_FACE_COUNTER_CLOCKWISE;
    p.depth_test = dsel != 0;
    p.depth_write = (variant & 0x2000) ? 0 : 1;
    const uint32_t ops[4] = {VK_COMPARE_OP_LESS, VK_COMPARE_OP_LESS_OR_EQUAL, VK_COMPARE_OP_GREATER, VK_COMPARE_OP_ALWAYS};
    p.depth_compare = ops[(variant >> 6) & 3];
    if (variant & 0x20) {
        set_src_over(p);
        if (seed & 1) {  // a second blend equation: additive colour, max alpha
            p.src_color = VK_BLEND_FACTOR_ONE;
            p.dst_color = VK_BLEND_FACTOR_ONE_MINUS_DST_COLOR;
            p.alpha_op = VK_BLEND_OP_MAX;
        }
    }
    if ((variant & 0x100) && dsel == 3) {
        p.stencil_test = 1;
        p.stencil_front = {VK_STENCIL_OP_KEEP, VK_STENCIL_OP_INCREMENT_AND_WRAP, VK_STENCIL_OP_REPLACE, VK_COMPARE_OP_GREATER_OR_EQUAL, 0xFF, 0xFF, 4};
        p.stencil_back = {VK_STENCIL_OP_INVERT, VK_STENCIL_OP_DECREMENT_AND_CLAMP, VK_STENCIL_OP_ZERO, VK_COMPARE_OP_NOT_EQUAL, 0x0F, 0xF0, 2};
    }
    const uint32_t topo_sel = (variant >> 10) & 3;
    p.topology = topo_sel == 1 ? VK_PRIMITIVE_TOPOLOGY_TRIANGLE_STRIP : (topo_sel == 2 ? VK_PRIMITIVE_TOPOLOGY_TRIANGLE_FAN : VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST);
    if (variant & 0x10000) {
        p.topology = topo_sel == 1 ? VK_PRIMITIVE_TOPOLOGY_LINE_LIST : (topo_sel == 2 ? VK_PRIMITIVE_TOPOLOGY_LINE_STRIP : VK_PRIMITIVE_TOPOLOGY_POINT_LIST);
        p.line_width = (variant & 0x20000) ? 3.5f : 1.0f;
    }
    if (variant & 0x40000) {  // logic op (bits 20-23) instead of blending
        p.logic_op_enable = 1;
        p.logic_op = (variant >> 20) & 0xF;
    }
    if (variant & 0x80000) p.color_write_mask = (variant >> 24) & 0xF;  // partial colour write mask (bits 24-27)
    // Colour attachments after the first: byte k of extra_formats is the
    // VkFormat of attachment k + 1 (0: an unused reference), byte k of
    // extra_blend its blend state: bit 0 src-over, bit 1 additive colour
    // with a MAX alpha, bits 4-7 a write mask (0: every channel).
    for (uint32_t k = 0; k < CPV_SCENE_MAX_EXTRA_COLOR; k++) {
        const uint32_t f = static_cast<uint32_t>((extra_formats >> (8 * k)) & 0xFFu);
        if (f) s.extra_color_count = k + 1;
        s.extra_color_formats[k] = f;
        const uint32_t b = static_cast<uint32_t>((extra_blend >> (8 * k)) & 0xFFu);
        cpv_scene_attachment_blend& eb = p.extra_blend[k];
        if (b & 1u) {
            eb.blend_enable = 1;
            eb.src_color = VK_BLEND_FACTOR_SRC_ALPHA;
            eb.dst_color = VK_BLEND_FACTOR_ONE_MINUS_SRC_ALPHA;
            eb.src_alpha = VK_BLEND_FACTOR_ONE;
            eb.dst_alpha = VK_BLEND_FACTOR_ONE_MINUS_SRC_ALPHA;
        } else if (b & 2u) {
            eb.blend_enable = 1;
            eb.src_color = eb.dst_color = VK_BLEND_FACTOR_ONE;
            eb.src_alpha = eb.dst_alpha = VK_BLEND_FACTOR_ONE;
            eb.alpha_op = VK_BLEND_OP_MAX;
        }
        if (b >> 4) eb.color_write_mask = b >> 4;
    }
    if (const uint32_t bounds = (variant >> 28) & 3u) {  // depth bounds test (bits 28-29) against the stored depth (cleared to 0.75 or 1)
        // 1: the whole range; 2: stored depth from 0.3 up; 3: above the clear depth, so nothing passes
        static const float range[4][2] = {{0.0f, 1.0f}, {0.0f, 1.0f}, {0.3f, 1.0f}, {0.8f, 1.0f}};
        p.depth_bounds_test = 1;
        p.min_depth_bounds = range[bounds][0];
        p.max_depth_bounds = range[bounds][1];
    }
    const bool u16 = (variant & 0x1000) != 0;

    uint32_t vcount = 0;
    uint64_t colour_offset = 0;
    if (program == CPV_PROGRAM_CUBE || program == CPV_PROGRAM_DISCARD || program == CPV_PROGRAM_NOPERSP || program == CPV_PROGRAM_POINTS ||
        program == CPV_PROGRAM_MRT || program == CPV_PROGRAM_MRTI || program == CPV_PROGRAM_MATHX ||
        program == CPV_PROGRAM_CALLS || program == CPV_PROGRAM_SSBO) {
        if (program == CPV_PROGRAM_SSBO) s.uniform_as_storage = 1;
        // Clip-space vertices with w in [0.5, 2] (positive, as the reference
        // requires), a shared-edge pair, and a zero-area triangle.
        st.uniform.resize(64);
        store_mat(Mat4::identity(), reinterpret_cast<float*>(st.uniform.data()));
        vcount = tris * 3;
        for (uint32_t v = 0; v < vcount; v++) {
            const double w = rng.range(0.5, 2.0);
            double x = rng.range(-1.2, 1.2), y = rng.range(-1.2, 1.2);
            if (v == 4) { x = -0.5; y = 0.25; }      // shares an edge with triangle 0 (vertices 1, 2 below)
            if (v == 1) { x = -0.5; y = 0.25; }
            if (v == 6 || v == 7 || v == 8) { x = 0.1 * (v - 6); y = 0.1 * (v - 6); }  // degenerate
            append_f(st.vertex, static_cast<float>(x * w));
            append_f(st.vertex, static_cast<float>(y * w));
            append_f(st.vertex, static_cast<float>(rng.range(0.0, 1.0) * w));
            append_f(st.vertex, static_cast<float>(w));
            for (int c = 0; c < 4; c++) append_f(st.vertex, static_cast<float>(rng.uniform()));
        }
        p.num_bindings = 1;
        p.bindings[0] = {0, 32, VK_VERTEX_INPUT_RATE_VERTEX};
        p.num_attributes = 2;
        p.attributes[0] = {0, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 0};
        p.attributes[1] = {1, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 16};
        if (const uint32_t cb = colour_attribute_bytes(colour_format)) {
            while (st.vertex.size() % 16) st.vertex.push_back(0);
            colour_offset = st.vertex.size();
            const bool half = colour_format == 76 || colour_format == 83 || colour_format == 90 || colour_format == 97;
            for (uint32_t v = 0; v < vcount; v++) {
                for (uint32_t b = 0; b < cb; b += half ? 2 : 1) {
                    if (half) {
                        const uint32_t h = (static_cast<uint32_t>(rng.below(2)) << 15) | (static_cast<uint32_t>(rng.below(16)) << 10) |
                                           static_cast<uint32_t>(rng.below(1024));
                        append(st.vertex, static_cast<uint16_t>(h));
                    } else {
                        st.vertex.push_back(static_cast<uint8_t>(rng.below(256)));
                    }
                }
            }
            p.num_bindings = 2;
            p.bindings[1] = {1, cb, VK_VERTEX_INPUT_RATE_VERTEX};
            p.attributes[1] = {1, 1, colour_format, 0};
        }
    } else if (program == CPV_PROGRAM_FLATQUAD) {
        vcount = tris * 3;
        for (uint32_t v = 0; v < vcount; v++) {
            append_f(st.vertex, static_cast<float>(rng.range(-1.1, 1.1)));
            append_f(st.vertex, static_cast<float>(rng.range(-1.1, 1.1)));
            for (int c = 0; c < 3; c++) append_f(st.vertex, static_cast<float>(rng.uniform()));
            append_f(st.vertex, static_cast<float>(rng.range(0.1, 0.9)));
        }
        p.num_bindings = 1;
        p.bindings[0] = {0, 24, VK_VERTEX_INPUT_RATE_VERTEX};
        p.num_attributes = 2;
        p.attributes[0] = {0, 0, VK_FORMAT_R32G32_SFLOAT, 0};
        p.attributes[1] = {1, 0, VK_FORMAT_R32G32B32A32_SFLOAT, 8};
    } else if (textured) {
        const Mat4 proj = perspective(60.0 * M_PI / 180.0, static_cast<double>(width) / height, 0.1, 10.0);
        const Mat4 view = look_at({0, 1.2, -1.8}, {0, 0, 0.1}, {0, -1, 0});
        st.uniform.resize(80);
        store_mat(mul(clip_matrix(), mul(proj, view)), reinterpret_cast<float*>(st.uniform.data()));
        float* lp = reinterpret_cast<float*>(st.uniform.data() + 64);
        lp[0] = 0.4f; lp[1] = 0.8f; lp[2] = -0.45f; lp[3] = 0.0f;
        vcount = tris * 3;
        for (uint32_t v = 0; v < vcount; v++) {
            append_f(st.vertex, static_cast<float>(rng.range(-1, 1)));
            append_f(st.vertex, static_cast<float>(rng.range(0, 0.3)));
            append_f(st.vertex, static_cast<float>(rng.range(-1, 1)));
            append_f(st.vertex, static_cast<float>(rng.range(-2, 3)));
            append_f(st.vertex, static_cast<float>(rng.range(-2, 3)));
            const V3 nn = norm({rng.range(-1, 1), rng.range(0.2, 1), rng.range(-1, 1)});
            append_f(st.vertex, static_cast<float>(nn.x));
            append_f(st.vertex, static_cast<float>(nn.y));
            append_f(st.vertex, static_cast<float>(nn.z));
        }
        make_texture(st, 64, seed + 7);
        if (variant & 0x4000) {  // nearest filtering + mirrored / clamp-to-border addressing
            st.scene.sampler.mag_filter = VK_FILTER_NEAREST;
            st.scene.sampler.address_u = VK_SAMPLER_ADDRESS_MODE_MIRRORED_REPEAT;
            st.scene.sampler.address_v = VK_SAMPLER_ADDRESS_MODE_CLAMP_TO_BORDER;
        }
        if (variant & 0x8000) {  // positive LOD bias → mip blending
            st.scene.sampler.mip_lod_bias = 1.3f;
            st.scene.sampler.address_u = VK_SAMPLER_ADDRESS_MODE_CLAMP_TO_EDGE;
        }
        cpv_scene_pipeline t = texlit_pipeline();
        t.cull_mode = p.cull_mode;
        t.front_face = p.front_face;
        t.depth_test = p.depth_test;
        t.depth_write = p.depth_write;
        t.depth_compare = p.depth_compare;
        t.topology = p.topology;
        t.line_width = p.line_width;
        t.blend_enable = p.blend_enable;
        t.src_color = p.src_color; t.dst_color = p.dst_color; t.color_op = p.color_op;
        t.src_alpha = p.src_alpha; t.dst_alpha = p.dst_alpha; t.alpha_op = p.alpha_op;
        t.stencil_test = p.stencil_test;
        t.stencil_front = p.stencil_front;
        t.stencil_back = p.stencil_back;
        t.program = program;
        if (program == CPV_PROGRAM_FETCH) t.spec_k = colour_format;  // parameter 5: the specialisation constant (0: none)
        if (program == CPV_PROGRAM_STORAGE) s.texture_binding = CPV_TEXTURE_STORAGE;
        if (program == CPV_PROGRAM_SEPARATE) s.texture_binding = CPV_TEXTURE_SEPARATE;
        p = t;
    } else if (program == CPV_PROGRAM_MESHPC) {
        const double phase[3] = {1.0, 2.0, 3.0};
        std::vector<uint8_t> ib;
        uint32_t vc = 0, ic = 0;
        icosphere(3, 0.15, phase, false, st.vertex, ib, vc, ic);
        const uint64_t inst_off = (st.vertex.size() + 15) & ~15ull;
        st.vertex.resize(inst_off);
        for (int k = 0; k < 3; k++) {
            append_f(st.vertex, static_cast<float>(k) * 0.6f - 0.6f);
            append_f(st.vertex, 0.0f);
            append_f(st.vertex, static_cast<float>(k) * 0.3f);
            append_f(st.vertex, 0.0f);
        }
        st.index = ib;
        s.index_type = VK_INDEX_TYPE_UINT32;
        const Mat4 proj = perspective(50.0 * M_PI / 180.0, static_cast<double>(width) / height, 0.5, 20.0);
        const Mat4 vp = mul(clip_matrix(), mul(proj, look_at({0, 0, -4}, {0, 0, 0}, {0, -1, 0})));
        p.num_bindings = 2;
        p.bindings[0] = {0, 24, VK_VERTEX_INPUT_RATE_VERTEX};
        p.bindings[1] = {1, 16, VK_VERTEX_INPUT_RATE_INSTANCE};
        p.num_attributes = 3;
        p.attributes[0] = {0, 0, VK_FORMAT_R32G32B32_SFLOAT, 0};
        p.attributes[1] = {1, 0, VK_FORMAT_R32G32B32_SFLOAT, 12};
        p.attributes[2] = {2, 1, VK_FORMAT_R32G32B32A32_SFLOAT, 0};
        p.topology = VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST;
        st.pipelines.push_back(p);
        cpv_scene_draw d{};
        d.indexed = 1;
        d.count = ic;
        d.instance_count = 3;
        d.push_size = 80;
        float push[20];
        store_mat(mul(vp, translate_scale({0, 0, 0}, 0.7)), push);
        push[16] = 0.8f; push[17] = 0.5f; push[18] = 0.2f; push[19] = (variant & 0x20) ? 0.5f : 1.0f;
        std::memcpy(d.push, push, sizeof(push));
        d.vertex_offsets[1] = inst_off;
        st.draws.push_back(d);
        return;
    }
    // Indexed variant: indices are a seeded permutation (with repeats) of the vertices.
    cpv_scene_draw d{};
    d.pipeline = 0;
    d.instance_count = 1;
    d.vertex_offsets[1] = colour_offset;
    if (variant & 0x1000 || seed % 3 == 0) {
        d.indexed = 1;
        s.index_type = u16 ? VK_INDEX_TYPE_UINT16 : VK_INDEX_TYPE_UINT32;
        const uint32_t count = vcount + 3;
        for (uint32_t i = 0; i < count; i++) {
            const uint32_t idx = i < vcount ? i : rng.below(vcount);
            if (u16) append(st.index, static_cast<uint16_t>(idx));
            else append(st.index, idx);
        }
        d.count = count;
    } else {
        d.count = vcount;
    }
    st.pipelines.push_back(p);
    // Two draws (the second with a different first vertex) to exercise
    // draw-to-draw ordering.
    st.draws.push_back(d);
    if (!d.indexed && vcount > 6) {
        cpv_scene_draw d2 = d;
        d2.first = 3;
        d2.count = vcount - 3;
        st.draws.push_back(d2);
    }
}

}  // namespace

extern "C" {

cpv_scene* cpvh_scene_create(uint32_t config, uint64_t seed, const uint64_t* params, uint32_t np) {
    auto param = [&](uint32_t i, uint64_t dflt) { return (params && i < np && params[i]) ? params[i] : dflt; };
    auto st = std::make_unique<Store>();
    st->config = config;
    switch (config) {
    case CPVH_CUBE: build_cube(*st, static_cast<uint32_t>(param(0, 0))); break;
    case CPVH_HEIGHTFIELD: build_heightfield(*st, seed, static_cast<uint32_t>(param(0, 1024)), static_cast<uint32_t>(param(1, 1920)), static_cast<uint32_t>(param(2, 1080))); break;
    case CPVH_BLEND:
        build_blend(*st, seed, static_cast<uint32_t>(param(0, 200000)), static_cast<uint32_t>(param(1, 1920)), static_cast<uint32_t>(param(2, 1080)),
                    static_cast<uint32_t>(param(3, 0)));
        break;
    case CPVH_BATCH:
        build_batch(*st, seed, static_cast<uint32_t>(param(0, 4096)), static_cast<uint32_t>(param(1, 200000)), static_cast<uint32_t>(param(2, 2560)),
                    static_cast<uint32_t>(param(3, 1440)));
        break;
    case CPVH_PROGRAM:
        build_program(*st, seed, static_cast<uint32_t>(params && np > 0 ? params[0] : 0), static_cast<uint32_t>(params && np > 1 ? params[1] : 0),
                      static_cast<uint32_t>(param(2, 64)), static_cast<uint32_t>(param(3, 48)), static_cast<uint32_t>(param(4, 12)),
                      static_cast<uint32_t>(param(5, 0)), static_cast<uint32_t>(param(6, 0)), param(7, 0), param(8, 0));
        break;
    case CPVH_SERVE: build_serve(*st, seed, static_cast<uint32_t>(param(0, 512)), static_cast<uint32_t>(param(1, 20000)), static_cast<uint32_t>(params && np > 2 ? params[2] : 0)); break;
    default: return nullptr;
    }
    st->finish();
    return &st.release()->scene;
}

void cpvh_scene_destroy(cpv_scene* scene) { delete reinterpret_cast<Store*>(scene); }

void cpvh_scene_set_frame(cpv_scene* scene, uint32_t frame) {
    Store* st = reinterpret_cast<Store*>(scene);
    if (st->config == CPVH_CUBE) store_mat(cube_mvp(frame, scene->width, scene->height), reinterpret_cast<float*>(st->uniform.data()));
}

uint64_t cpvh_scene_triangles(const cpv_scene* s) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < s->num_draws; i++) {
        const auto& d = s->draws[i];
        const auto& p = s->pipelines[d.pipeline];
        uint64_t per;
        switch (p.topology) {
        case VK_PRIMITIVE_TOPOLOGY_POINT_LIST: per = d.count; break;
        case VK_PRIMITIVE_TOPOLOGY_LINE_LIST: per = d.count / 2; break;
        case VK_PRIMITIVE_TOPOLOGY_LINE_STRIP: per = d.count > 1 ? d.count - 1 : 0; break;
        case VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST: per = d.count / 3; break;
        default: per = d.count > 2 ? d.count - 2 : 0; break;
        }
        total += per * d.instance_count;
    }
    return total;
}

}  // extern "C"
