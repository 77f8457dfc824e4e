// Host-side per-view uniforms of the hair pass: the camera and DOM HairParams
// of one groom, computed each frame on the CPU before any pass runs.
//
// Reference: src/render/pass.rs:342-453 (camera position/forward,
// clip_from_world and its inverse, depth_is_reverse, the per-groom light fit
// and near/far), :676-709 (make_params), :711-719 (key_direction), :721-745
// (world_corners, world_extent), :747-776 (light_fit), :778-787
// (depth_is_reverse, clip_z).  glam's f32 arithmetic is followed operation by
// operation (sums left to right, no fused multiply-add: this file is built
// with -ffp-contract=off so x86-64 and AArch64 agree); 4x4 inverses are
// computed in f64 and rounded once.  Matrices are column-major, m[4 * col + row].
#include <cfloat>
#include <cmath>
#include <cstring>
#include <initializer_list>

#include "hairgb.h"

namespace {

struct V3 {
    float x, y, z;
};

V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 scale(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
float length(V3 a) { return std::sqrt(dot(a, a)); }

// glam Vec3::normalize_or: v * (1 / |v|) when that reciprocal is finite and > 0.
V3 normalize_or(V3 v, V3 fallback) {
    const float rcp = 1.0f / length(v);
    return (std::isfinite(rcp) && rcp > 0.0f) ? scale(v, rcp) : fallback;
}

struct M4 {
    float m[16];
    float at(int row, int col) const { return m[4 * col + row]; }
};

M4 identity() {
    M4 r{};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
    return r;
}

M4 load(const float* cols) {
    M4 r;
    std::memcpy(r.m, cols, sizeof(r.m));
    return r;
}

// Mat4 * Vec4: x_axis * v.x + y_axis * v.y + z_axis * v.z + w_axis * v.w.
void mul_vec(const M4& a, const float v[4], float out[4]) {
    for (int r = 0; r < 4; ++r)
        out[r] = ((a.at(r, 0) * v[0] + a.at(r, 1) * v[1]) + a.at(r, 2) * v[2]) + a.at(r, 3) * v[3];
}

M4 mul(const M4& a, const M4& b) {
    M4 c;
    for (int col = 0; col < 4; ++col) mul_vec(a, &b.m[4 * col], &c.m[4 * col]);
    return c;
}

V3 transform_point(const M4& a, V3 p) {
    const float v[4] = {p.x, p.y, p.z, 1.0f};
    float o[4];
    mul_vec(a, v, o);
    return {o[0], o[1], o[2]};
}

V3 transform_vector(const M4& a, V3 p) {
    return {(a.at(0, 0) * p.x + a.at(0, 1) * p.y) + a.at(0, 2) * p.z,
            (a.at(1, 0) * p.x + a.at(1, 1) * p.y) + a.at(1, 2) * p.z,
            (a.at(2, 0) * p.x + a.at(2, 1) * p.y) + a.at(2, 2) * p.z};
}

// Inverse by the adjugate in f64, rounded to f32 once.  A singular matrix
// gives non-finite entries, as glam's inverse does.
M4 inverse(const M4& a) {
    double s[16];
    for (int i = 0; i < 16; ++i) s[i] = a.m[i];
    auto e = [&](int r, int c) { return s[4 * c + r]; };
    double inv[16];
    // cofactors of the transpose, laid out so inv is the inverse in the same column-major order
    const double a00 = e(0, 0), a01 = e(0, 1), a02 = e(0, 2), a03 = e(0, 3);
    const double a10 = e(1, 0), a11 = e(1, 1), a12 = e(1, 2), a13 = e(1, 3);
    const double a20 = e(2, 0), a21 = e(2, 1), a22 = e(2, 2), a23 = e(2, 3);
    const double a30 = e(3, 0), a31 = e(3, 1), a32 = e(3, 2), a33 = e(3, 3);
    const double b00 = a00 * a11 - a01 * a10, b01 = a00 * a12 - a02 * a10, b02 = a00 * a13 - a03 * a10;
    const double b03 = a01 * a12 - a02 * a11, b04 = a01 * a13 - a03 * a11, b05 = a02 * a13 - a03 * a12;
    const double b06 = a20 * a31 - a21 * a30, b07 = a20 * a32 - a22 * a30, b08 = a20 * a33 - a23 * a30;
    const double b09 = a21 * a32 - a22 * a31, b10 = a21 * a33 - a23 * a31, b11 = a22 * a33 - a23 * a32;
    const double det = b00 * b11 - b01 * b10 + b02 * b09 + b03 * b08 - b04 * b07 + b05 * b06;
    const double id = 1.0 / det;
    // inverse(r, c)
    const double r00 = (a11 * b11 - a12 * b10 + a13 * b09) * id, r01 = (-a01 * b11 + a02 * b10 - a03 * b09) * id;
    const double r02 = (a31 * b05 - a32 * b04 + a33 * b03) * id, r03 = (-a21 * b05 + a22 * b04 - a23 * b03) * id;
    const double r10 = (-a10 * b11 + a12 * b08 - a13 * b07) * id, r11 = (a00 * b11 - a02 * b08 + a03 * b07) * id;
    const double r12 = (-a30 * b05 + a32 * b02 - a33 * b01) * id, r13 = (a20 * b05 - a22 * b02 + a23 * b01) * id;
    const double r20 = (a10 * b10 - a11 * b08 + a13 * b06) * id, r21 = (-a00 * b10 + a01 * b08 - a03 * b06) * id;
    const double r22 = (a30 * b04 - a31 * b02 + a33 * b00) * id, r23 = (-a20 * b04 + a21 * b02 - a23 * b00) * id;
    const double r30 = (-a10 * b09 + a11 * b07 - a12 * b06) * id, r31 = (a00 * b09 - a01 * b07 + a02 * b06) * id;
    const double r32 = (-a30 * b03 + a31 * b01 - a32 * b00) * id, r33 = (a20 * b03 - a21 * b01 + a22 * b00) * id;
    const double rows[4][4] = {{r00, r01, r02, r03}, {r10, r11, r12, r13}, {r20, r21, r22, r23}, {r30, r31, r32, r33}};
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[4 * c + r] = rows[r][c];
    M4 out;
    for (int i = 0; i < 16; ++i) out.m[i] = (float)inv[i];
    return out;
}

// world_from_view of a transform at `eye` whose -Z looks along `direction`
// (the basis Transform::looking_to builds: back, right = up x back, up' = back x right).
M4 looking_to(V3 eye, V3 direction, V3 up) {
    const V3 back = normalize_or(neg(direction), {0.0f, 0.0f, 1.0f});
    const V3 right = normalize_or(cross(up, back), {1.0f, 0.0f, 0.0f});
    const V3 up2 = cross(back, right);
    M4 r = identity();
    const V3 c[4] = {right, up2, back, eye};
    for (int k = 0; k < 4; ++k) {
        r.m[4 * k + 0] = c[k].x;
        r.m[4 * k + 1] = c[k].y;
        r.m[4 * k + 2] = c[k].z;
    }
    return r;
}

// glam Mat4::orthographic_rh (bevy::math::proj::orthographic).
M4 orthographic_rh(float left, float right, float bottom, float top, float near_, float far_) {
    const float rw = 1.0f / (right - left), rh = 1.0f / (top - bottom), r = 1.0f / (near_ - far_);
    M4 m = identity();
    m.m[0] = rw + rw;
    m.m[5] = rh + rh;
    m.m[10] = r;
    m.m[12] = -(left + right) * rw;
    m.m[13] = -(top + bottom) * rh;
    m.m[14] = r * near_;
    return m;
}

// clip_z / depth_is_reverse (src/render/pass.rs:778-787).
float clip_z(const M4& clip, V3 p) {
    const float v[4] = {p.x, p.y, p.z, 1.0f};
    float c[4];
    mul_vec(clip, v, c);
    return c[2] / std::fmax(c[3], 1e-5f);
}

bool depth_is_reverse(const M4& clip, V3 camera, V3 forward) {
    return clip_z(clip, add(camera, scale(forward, 0.5f))) > clip_z(clip, add(camera, scale(forward, 30.0f)));
}

// key_direction (src/render/pass.rs:711-719): the first shadow caster, else
// the first light, else (0.35, 0.82, 0.45); normalized or +Y.
V3 key_direction(const hg_directional* lights, uint32_t n) {
    const hg_directional* pick = nullptr;
    for (uint32_t i = 0; i < n && !pick; ++i)
        if (lights[i].casts_shadows) pick = &lights[i];
    if (!pick && n) pick = &lights[0];
    const V3 d = pick ? V3{pick->direction_to_light[0], pick->direction_to_light[1], pick->direction_to_light[2]}
                      : V3{0.35f, 0.82f, 0.45f};
    return normalize_or(d, {0.0f, 1.0f, 0.0f});
}

void world_corners(const hg_groom_desc& g, const M4& wfm, V3 out[8]) {
    int k = 0;
    for (float x : {g.bounds_min[0], g.bounds_max[0]})
        for (float y : {g.bounds_min[1], g.bounds_max[1]})
            for (float z : {g.bounds_min[2], g.bounds_max[2]}) out[k++] = transform_point(wfm, {x, y, z});
}

void world_extent(const hg_groom_desc& g, const M4& wfm, V3* center, float* radius) {
    V3 c[8];
    world_corners(g, wfm, c);
    V3 s{0.0f, 0.0f, 0.0f};
    for (const V3& p : c) s = add(s, p);
    *center = scale(s, 1.0f / 8.0f);  // division by 8 is exact as a product
    float r = 1.0f;
    for (const V3& p : c) r = std::fmax(r, length(sub(p, *center)));
    *radius = r;
}

struct LightFit {
    V3 eye, forward;
    M4 clip;
    float near_, far_;
};

LightFit light_fit(const hg_groom_desc& g, const M4& wfm, V3 direction_to_light) {
    V3 center;
    float radius;
    world_extent(g, wfm, &center, &radius);
    const V3 to_light = normalize_or(direction_to_light, {0.0f, 1.0f, 0.0f});
    LightFit f;
    f.forward = neg(to_light);
    f.eye = add(center, scale(to_light, radius));
    float near_ = FLT_MAX, far_ = -FLT_MAX;
    V3 c[8];
    world_corners(g, wfm, c);
    for (const V3& p : c) {
        const float d = dot(sub(p, f.eye), f.forward);
        near_ = std::fmin(near_, d);
        far_ = std::fmax(far_, d);
    }
    near_ = std::fmax(near_ - radius * 0.05f, 0.05f);
    far_ = std::fmax(far_ + radius * 0.05f, near_ + 1.0f);
    const V3 up = std::fabs(dot(f.forward, {0.0f, 1.0f, 0.0f})) > 0.95f ? V3{0.0f, 0.0f, 1.0f} : V3{0.0f, 1.0f, 0.0f};
    const M4 view = inverse(looking_to(f.eye, f.forward, up));
    f.clip = mul(orthographic_rh(-radius, radius, -radius, radius, near_, far_), view);
    f.near_ = near_;
    f.far_ = far_;
    return f;
}

struct ViewArgs {
    M4 clip_from_world, world_from_clip, light_clip_from_world;
    V3 camera_pos, camera_forward;
    float screen[4];
    V3 light_forward, light_eye;
    float dom_near, dom_far, dom_scale;
    uint32_t pass_mode[4];
    uint32_t dom_w, dom_h;
};

// make_params (src/render/pass.rs:676-709); DOM_SIGMA = 0.05 (:26).
void make_params(const ViewArgs& v, const hg_groom_desc& g, hg_hair_params* p) {
    std::memset(p, 0, sizeof(*p));
    std::memcpy(p->clip_from_world, v.clip_from_world.m, 64);
    std::memcpy(p->world_from_clip, v.world_from_clip.m, 64);
    std::memcpy(p->world_from_model, g.world_from_model, 64);
    std::memcpy(p->light_clip_from_world, v.light_clip_from_world.m, 64);
    const float cp[4] = {v.camera_pos.x, v.camera_pos.y, v.camera_pos.z, 1.0f};
    const float cf[4] = {v.camera_forward.x, v.camera_forward.y, v.camera_forward.z, 0.0f};
    std::memcpy(p->camera_pos, cp, 16);
    std::memcpy(p->camera_forward, cf, 16);
    std::memcpy(p->screen, v.screen, 16);
    p->appearance[0] = g.roughness;
    p->appearance[1] = g.tilt;
    p->appearance[2] = g.lambda;
    p->appearance[3] = g.center_diameter;
    p->filter_params[0] = 1.0f;
    p->filter_params[1] = 0.2f;
    p->filter_params[2] = std::fmax(v.dom_scale, 1e-3f);
    p->filter_params[3] = 0.05f;
    std::memcpy(p->albedo, g.albedo, 16);
    p->flags[0] = g.lod ? 1u : 0u;
    p->flags[1] = g.filter ? 1u : 0u;
    p->flags[2] = g.ambient_occlusion ? 1u : 0u;
    p->flags[3] = g.deep_opacity ? 1u : 0u;
    std::memcpy(p->pass_mode, v.pass_mode, 16);
    const float le[4] = {v.light_eye.x, v.light_eye.y, v.light_eye.z, 1.0f};
    const float lf[4] = {v.light_forward.x, v.light_forward.y, v.light_forward.z, 0.0f};
    std::memcpy(p->light_eye, le, 16);
    std::memcpy(p->light_forward, lf, 16);
    p->dom_info[0] = (float)v.dom_w;
    p->dom_info[1] = (float)v.dom_h;
    p->dom_info[2] = v.dom_near;
    p->dom_info[3] = v.dom_far;
}

}  // namespace

extern "C" hg_status hg_groom_params(const hg_view_desc* view, const hg_groom_desc* groom, const hg_directional* lights,
                                     uint32_t light_count, uint32_t dom_w, uint32_t dom_h, hg_hair_params* camera,
                                     hg_hair_params* dom) {
    if (!view || !groom || !camera || !dom || (light_count && !lights)) return HG_INVALID_ARG;
    if (view->width == 0 || view->height == 0) return HG_INVALID_ARG;
    const M4 wfv = load(view->world_from_view);
    const M4 wfm = load(groom->world_from_model);
    const V3 camera_pos = transform_point(wfv, {0.0f, 0.0f, 0.0f});
    const V3 forward = normalize_or(neg(transform_vector(wfv, {0.0f, 0.0f, 1.0f})), {0.0f, 0.0f, -1.0f});
    const M4 clip_from_world =
        view->has_clip_from_world ? load(view->clip_from_world) : mul(load(view->clip_from_view), inverse(wfv));
    const M4 world_from_clip = inverse(clip_from_world);
    const bool reverse = depth_is_reverse(clip_from_world, camera_pos, forward);
    const LightFit lf = light_fit(*groom, wfm, key_direction(lights, light_count));
    V3 center;
    float radius;
    world_extent(*groom, wfm, &center, &radius);
    const float dist = std::fmax(length(sub(camera_pos, center)), 0.5f);
    const float cam_near = 0.05f;
    const float cam_far = std::fmax(dist + radius * 4.0f, cam_near + 1.0f);
    const float dom_scale = (lf.far_ - lf.near_) / (float)HG_LAYER_COUNT;
    const uint32_t bundles = groom->bundle_count ? groom->bundle_count : 1u;

    ViewArgs v;
    v.light_clip_from_world = lf.clip;
    v.light_forward = lf.forward;
    v.light_eye = lf.eye;
    v.dom_near = lf.near_;
    v.dom_far = lf.far_;
    v.dom_scale = dom_scale;
    v.dom_w = dom_w;
    v.dom_h = dom_h;

    v.clip_from_world = clip_from_world;
    v.world_from_clip = world_from_clip;
    v.camera_pos = camera_pos;
    v.camera_forward = forward;
    v.screen[0] = (float)view->width;
    v.screen[1] = (float)view->height;
    v.screen[2] = cam_near;
    v.screen[3] = cam_far;
    const uint32_t pm_cam[4] = {0u, bundles, reverse ? 1u : 0u, 0u};
    std::memcpy(v.pass_mode, pm_cam, 16);
    make_params(v, *groom, camera);

    v.clip_from_world = lf.clip;
    v.world_from_clip = inverse(lf.clip);
    v.camera_pos = lf.eye;
    v.camera_forward = lf.forward;
    v.screen[0] = (float)dom_w;
    v.screen[1] = (float)dom_h;
    v.screen[2] = lf.near_;
    v.screen[3] = lf.far_;
    const uint32_t pm_dom[4] = {1u, bundles, reverse ? 1u : 0u, 1u};
    std::memcpy(v.pass_mode, pm_dom, 16);
    make_params(v, *groom, dom);
    return HG_OK;
}
